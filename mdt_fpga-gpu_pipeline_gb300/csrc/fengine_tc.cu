// fengine_tc.cu -- tensor-core F-engine for Nch = 1024: int8 I/Q -> PFB tap
// sum (packed FP32 FMA) -> 1024-point DFT as two 32-point DFT matrix
// products on tcgen05 (f16 operands, FP32 accumulators in TMEM) with the
// FP32 twiddle multiply between them -> f16 / bf16 output in the X16 operand
// layout of the tensor-core X-engine.
//
// Same result contract as fengine_x16 (PpS_Batch -> cufftExecC2C ->
// ReorderFOutput, reference MDT_device_functions.cu:113-161,183-208 and
// MDT_OneStation_client.cu:1105, then the power-of-two scale and rounding
// to f16 / bf16), within the f16 arithmetic of the DFT.
//
// Decomposition (n = 32 n1 + n2, k = k1 + 32 k2, w_M = e^{-2 pi i / M}):
//   Y[k1][n2] = sum_n1 P[32 n1 + n2] w_32^{n1 k1}                  (MMA 1)
//   Z[k1][n2] = Y[k1][n2] w_1024^{n2 k1}                            (FP32)
//   X[k1 + 32 k2] = sum_n2 Z[k1][n2] w_32^{n2 k2}                   (MMA 2)
// Both products are real GEMMs M = 128, N = 64, K = 64 over interleaved
// (re, im) pairs: MMA 1 rows are (spectrum, n2), K is n1; MMA 2 rows are
// (spectrum, k1), K is n2; B is the same real 64 x 64 form of the 32-point
// DFT matrix for both.
//
// Work: one CTA per SM walks runs of up to 256 spectra of one element in
// units of 8 spectra (two 128-row MMA tiles).  Warps 0-7 carry the last
// Ntaps-1 converted input rows in tensor memory, so every input sample is
// loaded (bulk copy of 2 KB rows into a two-slot shared-memory ring) and
// converted once; warps 8-23 run the twiddle and output stages of the
// previous unit meanwhile (see fengine_tc_kernel).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "fengine.cuh"
#include "mdt_common.cuh"
#include "tc_ptx.cuh"

namespace mdt {
namespace ftc {

constexpr int N = 1024;
constexpr int PT = 256;                 // PFB threads (warps 0-7)
constexpr int ET = 512;                 // epilogue threads (warps 8-23)
constexpr int THREADS = PT + ET;
constexpr int US = 8;                   // spectra per unit
constexpr int CPT = N / PT;             // channels per PFB thread
constexpr int ROWB = 2 * N;             // one (spectrum, element) row of int8 I/Q
constexpr int RUN = 256;                // spectra per work item
constexpr uint32_t TILE = 16384;        // 128 rows x 128 bytes
// shared memory: DFT matrix, twiddles, int8 requantisation scales, scaled
// window, two P operand buffers (two tiles each), the Z operand, the output
// staging S, the input ring (two slots of 8 rows)
constexpr uint32_t OFF_B = 0, OFF_TW = 8192, OFF_QS = 16384, OFF_W = 20480;
constexpr uint32_t OFF_P = 53248, OFF_Z = OFF_P + 4 * TILE, OFF_S = OFF_Z + 2 * TILE;
constexpr uint32_t OFF_RING = OFF_S + 2 * TILE;
constexpr uint32_t SMEM = OFF_RING + 2 * US * ROWB;
// TMEM columns: two accumulator buffers of two 64-column tiles (MMA 1 of unit
// u writes buffer u % 2, MMA 2 of the same unit overwrites it once the
// twiddle stage has read it), 64 columns holding the packed output of the
// first 8 spectra of each 16-spectrum pair, and the PFB carry: per PFB thread
// and channel the last Ntaps-1 converted input rows (16 columns).
constexpr uint32_t TMEM_COLS = 512, T_D = 0, T_STASH = 256, T_CARRY = 320;
// mbarriers
enum { BAR_RING = 0, BAR_MMA1 = 2, BAR_FREE = 4, BAR_MMA2 = 6, NBARS = 7 };

// One launch: a single job (with optional PFB history) or a device table of
// jobs (FJob, work items from wk0).
struct Launch {
    FJob one;
    const char2 *hist;  // first nhist spectra of the single job (may be null)
    int nhist;
    const FJob *table;  // non-null: jobs from the table, no history
    const float *qscales;  // requantisation scales (int8 mode, single job)
    int njobs;
    int nwork;
    int *err;
};

__device__ __forceinline__ uint64_t pk2(float a, float b)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 up2(uint64_t v)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b)
{
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// int8 (re, im) in the low 16 bits -> exact float pair: each byte, offset by
// 128, becomes the low mantissa byte of 2^23; subtracting 2^23 + 128 leaves
// the value.
__device__ __forceinline__ uint64_t iq_to_f2(uint32_t v)
{
    const uint32_t u = v ^ 0x8080u;
    uint32_t re, im;
    asm("prmt.b32 %0, %1, %2, 0x7650;" : "=r"(re) : "r"(u), "r"(0x4B000000u));
    asm("prmt.b32 %0, %1, %2, 0x7651;" : "=r"(im) : "r"(u), "r"(0x4B000000u));
    uint64_t p, d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(p) : "r"(re), "r"(im));
    const uint64_t off = 0xCB000080CB000080ull;  // (-8388736.f, -8388736.f)
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(p), "l"(off));
    return d;
}

__device__ __forceinline__ float2 lds_f2(uint32_t a)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}
// One 32-byte (full sector) global store.
__device__ __forceinline__ void stg32(void *p, const uint4 &a, const uint4 &b)
{
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(a.x),
                 "r"(a.y), "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w)
                 : "memory");
}
// Position of channel c's window pair in the shared window table: channels
// c and c ^ 1 swap when bit 5 is set, which makes the loads of the channel
// map below conflict-free.
__device__ __forceinline__ int wpos(int c) { return c ^ ((c >> 5) & 1); }

__device__ __forceinline__ uint32_t lds_u16(uint32_t a)
{
    uint16_t v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ void sts_u32(uint32_t a, uint32_t v)
{
    asm volatile("st.shared.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lds_u32(uint32_t a)
{
    uint32_t v;
    asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}

// Output modes: f16, bf16, or per-channel int8 requantisation (rint, clamp to
// [-127, 127]) held exactly in f16 -- the operand of the exact int8 X-engine.
enum { OUT_F16 = 0, OUT_BF16 = 1, OUT_Q8 = 2 };

template <typename H>
__device__ __forceinline__ uint32_t pack_h2(float re, float im);
template <>
__device__ __forceinline__ uint32_t pack_h2<__half>(float re, float im)
{
    __half2 h = __floats2half2_rn(re, im);
    return *reinterpret_cast<uint32_t *>(&h);
}
template <>
__device__ __forceinline__ uint32_t pack_h2<__nv_bfloat16>(float re, float im)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(re, im);
    return *reinterpret_cast<uint32_t *>(&h);
}

template <int MODE>
__device__ __forceinline__ uint32_t pack_out(float re, float im, float qs)
{
    if constexpr (MODE == OUT_Q8) {
        re = fminf(fmaxf(rintf(re * qs), -127.0f), 127.0f);
        im = fminf(fmaxf(rintf(im * qs), -127.0f), 127.0f);
        return pack_h2<__half>(re, im);
    } else if constexpr (MODE == OUT_BF16) {
        return pack_h2<__nv_bfloat16>(re, im);
    } else {
        return pack_h2<__half>(re, im);
    }
}

// Channel of slot q (0..31: q = 8 * j + warp) for lane l.  The map is a
// bijection onto the 1024 channels chosen so that, for every q, the lanes'
// 2-byte input reads hit 32 different banks and their stores into the
// swizzled MMA tile (row n2, word n1) hit 32 different banks.
__device__ __forceinline__ void chan_of(int q, int l, int &n1, int &n2)
{
    const int b0 = q & 1, y = (q >> 1) & 7, z = q >> 4;
    n2 = 2 * (l >> 1) + b0;
    const int lo = (l & 3) ^ (z << 1);
    const int hi = (l >> 2) ^ (n2 & 7) ^ y;
    n1 = 4 * hi + lo;
}

// Byte offset of 32-bit word `w` (0..31) of row `r` in a 128-byte-swizzled tile.
__device__ __forceinline__ uint32_t tile_word(int r, int w)
{
    return (uint32_t)r * 128u + ((uint32_t)((w >> 2) ^ (r & 7)) << 4) + ((uint32_t)(w & 3) << 2);
}

// Bounded wait on an mbarrier phase that also gives up once the CTA's abort
// flag is raised (so one role's failure does not leave the other spinning).
__device__ __forceinline__ bool wait_or_abort(uint32_t bar, uint32_t parity, volatile int *abort)
{
    if (tc::mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    for (int k = 1; !tc::mbar_try_wait(bar, parity); k++) {
        if ((k & 31) == 0 && *abort) return false;
        if (clock64() - t0 > tc::kWaitCycles) return false;
    }
    return true;
}

// Work item w of the launch -> job (updates `a` / `cur`), element, first
// spectrum, number of 8-spectrum units.
struct Item {
    int e, s0, nunits;
};
__device__ __forceinline__ bool next_job(const Launch &L, int w, FJob &a, int &cur)
{
    int j = cur < 0 ? 0 : cur;
    if (L.table)
        while (j + 1 < L.njobs && w >= L.table[j + 1].wk0) j++;
    if (j == cur) return false;
    if (L.table) a = L.table[j];
    cur = j;
    return true;
}
__device__ __forceinline__ Item item_of(const FJob &a, int w)
{
    const int runs_per_e = (a.nsp + RUN - 1) / RUN;
    const int wl = w - a.wk0;
    Item it;
    it.e = wl / runs_per_e;
    it.s0 = (wl % runs_per_e) * RUN;
    it.nunits = (min(it.s0 + RUN, a.nsp) - it.s0 + US - 1) / US;
    return it;
}

// One staged unit waiting for its copy-out.
struct OutUnit {
    uint8_t *X16;
    int nep, e, kc, j0, nvalid;
    bool second, lone;
};

// Warp-specialised pipeline, one CTA per SM.  Warps 0-7 (PFB role) stream
// the input, run the tap sum into P buffer u % 2 (the tap carry lives in
// TMEM) and issue MMA 1 into TMEM accumulator buffer u % 2.  Warps 8-23
// (epilogue role) read that buffer, apply the twiddles into Z, issue MMA 2
// into the same buffer, store the previous unit (from the staging buffer S)
// while MMA 2 works, then pack this unit's result into S.  The roles meet
// only at mbarriers: MMA 1 done (P written, accumulators ready) and buffer
// free (the epilogue has read MMA 2's result), so the PFB of unit u + 1 runs
// while the epilogue of unit u works.
template <int NT, int MODE>
__global__ void __launch_bounds__(THREADS, 1) fengine_tc_kernel(Launch L)
{
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t bars[NBARS];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    __shared__ OutUnit prev_s;  // the epilogue's staged unit awaiting its copy-out

    const uint32_t sbase = tc::smem_u32(sm);
    const int tid = threadIdx.x;

    if (sbase & 1023) {  // the operand tiles need 1024-byte alignment
        if (tid == 0) atomicExch(L.err, 2);
        return;
    }

    // ---------------------------------------------------------------- setup
    for (int i = tid; i < 64 * 64; i += THREADS) {
        // 32-point DFT matrix, real form: row kout = 2 k + (re|im), column kin = 2 n + (re|im)
        const int kout = i >> 6, kin = i & 63;
        const int k = kout >> 1, n = kin >> 1;
        float s, c;
        sincospif((float)((n * k) & 31) / 16.0f, &s, &c);
        const float v = (kout & 1) ? ((kin & 1) ? c : -s) : ((kin & 1) ? s : c);
        const __half hv = __float2half_rn(v);
        *reinterpret_cast<__half *>(sm + OFF_B + kout * 128 +
                                    (((kin >> 3) ^ (kout & 7)) << 4) + ((kin & 7) << 1)) = hv;
    }
    float2 *tw = reinterpret_cast<float2 *>(sm + OFF_TW);
    for (int i = tid; i < 32 * 32; i += THREADS) {
        const int k1 = i >> 5, n2 = i & 31;
        float s, c;
        sincospif((float)(k1 * n2) / 512.0f, &s, &c);
        tw[i] = make_float2(c, -s);
    }
    float *qs_s = reinterpret_cast<float *>(sm + OFF_QS);
    if constexpr (MODE == OUT_Q8)
        for (int i = tid; i < N; i += THREADS) qs_s[i] = __ldg(L.qscales + i);
    if (tid == 0) {
        for (int b = 0; b < NBARS; b++)
            tc::mbar_init(tc::smem_u32(&bars[b]), (b == BAR_FREE || b == BAR_FREE + 1) ? ET : 1);
        abort_flag = 0;
        tc::fence_mbar_init();
    }
    if (tid < 32) {
        tc::tmem_alloc(tc::smem_u32(&tmem_slot), TMEM_COLS);
        tc::tmem_relinquish();
        tc::fence_before_sync();
    }
    tc::fence_proxy_async();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    volatile int *abortp = &abort_flag;
    // A failed wait raises the CTA's abort flag (which ends the other role's
    // waits early) and the thread's own flag; each role leaves its loop only
    // at a barrier that ORs the threads' flags, so all its threads leave
    // together and none is left at a named barrier.
    bool bad = false;
    auto fail = [&]() {
        atomicExch(L.err, 1);
        *abortp = 1;
        bad = true;
    };
    const uint32_t id_mma = tc::idesc_f16(64, 0, 0);  // M 128, N 64, f16 operands
    const uint64_t bdesc = tc::sw128_kmajor_desc(sbase + OFF_B);
    const uint32_t bar_mma1 = tc::smem_u32(&bars[BAR_MMA1]);    // + 8 * b
    const uint32_t bar_free = tc::smem_u32(&bars[BAR_FREE]);  // + 8 * b
    const uint32_t bar_mma2 = tc::smem_u32(&bars[BAR_MMA2]);
    const uint32_t gZ = sbase + OFF_Z;

    if (tid < PT) {
        // ============================================================ PFB role
        const int t = tid, wg = t >> 5, l = t & 31;
        const uint32_t gR = sbase + OFF_RING;
        // scaled window, tap pairs: wsp[p][wpos(c)] = (W[2p][c], W[2p+1][c]) * scale
        float2 *wsp = reinterpret_cast<float2 *>(sm + OFF_W);
        const uint32_t wsp_s = sbase + OFF_W;
        const uint32_t bar_in0 = tc::smem_u32(&bars[BAR_RING]), bar_in1 = bar_in0 + 8;
        uint32_t ph_in0 = 0, ph_in1 = 0;
        bool pend0 = false, pend1 = false;  // loads in flight (for the drain on abort)
        const bool issuer = (t == 0);
        long last_mma = -1;
        // carry of channel j: TMEM columns carry_t + 16 j (words 2i, 2i + 1 = row i)
        const uint32_t carry_t = tmem + ((uint32_t)((wg & 3) * 32) << 16) + T_CARRY + (uint32_t)((wg >> 2) * 64);
        bool ok = true;
        long n = 0;  // units of this CTA so far
        FJob a = L.one;
        int cur = -1;
        const int nhist = L.table ? 0 : L.nhist;
        auto row_src = [&](long rho, int e) -> const char2 * {
            return rho < nhist ? L.hist + (rho * a.ne + e) * (long)N
                               : a.iq + ((rho - nhist) * a.ne + e) * (long)N;
        };
        // issue the bulk copies of rows [r0, r0 + cnt) of element e into slot s
        auto load_rows = [&](int s, long r0, int cnt, int e) {
            const uint32_t bar = s ? bar_in1 : bar_in0;
            tc::mbar_expect_tx(bar, (uint32_t)(cnt * ROWB));
            for (int r = 0; r < cnt; r++)
                tc::bulk_g2s(gR + (uint32_t)(s * 8 * ROWB + r * ROWB), row_src(r0 + r, e), ROWB, bar);
        };
        auto sync_pfb = [&]() { tc::named_barrier(1, PT); };
        auto sync_pfb_bad = [&]() { return tc::named_barrier_or(1, PT, bad); };

        for (int w = blockIdx.x; w < L.nwork && ok; w += gridDim.x) {
            if (next_job(L, w, a, cur)) {
                sync_pfb();  // the previous job's window is no longer read
                for (int i = t; i < N * 4; i += PT) {
                    const int pr = i >> 10, c = i & (N - 1);
                    const float w0 = 2 * pr < NT ? __ldg(a.win + 2 * pr * N + c) * a.scale : 0.0f;
                    const float w1 =
                        2 * pr + 1 < NT ? __ldg(a.win + (2 * pr + 1) * N + c) * a.scale : 0.0f;
                    wsp[pr * N + wpos(c)] = make_float2(w0, w1);
                }
                sync_pfb();
            }
            const Item it = item_of(a, w);
            const int e = it.e, s0 = it.s0, nunits = it.nunits;
            auto unit_rows = [&](int u) {
                const int r = a.nsp - s0 - US * u;
                return r < 0 ? 0 : (r > US ? US : r);
            };
            // lead-in rows into slot 1, unit 0 into slot 0
            if (issuer) {
                load_rows(1, s0, NT - 1, e);
                load_rows(0, s0 + NT - 1, unit_rows(0), e);
            }
            pend0 = pend1 = true;
            if (!wait_or_abort(bar_in1, ph_in1, abortp)) fail();
            ph_in1 ^= 1;
            pend1 = false;
#pragma unroll
            for (int j = 0; j < CPT; j++) {
                int n1, n2;
                chan_of(8 * j + wg, l, n1, n2);
                const uint32_t cb = (uint32_t)(2 * (32 * n1 + n2));
                uint32_t cv[16] = {};
#pragma unroll
                for (int i = 0; i < NT - 1; i++) {
                    const float2 x = up2(iq_to_f2(lds_u16(gR + (uint32_t)(8 * ROWB + i * ROWB) + cb)));
                    cv[2 * i] = __float_as_uint(x.x);
                    cv[2 * i + 1] = __float_as_uint(x.y);
                }
                tc::tmem_st16(carry_t + (uint32_t)(16 * j), cv);
            }
            tc::tmem_st_wait();
            if (sync_pfb_bad()) {
                ok = false;
                break;
            }
            if (issuer && nunits > 1) load_rows(1, s0 + US + NT - 1, unit_rows(1), e);
            pend1 = nunits > 1;

            for (int u = 0; u < nunits; u++, n++) {
                const int slot = u & 1, b = (int)(n & 1);
                const uint32_t ring = gR + (uint32_t)(slot * 8 * ROWB);
                if (!wait_or_abort(slot ? bar_in1 : bar_in0, slot ? ph_in1 : ph_in0, abortp)) fail();
                if (slot) {
                    ph_in1 ^= 1;
                    pend1 = false;
                } else {
                    ph_in0 ^= 1;
                    pend0 = false;
                }
                // P buffer b is free once MMA 1 of unit n - 2 has completed
                if (n >= 2 && !wait_or_abort(bar_mma1 + 8 * b, (uint32_t)(((n >> 1) & 1) ^ 1), abortp))
                    fail();
                const uint32_t gP = sbase + OFF_P + (uint32_t)b * 2 * TILE;
                // ---- PFB: 8 spectra x 4 channels per thread -> P tiles (f16, scaled)
#pragma unroll
                for (int j = 0; j < CPT; j++) {
                    int n1, n2;
                    chan_of(8 * j + wg, l, n1, n2);
                    const int c = 32 * n1 + n2;
                    uint32_t cv[16];
                    tc::tmem_ld16(carry_t + (uint32_t)(16 * j), cv);
                    uint64_t w2[NT];
#pragma unroll
                    for (int pr = 0; pr < NT / 2; pr++) {
                        const float2 wv = lds_f2(wsp_s + (uint32_t)((pr * N + wpos(c)) * 8));
                        w2[2 * pr] = pk2(wv.x, wv.x);
                        w2[2 * pr + 1] = pk2(wv.y, wv.y);
                    }
                    uint64_t xw[NT - 1 + US];
#pragma unroll
                    for (int r = 0; r < US; r++)
                        xw[NT - 1 + r] = iq_to_f2(lds_u16(ring + (uint32_t)(r * ROWB + 2 * c)));
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < NT - 1; i++)
                        xw[i] = pk2(__uint_as_float(cv[2 * i]), __uint_as_float(cv[2 * i + 1]));
#pragma unroll
                    for (int s = 0; s < US; s++) {
                        uint64_t acc = mul2(xw[s], w2[0]);
#pragma unroll
                        for (int i = 1; i < NT; i++) acc = fma2(xw[s + i], w2[i], acc);
                        const float2 p = up2(acc);
                        const int row = (s & 3) * 32 + n2;
                        sts_u32(gP + (uint32_t)(s >> 2) * TILE + tile_word(row, n1),
                                pack_h2<__half>(p.x, p.y));
                    }
#pragma unroll
                    for (int i = 0; i < NT - 1; i++) {
                        const float2 x = up2(xw[US + i]);
                        cv[2 * i] = __float_as_uint(x.x);
                        cv[2 * i + 1] = __float_as_uint(x.y);
                    }
                    tc::tmem_st16(carry_t + (uint32_t)(16 * j), cv);
                }
                tc::tmem_st_wait();  // the next unit reads the carry back
                tc::fence_proxy_async();
                if (sync_pfb_bad()) {
                    ok = false;
                    break;
                }
                if (issuer) {
                    if (u + 2 < nunits) load_rows(slot, s0 + US * (u + 2) + NT - 1, unit_rows(u + 2), e);
                    // accumulator buffer b is free once the epilogue has read unit n - 2
                    if (n >= 2 && !wait_or_abort(bar_free + 8 * b, (uint32_t)(((n >> 1) & 1) ^ 1), abortp)) {
                        fail();
                    } else {
                        tc::fence_after_sync();
#pragma unroll
                        for (int tl = 0; tl < 2; tl++) {
                            const uint64_t ad = tc::sw128_kmajor_desc(gP + (uint32_t)tl * TILE);
#pragma unroll
                            for (int k = 0; k < 4; k++)
                                tc::mma_f16(tmem + T_D + (uint32_t)(b * 128 + tl * 64), ad + 2 * k,
                                            bdesc + 2 * k, id_mma, k > 0);
                        }
                        tc::mma_commit(bar_mma1 + 8 * b);
                        last_mma = n;
                    }
                }
                if (u + 2 < nunits) {
                    if (slot) pend1 = true;
                    else pend0 = true;
                }
            }
        }
        // drain what is still in flight, bounded (copies only after an abort)
        if (issuer) {
            if (!ok) {
                if (pend0) tc::mbar_wait(bar_in0, ph_in0);
                if (pend1) tc::mbar_wait(bar_in1, ph_in1);
            }
            if (last_mma >= 0)
                tc::mbar_wait(bar_mma1 + 8 * (uint32_t)(last_mma & 1), (uint32_t)((last_mma >> 1) & 1));
        }
    } else {
        // ======================================================= epilogue role
        // 16 warps: warp 8 + ew reads TMEM lane quarter qd = ew % 4 of tile
        // tl = (ew / 4) % 2, columns [32 hc, 32 hc + 32) with hc = ew / 8.
        const int t = tid - PT, ew = t >> 5, l = t & 31;
        const uint32_t lane_q = (uint32_t)((ew & 3) * 32) << 16;
        const int qd = ew & 3, tl = (ew >> 2) & 1, hc = ew >> 3;
        const int su = tl * 4 + qd;  // spectrum of this thread's accumulator rows within the unit
        const bool issuer = (t == 0);
        const uint32_t gS = sbase + OFF_S;
        const uint32_t stash = tmem + lane_q + T_STASH + (uint32_t)((ew >> 2) * 16);
        long last_mma = -1;
        bool ok = true;
        long n = 0;
        FJob a = L.one;
        int cur = -1;
        auto sync_epi = [&]() { tc::named_barrier(2, ET); };
        auto sync_epi_bad = [&]() { return tc::named_barrier_or(2, ET, bad); };

        // Copy-out of a staged unit.  Units pair up into 16 spectra: the first
        // unit's packed 16-byte re and im chunks wait in TMEM, the second writes
        // both units' chunks as full 32-byte sectors (re chunks j, j+1 and im
        // chunks 4+j, 5+j of a row are sector neighbours under the row swizzle).
        bool have_prev = false;
        auto copy_out = [&]() {
            const OutUnit &o = prev_s;
            const bool stash_only = !o.second && !o.lone;
            const bool swap = (o.e & 1) != 0;  // the odd chunk comes first in the sector
            // Lanes 2i and 2i+1 share a channel: lane 2i packs spectra 0-3 and
            // writes the re sector, lane 2i+1 packs spectra 4-7 and writes the im
            // sector, so each store instruction covers 16 rows (two sectors each)
            // instead of 32.
            const int hs = l & 1;
            const uint32_t soff = hs ? (uint32_t)((((4 + o.j0) ^ (o.e & 7)) & ~1) << 4)
                                     : (uint32_t)(((o.j0 ^ (o.e & 7)) & ~1) << 4);
            const int nv = o.nvalid - 4 * hs;  // valid spectra of this lane's half
#pragma unroll
            for (int kp = 0; kp < 2; kp++) {
                uint32_t p0[8];  // the first unit's chunks of rounds 2 kp, 2 kp + 1 (second unit only)
                if (o.second) tc::tmem_ld8(stash + (uint32_t)(8 * kp), p0);
                uint32_t q[8];  // this lane's 16-byte chunks of the unit, rounds 2 kp, 2 kp + 1
#pragma unroll
                for (int kr = 0; kr < 2; kr++) {
                    const int c = (t >> 1) + 256 * (2 * kp + kr);
                    uint32_t w[4];
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const int sp = 4 * hs + i;
                        w[i] = lds_u32(gS + (uint32_t)(c * 32) + (uint32_t)((sp ^ ((c >> 2) & 7)) << 2));
                    }
                    if (nv < 4) {
#pragma unroll
                        for (int i = 0; i < 4; i++)
                            if (i >= nv) w[i] = 0u;
                    }
                    const uint32_t re0 = __byte_perm(w[0], w[1], 0x5410), re1 = __byte_perm(w[2], w[3], 0x5410);
                    const uint32_t im0 = __byte_perm(w[0], w[1], 0x7632), im1 = __byte_perm(w[2], w[3], 0x7632);
                    // lane 2i keeps re and sends im, lane 2i+1 keeps im and sends re
                    const uint32_t x0 = __shfl_xor_sync(0xffffffffu, hs ? re0 : im0, 1);
                    const uint32_t x1 = __shfl_xor_sync(0xffffffffu, hs ? re1 : im1, 1);
                    q[4 * kr + 0] = hs ? x0 : re0;  // spectra 0-3, then 4-7, of this lane's component
                    q[4 * kr + 1] = hs ? x1 : re1;
                    q[4 * kr + 2] = hs ? im0 : x0;
                    q[4 * kr + 3] = hs ? im1 : x1;
                }
                if (stash_only) {
                    tc::tmem_st8(stash + (uint32_t)(8 * kp), q);
                    continue;
                }
                if (o.second) tc::tmem_ld_wait();
#pragma unroll
                for (int kr = 0; kr < 2; kr++) {
                    const int c = (t >> 1) + 256 * (2 * kp + kr);
                    const uint32_t *fw = o.second ? p0 + 4 * kr : q + 4 * kr;  // first unit's chunk
                    const uint4 f = make_uint4(fw[0], fw[1], fw[2], fw[3]);
                    const uint4 sc = o.second ? make_uint4(q[4 * kr], q[4 * kr + 1], q[4 * kr + 2], q[4 * kr + 3])
                                              : make_uint4(0u, 0u, 0u, 0u);
                    uint8_t *row = o.X16 + (((size_t)o.kc * N + c) * o.nep + o.e) * 128;
                    if (swap) stg32(row + soff, sc, f);
                    else stg32(row + soff, f, sc);
                }
            }
            if (stash_only) tc::tmem_st_wait();
        };

        for (int w = blockIdx.x; w < L.nwork && ok; w += gridDim.x) {
            next_job(L, w, a, cur);
            const Item it = item_of(a, w);
            const int e = it.e, s0 = it.s0, nunits = it.nunits;
            for (int u = 0; u < nunits; u++, n++) {
                const int b = (int)(n & 1);
                const uint32_t tacc = tmem + lane_q + T_D + (uint32_t)(b * 128 + tl * 64 + 32 * hc);
                // ---- twiddle: MMA 1 result (row = (spectrum, n2), col = k1) -> Z (row = (spectrum, k1), K = n2)
                if (!wait_or_abort(bar_mma1 + 8 * b, (uint32_t)((n >> 1) & 1), abortp)) fail();
                tc::fence_after_sync();
                {
                    uint32_t v[32];
                    tc::tmem_ld16(tacc, *reinterpret_cast<uint32_t(*)[16]>(v));
                    tc::tmem_ld16(tacc + 16, *reinterpret_cast<uint32_t(*)[16]>(v + 16));
                    tc::tmem_ld_wait();
                    const uint32_t abase = gZ + (uint32_t)tl * TILE;
#pragma unroll
                    for (int kk = 0; kk < 16; kk++) {
                        const int k1 = 16 * hc + kk;
                        const float yr = __uint_as_float(v[2 * kk]), yi = __uint_as_float(v[2 * kk + 1]);
                        const float2 tv = tw[k1 * 32 + l];
                        const float zr = fmaf(yr, tv.x, -yi * tv.y);
                        const float zi = fmaf(yr, tv.y, yi * tv.x);
                        sts_u32(abase + tile_word(qd * 32 + k1, l), pack_h2<__half>(zr, zi));
                    }
                }
                tc::fence_proxy_async();
                tc::fence_before_sync();
                if (sync_epi_bad()) {  // also orders the previous unit's staging before its copy-out
                    ok = false;
                    break;
                }
                if (issuer) {  // MMA 2 overwrites the accumulator buffer the twiddle stage has read
                    tc::fence_after_sync();
#pragma unroll
                    for (int tt = 0; tt < 2; tt++) {
                        const uint64_t ad = tc::sw128_kmajor_desc(gZ + (uint32_t)tt * TILE);
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            tc::mma_f16(tmem + T_D + (uint32_t)(b * 128 + tt * 64), ad + 2 * k, bdesc + 2 * k,
                                        id_mma, k > 0);
                    }
                    tc::mma_commit(bar_mma2);
                    last_mma = n;
                }
                // ---- the previous unit's copy-out runs while MMA 2 works
                if (have_prev) copy_out();
                // ---- output: MMA 2 result (row = (spectrum, k1), col = k2) -> staging S [channel][spectrum]
                if (!wait_or_abort(bar_mma2, (uint32_t)(n & 1), abortp)) fail();
                tc::fence_after_sync();
                uint32_t v[32];
                tc::tmem_ld16(tacc, *reinterpret_cast<uint32_t(*)[16]>(v));
                tc::tmem_ld16(tacc + 16, *reinterpret_cast<uint32_t(*)[16]>(v + 16));
                tc::tmem_ld_wait();
                tc::fence_before_sync();
                tc::mbar_arrive(bar_free + 8 * b);  // buffer b may take MMA 1 of unit n + 2
                sync_epi();  // S is no longer read by the previous copy-out
#pragma unroll
                for (int kk = 0; kk < 16; kk++) {
                    const int c = l + 32 * (16 * hc + kk);
                    const float qs = MODE == OUT_Q8 ? qs_s[c] : 1.0f;
                    sts_u32(gS + (uint32_t)(c * 32) + (uint32_t)((su ^ ((c >> 2) & 7)) << 2),
                            pack_out<MODE>(__uint_as_float(v[2 * kk]), __uint_as_float(v[2 * kk + 1]), qs));
                }
                if (issuer) {  // read by every epilogue thread after the next barrier
                    const int sabs = s0 + US * u;
                    const bool second = (u & 1) != 0;
                    const int s_first = second ? sabs - US : sabs;
                    prev_s.X16 = a.X16;
                    prev_s.nep = a.nep;
                    prev_s.e = e;
                    prev_s.kc = s_first >> 5;
                    prev_s.j0 = (s_first & 31) >> 3;  // even
                    prev_s.nvalid = min(US, a.nsp - sabs);
                    prev_s.second = second;
                    prev_s.lone = !second && u + 1 == nunits;  // first unit without a partner
                }
                have_prev = true;
            }
        }
        if (ok && have_prev) {
            sync_epi();  // the last unit's staging is complete
            copy_out();
        }
        if (issuer && last_mma >= 0) tc::mbar_wait(bar_mma2, (uint32_t)(last_mma & 1));
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem_slot, TMEM_COLS);
    }
}

}  // namespace ftc

static mdt_status launch_tc(int ntaps, int mode, const ftc::Launch &L, cudaStream_t stream)
{
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_status(e, "fengine_tc: device query");
    const long blocks = std::max(1L, std::min<long>(nsm, (long)L.nwork));
    auto launch = [&](auto kern) -> mdt_status {
        cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)ftc::SMEM);
        if (e2 != cudaSuccess) return cuda_status(e2, "fengine_tc: smem attribute");
        kern<<<(unsigned)blocks, ftc::THREADS, ftc::SMEM, stream>>>(L);
        return launch_status("fengine_tc_kernel");
    };
    using namespace ftc;
    if (ntaps == 8)
        return mode == OUT_Q8 ? launch(fengine_tc_kernel<8, OUT_Q8>)
             : mode == OUT_BF16 ? launch(fengine_tc_kernel<8, OUT_BF16>)
                                : launch(fengine_tc_kernel<8, OUT_F16>);
    return mode == OUT_Q8 ? launch(fengine_tc_kernel<4, OUT_Q8>)
         : mode == OUT_BF16 ? launch(fengine_tc_kernel<4, OUT_BF16>)
                            : launch(fengine_tc_kernel<4, OUT_F16>);
}

// Tensor-core F-engine, Nch = 1024, Ntaps 4 or 8.  `err` (device int) is set
// to 1 if a wait timed out.  Same arguments and output as fengine_x16, or,
// with `qscales`, as fengine_q8 (int8 requantisation, `scale` and `ab_fmt`
// unused).
mdt_status fengine_tc(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                      const int8_t *iq, const float *win, void *X16, int nep, int nkc, int ab_fmt,
                      float scale, int *err, cudaStream_t stream, const float *qscales)
{
    if (!fengine_tc_shape(nch, ntaps))
        return invalid("fengine_tc: needs Nch = 1024 and Ntaps 4 or 8");
    if (ne < 1 || nsp < 1 || !iq || !win || !X16 || !err || (nhist > 0 && !hist))
        return invalid("fengine_tc: bad arguments");
    if (((uintptr_t)iq | (uintptr_t)hist | (uintptr_t)X16) & 15)
        return invalid("fengine_tc: buffers must be 16-byte aligned");
    const long nwork = fjob_tc_items(ne, nsp);
    if (nwork > 0x7fffffffL) return invalid("fengine_tc: too many work items");
    ftc::Launch L{};
    L.one.iq = reinterpret_cast<const char2 *>(iq);
    L.one.win = win;
    L.one.X16 = (uint8_t *)X16;
    L.one.ne = ne;
    L.one.nsp = nsp;
    L.one.nep = nep;
    L.one.nkc = nkc;
    L.one.scale = qscales ? 1.0f : scale;
    L.one.blk0 = 0;
    L.one.wk0 = 0;
    L.hist = reinterpret_cast<const char2 *>(hist);
    L.nhist = nhist;
    L.table = nullptr;
    L.njobs = 1;
    L.nwork = (int)nwork;
    L.err = err;
    L.qscales = qscales;
    return launch_tc(ntaps, qscales ? ftc::OUT_Q8 : (ab_fmt ? ftc::OUT_BF16 : ftc::OUT_F16), L,
                     stream);
}

mdt_status fengine_tc_batched(int ntaps, const FJob *jobs, int njobs, long nwork, int *err,
                              cudaStream_t stream)
{
    if (!jobs || njobs < 1 || !err || (ntaps != 4 && ntaps != 8) || nwork < 1 ||
        nwork > 0x7fffffffL)
        return invalid("fengine_tc_batched: bad arguments");
    ftc::Launch L{};
    L.table = jobs;
    L.njobs = njobs;
    L.nwork = (int)nwork;
    L.err = err;
    return launch_tc(ntaps, ftc::OUT_F16, L, stream);
}

}  // namespace mdt

extern "C" MDT_API mdt_status mdt_fengine_tc(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                             const float *window, void *X16, int ab_fmt,
                                             float scale, int *err, cudaStream_t stream)
{
    if (ab_fmt != 0 && ab_fmt != 1) return mdt::invalid("fengine_tc: ab_fmt must be 0 or 1");
    if (!(scale > 0.0f)) return mdt::invalid("fengine_tc: scale must be positive");
    const int nep = (ne + 15) / 16 * 16, nkc = (nsp + 31) / 32;
    return mdt::fengine_tc(ne, nch, ntaps, nsp, nullptr, 0, iq, window, X16, nep, nkc, ab_fmt,
                           scale, err, stream, nullptr);
}

extern "C" MDT_API mdt_status mdt_fengine_tc_q8(int ne, int nch, int ntaps, int nsp,
                                                const int8_t *iq, const float *window, void *X16,
                                                const float *qscales, int *err,
                                                cudaStream_t stream)
{
    if (!qscales) return mdt::invalid("fengine_tc_q8: null scales");
    const int nep = (ne + 15) / 16 * 16, nkc = (nsp + 31) / 32;
    return mdt::fengine_tc(ne, nch, ntaps, nsp, nullptr, 0, iq, window, X16, nep, nkc, 0, 1.0f,
                           err, stream, qscales);
}
