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
// Both are real GEMMs over interleaved (re, im) pairs with the real 64 x 64
// form of the 32-point DFT matrix.  MMA 1: M = 128 rows (spectrum, n2), K =
// n1, N = 64 (k1); the DFT matrix is the B operand.  MMA 2 is transposed so
// that each output channel's spectra land along one TMEM lane: D = A Z^T
// with A = blockdiag(DFT, DFT) (M = 128 rows: (k2, re|im) for k1 < 16, then
// for k1 >= 16; K = 128) and Z as the B operand (N = 128 rows (k1 mod 16,
// spectrum), K = [n2 of k1 | n2 of k1 + 16]).  A thread reading TMEM lane
// (k2, re|im) then holds 8 consecutive spectra of one component of a channel
// per 8 columns: one 16-byte chunk of the X16 output, converted and stored
// straight from registers.
//
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
constexpr int THREADS = PT + ET + 64;   // + the loader (warp 24) and MMA (warp 25) warps
constexpr int NSLOT = 4;                // input ring slots
constexpr int US = 8;                   // spectra per unit
constexpr int CPT = N / PT;             // channels per PFB thread
constexpr int ROWB = 2 * N;             // one (spectrum, element) row of int8 I/Q
constexpr int RUN = 512;                // spectra per work item
constexpr uint32_t TILE = 16384;        // 128 rows x 128 bytes
// shared memory: the 128 x 128 block-diagonal DFT operand of MMA 2 as two
// 128-row tiles of K 64 (the first 64 rows of the first tile are MMA 1's
// B operand), twiddles, int8 requantisation scales, scaled window, two
// operand buffers of two tiles each (unit u's P tiles, read by MMA 1, then
// its Z tiles -- k1 < 16 and k1 >= 16 -- read by MMA 2), the input ring
// (NSLOT slots of 8 rows)
constexpr uint32_t OFF_B = 0, OFF_B2 = 16384, OFF_TW = 32768, OFF_QS = 40960, OFF_W = 45056;
constexpr uint32_t OFF_P = 77824;
constexpr uint32_t OFF_RING = OFF_P + 4 * TILE;
constexpr uint32_t SMEM = OFF_RING + NSLOT * US * ROWB;
// TMEM columns: two accumulator buffers of 128 columns (MMA 1 of unit u
// writes buffer u % 2 as two 64-column tiles, MMA 2 of the same unit
// overwrites all 128 columns once the twiddle stage has read them), the
// packed output chunks of the first unit of each pair of 8-spectrum units
// (16 columns per epilogue thread), the PFB carry: per PFB thread and
// channel the last Ntaps-1 converted input rows (16 columns), and the
// twiddles w_1024^{n2 k1} of the epilogue's twiddle stage (lane n2 of each
// lane quarter, 32 columns per half of the k1 range).
constexpr uint32_t TMEM_COLS = 512, T_D = 0, T_STASH = 256, T_CARRY = 320, T_TW = 448;
// mbarriers (per ring slot, or per operand / accumulator buffer, so that no
// waiter is ever more than one phase behind): ring slot filled (bulk copies
// landed) / emptied (PFB has read it); P written; MMA 1 done; Z written;
// MMA 2 done (accumulators readable); operand buffer free (MMA 2 has read Z);
// accumulator buffer free (the epilogue has read MMA 2's result)
enum {
    BAR_FULL = 0, BAR_EMPTY = NSLOT, BAR_PFULL = 2 * NSLOT, BAR_MMA1 = 2 * NSLOT + 2,
    BAR_ZFULL = 2 * NSLOT + 4, BAR_MMA2 = 2 * NSLOT + 6, BAR_PFREE = 2 * NSLOT + 8,
    BAR_DFREE = 2 * NSLOT + 10, NBARS = 2 * NSLOT + 12
};
__host__ __device__ constexpr uint32_t bar_count(int b)
{
    return (b >= BAR_EMPTY && b < BAR_EMPTY + NSLOT) || (b >= BAR_PFULL && b < BAR_PFULL + 2)
               ? PT
               : ((b >= BAR_DFREE && b < BAR_DFREE + 2) || (b >= BAR_ZFULL && b < BAR_ZFULL + 2)
                      ? ET
                      : 1);
}

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
// One 32-byte (full sector) global store of two 16-byte chunks.
__device__ __forceinline__ void stg32(void *p, const uint32_t *lo, const uint32_t *hi)
{
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(lo[0]),
                 "r"(lo[1]), "r"(lo[2]), "r"(lo[3]), "r"(hi[0]), "r"(hi[1]), "r"(hi[2]), "r"(hi[3])
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

// Two consecutive spectra (a, b) of one component -> one 32-bit word of the
// X16 row (a in the low half).
template <int MODE>
__device__ __forceinline__ uint32_t pack_out(float a, float b, float qs)
{
    if constexpr (MODE == OUT_Q8) {
        a = fminf(fmaxf(rintf(a * qs), -127.0f), 127.0f);
        b = fminf(fmaxf(rintf(b * qs), -127.0f), 127.0f);
        return pack_h2<__half>(a, b);
    } else if constexpr (MODE == OUT_BF16) {
        return pack_h2<__nv_bfloat16>(a, b);
    } else {
        return pack_h2<__half>(a, b);
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

// Warp-specialised pipeline, one CTA per SM, four roles that meet only at
// mbarriers (no named barrier between warps):
//  * loader (warp 24, one thread): the bulk copies of the input rows into an
//    NSLOT-slot ring, up to NSLOT uses ahead of the PFB;
//  * MMA issuer (warp 25, one thread): in a fixed order, MMA 2 of unit k
//    once its Z tiles are written, then MMA 1 of unit k + 1 once its P tiles
//    are written and its accumulator buffer is free, each as soon as its
//    mbarriers complete (the waiting thread is suspended, not polling);
//  * PFB (warps 0-7): per ring use, either a work item's Ntaps-1 lead-in rows
//    into the tap carry (TMEM) or one unit's tap sum into operand buffer
//    u % 2, once MMA 2 of unit u - 2 has read that buffer;
//  * epilogue (warps 8-23), pipelined over two units: the twiddle stage of
//    unit u from MMA 1's accumulators into Z (operand buffer u % 2, whose P
//    tiles MMA 1 has consumed), then the output of unit u - 1 (MMA 2's
//    result, converted and stored) while MMA 2 of unit u runs.
// Every wait is bounded and warp-uniform (the warp's lanes agree before
// acting); a failed wait raises the CTA's abort flag, which ends every other
// wait early, and the roles leave their loops without further tensor-memory
// traffic.
template <int NT, int MODE>
__global__ void __launch_bounds__(THREADS, 1) fengine_tc_kernel(Launch L)
{
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t bars[NBARS];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;

    const uint32_t sbase = tc::smem_u32(sm);
    const int tid = threadIdx.x;

    if (sbase & 1023) {  // the operand tiles need 1024-byte alignment
        if (tid == 0) atomicExch(L.err, 2);
        return;
    }

    // ---------------------------------------------------------------- setup
    for (int i = tid; i < 128 * 128; i += THREADS) {
        // block-diagonal real form of the 32-point DFT matrix: row r =
        // 64 h + 2 k + (re|im), column K = 64 h' + 2 n + (re|im), zero unless
        // h == h'; stored as two K-major 128-byte-swizzled tiles (K 0-63, 64-127)
        const int r = i >> 7, K = i & 127;
        const int kout = r & 63, kin = K & 63;
        float v = 0.0f;
        if ((r >> 6) == (K >> 6)) {
            const int k = kout >> 1, n = kin >> 1;
            float s, c;
            sincospif((float)((n * k) & 31) / 16.0f, &s, &c);
            v = (kout & 1) ? ((kin & 1) ? c : -s) : ((kin & 1) ? s : c);
        }
        *reinterpret_cast<__half *>(sm + OFF_B + (uint32_t)(K >> 6) * TILE + r * 128 +
                                    (((kin >> 3) ^ (r & 7)) << 4) + ((kin & 7) << 1)) =
            __float2half_rn(v);
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
    const uint32_t bar0 = tc::smem_u32(&bars[0]);
    auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
    if (tid == 0) {
        for (int b = 0; b < NBARS; b++) tc::mbar_init(bar(b), bar_count(b));
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
    auto fail = [&]() {
        atomicExch(L.err, 1);
        *abortp = 1;
    };
    // bounded wait whose outcome every lane of the warp shares
    auto wait_warp = [&](uint32_t b, uint32_t parity) {
        const bool okw = wait_or_abort(b, parity, abortp);
        return __all_sync(0xffffffffu, okw);
    };
    const uint32_t gR = sbase + OFF_RING;

    if (tid < PT) {
        // ============================================================ PFB role
        const int t = tid, wg = t >> 5, l = t & 31;
        // scaled window, tap pairs: wsp[p][wpos(c)] = (W[2p][c], W[2p+1][c]) * scale
        float2 *wsp = reinterpret_cast<float2 *>(sm + OFF_W);
        const uint32_t wsp_s = sbase + OFF_W;
        // carry of channel j: TMEM columns carry_t + 16 j (words 2i, 2i + 1 = row i)
        const uint32_t carry_t = tmem + ((uint32_t)((wg & 3) * 32) << 16) + T_CARRY + (uint32_t)((wg >> 2) * 64);
        bool ok = true;
        long n = 0, r = 0;  // units and ring uses of this CTA so far
        FJob a = L.one;
        int cur = -1;
        for (int w = blockIdx.x; w < L.nwork && ok; w += gridDim.x) {
            if (next_job(L, w, a, cur)) {
                // the job's scaled window for this thread's own channels (only this thread reads them)
#pragma unroll
                for (int j = 0; j < CPT; j++) {
                    int n1, n2;
                    chan_of(8 * j + wg, l, n1, n2);
                    const int c = 32 * n1 + n2;
#pragma unroll
                    for (int pr = 0; pr < NT / 2; pr++)
                        wsp[pr * N + wpos(c)] = make_float2(__ldg(a.win + 2 * pr * N + c) * a.scale,
                                                            __ldg(a.win + (2 * pr + 1) * N + c) * a.scale);
                }
            }
            const Item it = item_of(a, w);
            const int nunits = it.nunits;
            {  // ---- lead-in use: the item's first Ntaps-1 rows into the carry
                const int slot = (int)(r % NSLOT);
                if (!wait_warp(bar(BAR_FULL + slot), (uint32_t)((r / NSLOT) & 1))) {
                    fail();
                    ok = false;
                    break;
                }
                const uint32_t ring = gR + (uint32_t)(slot * US * ROWB);
#pragma unroll
                for (int j = 0; j < CPT; j++) {
                    int n1, n2;
                    chan_of(8 * j + wg, l, n1, n2);
                    const uint32_t cb = (uint32_t)(2 * (32 * n1 + n2));
                    uint32_t cv[16] = {};
#pragma unroll
                    for (int i = 0; i < NT - 1; i++) {
                        const float2 x = up2(iq_to_f2(lds_u16(ring + (uint32_t)(i * ROWB) + cb)));
                        cv[2 * i] = __float_as_uint(x.x);
                        cv[2 * i + 1] = __float_as_uint(x.y);
                    }
                    tc::tmem_st16(carry_t + (uint32_t)(16 * j), cv);
                }
                tc::mbar_arrive(bar(BAR_EMPTY + slot));
                r++;
            }
            for (int u = 0; u < nunits; u++, n++, r++) {
                const int slot = (int)(r % NSLOT), b = (int)(n & 1);
                const uint32_t ring = gR + (uint32_t)(slot * US * ROWB);
                if (!wait_warp(bar(BAR_FULL + slot), (uint32_t)((r / NSLOT) & 1)) ||
                    // operand buffer b is free once MMA 2 of unit n - 2 has read its Z
                    (n >= 2 && !wait_warp(bar(BAR_PFREE + b), (uint32_t)(((n >> 1) & 1) ^ 1)))) {
                    fail();
                    ok = false;
                    break;
                }
                tc::tmem_st_wait();  // the previous unit's (or lead-in's) carry stores
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
                    for (int q = 0; q < US; q++)
                        xw[NT - 1 + q] = iq_to_f2(lds_u16(ring + (uint32_t)(q * ROWB + 2 * c)));
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < NT - 1; i++)
                        xw[i] = pk2(__uint_as_float(cv[2 * i]), __uint_as_float(cv[2 * i + 1]));
#pragma unroll
                    for (int sp = 0; sp < US; sp++) {
                        uint64_t acc = mul2(xw[sp], w2[0]);
#pragma unroll
                        for (int i = 1; i < NT; i++) acc = fma2(xw[sp + i], w2[i], acc);
                        const float2 p = up2(acc);
                        const int row = (sp & 3) * 32 + n2;
                        sts_u32(gP + (uint32_t)(sp >> 2) * TILE + tile_word(row, n1),
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
                tc::mbar_arrive(bar(BAR_EMPTY + slot));  // the ring slot may be refilled
                tc::fence_proxy_async();                 // P is read by the tensor cores
                tc::mbar_arrive(bar(BAR_PFULL + b));
            }
        }
        tc::tmem_st_wait();  // no carry store in flight when the CTA frees TMEM
    } else if (tid < PT + ET) {
        // ======================================================= epilogue role
        // 16 warps.  Twiddle stage: warp 8 + ew reads TMEM lane quarter
        // qd = ew % 4 of MMA 1 tile tl = (ew / 4) % 2, columns [32 hc, 32 hc + 32)
        // with hc = ew / 8 (k1 in [16 hc, 16 hc + 16)).  Output stage: the same
        // lane quarter of MMA 2's result, columns [32 cb, 32 cb + 32) with
        // cb = ew / 4 (k1 mod 16 in [4 cb, 4 cb + 4), 8 spectra each).
        const int t = tid - PT, ew = t >> 5, l = t & 31;
        const uint32_t lane_q = (uint32_t)((ew & 3) * 32) << 16;
        const int qd = ew & 3, tl = (ew >> 2) & 1, hc = ew >> 3, cb = ew >> 2;
        const int su = tl * 4 + qd;  // spectrum of this thread's MMA 1 rows within the unit
        // MMA 2 row of this thread: (k2, re|im) for k1 in the lower (qd < 2) or upper half
        const int k2 = (32 * (qd & 1) + l) >> 1, comp = l & 1;
        const int k1base = 16 * (qd >> 1) + 4 * cb;
        // twiddles of this thread's twiddle stage (k1 in [16 hc, 16 hc + 16), n2 = l) in
        // TMEM columns T_TW + 32 hc of its lane quarter, written once by the tl = 0 warps
        const uint32_t ttw = tmem + lane_q + T_TW + (uint32_t)(32 * hc);
        if (tl == 0) {
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                uint32_t tv[16];
#pragma unroll
                for (int kk = 0; kk < 8; kk++) {
                    const float2 w = tw[(16 * hc + 8 * hh + kk) * 32 + l];
                    tv[2 * kk] = __float_as_uint(w.x);
                    tv[2 * kk + 1] = __float_as_uint(w.y);
                }
                tc::tmem_st16(ttw + (uint32_t)(16 * hh), tv);
            }
            tc::tmem_st_wait();
        }
        tc::fence_before_sync();
        tc::named_barrier(2, ET);
        tc::fence_after_sync();
        bool ok = true;
        long n = 0;
        FJob a = L.one;
        int cur = -1;
        // the unit whose output is pending (its MMA 2 was issued last)
        struct Pending {
            uint8_t *X16;
            int nep, nsp, e, sabs;
        } pend{};
        bool have_pend = false;
        // output of unit m (MMA 2 result, converted and stored); false if a wait failed
        auto output = [&](long m, const Pending &o) -> bool {
            const int b = (int)(m & 1);
            if (!wait_warp(bar(BAR_MMA2 + b), (uint32_t)((m >> 1) & 1))) return false;
            tc::fence_after_sync();
            uint32_t v[32];
            const uint32_t tout = tmem + lane_q + T_D + (uint32_t)(b * 128 + 32 * cb);
            tc::tmem_ld16(tout, *reinterpret_cast<uint32_t(*)[16]>(v));
            tc::tmem_ld16(tout + 16, *reinterpret_cast<uint32_t(*)[16]>(v + 16));
            tc::tmem_ld_wait();
            tc::fence_before_sync();
            tc::mbar_arrive(bar(BAR_DFREE + b));  // buffer b may take MMA 1 of unit m + 2
            const int nvalid = o.nsp - o.sabs;     // valid spectra of the unit (>= 8: all)
            const int j0 = (o.sabs & 31) >> 3;
            if (nvalid < US) {
#pragma unroll
                for (int j = 0; j < 32; j++)
                    if ((j & 7) >= nvalid) v[j] = 0u;
            }
            // this unit's four 16-byte chunks (one per channel k1base + i)
            uint32_t q[16];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float qs = MODE == OUT_Q8 ? qs_s[k1base + i + 32 * k2] : 1.0f;
                const float *x = reinterpret_cast<const float *>(v + 8 * i);
#pragma unroll
                for (int h = 0; h < 4; h++) q[4 * i + h] = pack_out<MODE>(x[2 * h], x[2 * h + 1], qs);
            }
            // Units pair up into 16 spectra: chunks j and j + 1 of a component are
            // neighbours in one 32-byte sector under the row swizzle, so the first
            // unit of a pair parks its chunks in TMEM and the second writes both.
            const bool second = (j0 & 1) != 0;
            const bool last = nvalid <= US;  // the element's last unit
            const uint32_t stash = tmem + lane_q + T_STASH + (uint32_t)(16 * cb);
            if (!second && !last) {
                tc::tmem_st16(stash, q);  // waited for before the second unit reads it
                return true;
            }
            uint32_t f[16];
            if (second) {
                tc::tmem_st_wait();
                tc::tmem_ld16(stash, f);
                tc::tmem_ld_wait();
            }
            const int jf = j0 & ~1;  // the pair's first chunk
            const int xe = o.e & 7;
            const uint32_t sec = (uint32_t)((((jf + 4 * comp) ^ xe) & ~1) << 4);
            const bool swap = (xe & 1) != 0;  // the pair's second chunk comes first in the sector
            const uint32_t zero4[4] = {0u, 0u, 0u, 0u};
            const size_t rstride = (size_t)o.nep * 128;
            uint8_t *row = o.X16 + ((size_t)((o.sabs >> 5) * N + k1base + 32 * k2) * o.nep + o.e) * 128;
#pragma unroll
            for (int i = 0; i < 4; i++, row += rstride) {
                const uint32_t *c0 = second ? f + 4 * i : q + 4 * i;  // chunk jf
                const uint32_t *c1 = second ? q + 4 * i : zero4;      // chunk jf + 1
                if (swap) stg32(row + sec, c1, c0);
                else stg32(row + sec, c0, c1);
                if (last && jf == 0)  // zero the rest of the element's last 32-spectrum chunk
                    stg32(row + (uint32_t)((((2 + 4 * comp) ^ xe) & ~1) << 4), zero4, zero4);
            }
            return true;
        };
        for (int w = blockIdx.x; w < L.nwork && ok; w += gridDim.x) {
            next_job(L, w, a, cur);
            const Item it = item_of(a, w);
            const int e = it.e, s0 = it.s0, nunits = it.nunits;
            for (int u = 0; u < nunits; u++, n++) {
                const int b = (int)(n & 1);
                // ---- twiddle: MMA 1 result (row = (spectrum, n2), col = k1) -> Z in
                //      operand buffer b, tile hc (row = 8 (k1 mod 16) + spectrum, K = n2)
                if (!wait_warp(bar(BAR_MMA1 + b), (uint32_t)((n >> 1) & 1))) {
                    fail();
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                {
                    const uint32_t tacc = tmem + lane_q + T_D + (uint32_t)(b * 128 + tl * 64 + 32 * hc);
                    const uint32_t zbase = sbase + OFF_P + (uint32_t)(b * 2 + hc) * TILE;
#pragma unroll
                    for (int hh = 0; hh < 2; hh++) {
                        uint32_t v[16], tv[16];
                        tc::tmem_ld16(tacc + (uint32_t)(16 * hh), v);
                        tc::tmem_ld16(ttw + (uint32_t)(16 * hh), tv);
                        tc::tmem_ld_wait();
#pragma unroll
                        for (int k = 0; k < 8; k++) {
                            const int kk = 8 * hh + k;
                            const float yr = __uint_as_float(v[2 * k]), yi = __uint_as_float(v[2 * k + 1]);
                            const float tr = __uint_as_float(tv[2 * k]), ti = __uint_as_float(tv[2 * k + 1]);
                            const float zr = fmaf(yr, tr, -yi * ti);
                            const float zi = fmaf(yr, ti, yi * tr);
                            sts_u32(zbase + tile_word(8 * kk + su, l), pack_h2<__half>(zr, zi));
                        }
                    }
                }
                tc::fence_proxy_async();  // Z is read by the tensor cores
                tc::fence_before_sync();  // MMA 2 overwrites the accumulators just read
                tc::mbar_arrive(bar(BAR_ZFULL + b));
                // ---- the previous unit's output while MMA 2 of this one runs
                if (have_pend && !output(n - 1, pend)) {
                    fail();
                    ok = false;
                    break;
                }
                pend = Pending{a.X16, a.nep, a.nsp, e, s0 + US * u};
                have_pend = true;
            }
        }
        if (ok && have_pend && !output(n - 1, pend)) fail();
        tc::tmem_st_wait();  // no stash store in flight when the CTA frees TMEM
    } else if (tid == PT + ET) {
        // ========================================================= loader role
        long total_uses = 0;  // this CTA's ring uses: one lead-in per work item, then its units
        {
            FJob a2 = L.one;
            int c2 = -1;
            for (int w = blockIdx.x; w < L.nwork; w += gridDim.x) {
                next_job(L, w, a2, c2);
                total_uses += 1 + item_of(a2, w).nunits;
            }
        }
        FJob al = L.one;
        int curl = -1, wl = blockIdx.x, ul = -1;  // ul = -1: the item's lead-in use
        Item itl{};
        const int nhist = L.table ? 0 : L.nhist;
        auto row_src = [&](long rho, int e) -> const char2 * {
            return rho < nhist ? L.hist + (rho * al.ne + e) * (long)N
                               : al.iq + ((rho - nhist) * al.ne + e) * (long)N;
        };
        long rl = 0;  // next ring use to load
        for (; rl < total_uses; rl++) {
            const int slot = (int)(rl % NSLOT);
            // the slot is free once the PFB has read use rl - NSLOT
            if (rl >= NSLOT &&
                !wait_or_abort(bar(BAR_EMPTY + slot), (uint32_t)(((rl / NSLOT) & 1) ^ 1), abortp)) {
                fail();
                break;
            }
            if (ul < 0) {
                next_job(L, wl, al, curl);
                itl = item_of(al, wl);
            }
            long r0;
            int cnt;
            if (ul < 0) {
                r0 = itl.s0;
                cnt = NT - 1;
            } else {
                r0 = itl.s0 + NT - 1 + US * ul;
                const int rem = al.nsp - itl.s0 - US * ul;
                cnt = rem < US ? rem : US;
            }
            const uint32_t full = bar(BAR_FULL + slot);
            const uint32_t dst = gR + (uint32_t)(slot * US * ROWB);
            tc::mbar_expect_tx(full, (uint32_t)(cnt * ROWB));
            for (int q = 0; q < cnt; q++)
                tc::bulk_g2s(dst + (uint32_t)(q * ROWB), row_src(r0 + q, itl.e), ROWB, full);
            if (++ul == itl.nunits) {
                ul = -1;
                wl += gridDim.x;
            }
        }
        // the copies issued are complete before the CTA ends (bounded waits)
        for (long q = rl > NSLOT ? rl - NSLOT : 0; q < rl; q++)
            tc::mbar_wait(bar(BAR_FULL + (int)(q % NSLOT)), (uint32_t)((q / NSLOT) & 1));
    } else if (tid == PT + ET + 32) {
        // ========================================================== MMA role
        const uint32_t id_mma = tc::idesc_f16(64, 0, 0);    // MMA 1: M 128, N 64, f16 operands
        const uint32_t id_mma2 = tc::idesc_f16(128, 0, 0);  // MMA 2: M 128, N 128
        const uint64_t bdesc = tc::sw128_kmajor_desc(sbase + OFF_B);  // DFT rows 0-63
        const uint64_t a2desc1 = tc::sw128_kmajor_desc(sbase + OFF_B2);
        long total_units = 0;
        {
            FJob a2 = L.one;
            int c2 = -1;
            for (int w = blockIdx.x; w < L.nwork; w += gridDim.x) {
                next_job(L, w, a2, c2);
                total_units += item_of(a2, w).nunits;
            }
        }
        // MMA 1 of unit u: accumulator buffer u % 2 <- P tiles x DFT
        auto issue_mma1 = [&](long u) {
            const int b = (int)(u & 1);
            const uint32_t gP = sbase + OFF_P + (uint32_t)b * 2 * TILE;
#pragma unroll
            for (int tt = 0; tt < 2; tt++) {
                const uint64_t ad = tc::sw128_kmajor_desc(gP + (uint32_t)tt * TILE);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    tc::mma_f16(tmem + T_D + (uint32_t)(b * 128 + tt * 64), ad + 2 * k,
                                bdesc + 2 * k, id_mma, k > 0);
            }
            tc::mma_commit(bar(BAR_MMA1 + b));
        };
        // MMA 2 of unit u: accumulator buffer u % 2 <- blockdiag(DFT, DFT) x Z^T
        auto issue_mma2 = [&](long u) {
            const int b = (int)(u & 1);
            const uint32_t dcol = tmem + T_D + (uint32_t)(b * 128);
            const uint32_t gz = sbase + OFF_P + (uint32_t)b * 2 * TILE;
            const uint64_t z0 = tc::sw128_kmajor_desc(gz), z1 = tc::sw128_kmajor_desc(gz + TILE);
#pragma unroll
            for (int k = 0; k < 4; k++) tc::mma_f16(dcol, bdesc + 2 * k, z0 + 2 * k, id_mma2, k > 0);
#pragma unroll
            for (int k = 0; k < 4; k++) tc::mma_f16(dcol, a2desc1 + 2 * k, z1 + 2 * k, id_mma2, 1);
            tc::mma_commit(bar(BAR_MMA2 + b));   // the accumulators are readable
            tc::mma_commit(bar(BAR_PFREE + b));  // the operand buffer may take P again
        };
        // Fixed order, each step issued as soon as its inputs are ready (blocking,
        // bounded waits): MMA 1 of unit 0, then per unit k, MMA 2 of k once its Z
        // tiles are written, and MMA 1 of k + 1 once its P tiles are written and
        // its accumulator buffer is free (the epilogue has read MMA 2 of k - 1).
        // In the epilogue's order these events come as Z(k), then the read of
        // MMA 2 of k - 1, so no step waits on a later one.
        long n1 = 0, n2 = 0;  // MMA 1 and MMA 2 units issued
        bool okm = true;
        if (total_units > 0) {
            okm = wait_or_abort(bar(BAR_PFULL), 0u, abortp);
            if (okm) {
                tc::fence_after_sync();
                issue_mma1(0);
                n1 = 1;
            }
        }
        for (long k = 0; okm && k < total_units; k++) {
            okm = wait_or_abort(bar(BAR_ZFULL + (int)(k & 1)), (uint32_t)((k >> 1) & 1), abortp);
            if (!okm) break;
            tc::fence_after_sync();
            issue_mma2(k);
            n2 = k + 1;
            const long u = k + 1;
            if (u < total_units) {
                const int b = (int)(u & 1);
                okm = wait_or_abort(bar(BAR_PFULL + b), (uint32_t)((u >> 1) & 1), abortp) &&
                      (u < 2 || wait_or_abort(bar(BAR_DFREE + b), (uint32_t)(((u >> 1) & 1) ^ 1), abortp));
                if (!okm) break;
                tc::fence_after_sync();
                issue_mma1(u);
                n1 = u + 1;
            }
        }
        if (!okm) fail();
        // the products issued are complete before the CTA frees its tensor memory
        if (n1 > 0) tc::mbar_wait(bar(BAR_MMA1 + (int)((n1 - 1) & 1)), (uint32_t)(((n1 - 1) >> 1) & 1));
        if (n2 > 0)
            tc::mbar_wait(bar(BAR_MMA2 + (int)((n2 - 1) & 1)), (uint32_t)(((n2 - 1) >> 1) & 1));
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
