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
// Work: one CTA per SM, two independent groups of 256 threads; a group walks
// runs of up to 256 spectra of one element in units of 8 spectra (two
// 128-row MMA tiles), carrying the last Ntaps-1 converted input rows in
// registers, so every input sample is loaded (bulk copy of 2 KB rows into a
// two-slot shared-memory ring) and converted once.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "fengine.cuh"
#include "mdt_common.cuh"
#include "tc_ptx.cuh"

namespace mdt {
namespace ftc {

constexpr int N = 1024;
constexpr int GROUPS = 2;
constexpr int GTHREADS = 256;
constexpr int THREADS = GROUPS * GTHREADS;
constexpr int US = 8;                   // spectra per unit
constexpr int CPT = N / GTHREADS;       // channels per thread
constexpr int ROWB = 2 * N;             // one (spectrum, element) row of int8 I/Q
constexpr int RUN = 256;                // spectra per work item
constexpr uint32_t TILE = 16384;        // 128 rows x 128 bytes
// shared memory: DFT matrix, twiddles, int8 requantisation scales, then per
// group: scaled window,
// operand tiles (also the twiddled operand and the output staging), input ring
constexpr uint32_t OFF_B = 0, OFF_TW = 8192, OFF_QS = 16384, OFF_G = 20480;
constexpr uint32_t G_W = 0, G_A = 32768, G_RING = 65536, G_BYTES = 98304;
constexpr uint32_t SMEM = OFF_G + GROUPS * G_BYTES;
// TMEM: per group 256 columns -- two 64-column MMA tiles, then 64 columns
// holding the packed output of the first 8 spectra of each 16-spectrum pair
constexpr uint32_t TMEM_COLS = 512, TMEM_GROUP = 256, TMEM_STASH = 128;

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

template <int NT, int MODE>
__global__ void __launch_bounds__(THREADS, 1) fengine_tc_kernel(Launch L)
{
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t bars[GROUPS][3];  // ring slot 0, ring slot 1, MMA done
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag[GROUPS];

    const uint32_t sbase = tc::smem_u32(sm);
    const int tid = threadIdx.x;
    const int g = tid / GTHREADS, t = tid % GTHREADS, wg = t >> 5, l = t & 31;

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
        for (int gg = 0; gg < GROUPS; gg++)
            for (int b = 0; b < 3; b++) tc::mbar_init(tc::smem_u32(&bars[gg][b]), 1);
        abort_flag[0] = abort_flag[1] = 0;
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
    const uint32_t tmem = tmem_slot + (uint32_t)(g * TMEM_GROUP);
    const uint32_t lane_q = (uint32_t)((wg & 3) * 32) << 16;

    // ---------------------------------------------------------------- group
    const uint32_t gA = sbase + OFF_G + (uint32_t)g * G_BYTES + G_A;     // tiles / A' / staging
    const uint32_t gR = sbase + OFF_G + (uint32_t)g * G_BYTES + G_RING;  // input ring, 2 x 8 rows
    // scaled window, tap pairs: wsp[p][wpos(c)] = (W[2p][c], W[2p+1][c]) * scale
    float2 *wsp = reinterpret_cast<float2 *>(sm + OFF_G + (size_t)g * G_BYTES + G_W);
    const uint32_t wsp_s = sbase + OFF_G + (uint32_t)g * G_BYTES + G_W;
    const uint32_t bar_in0 = tc::smem_u32(&bars[g][0]), bar_in1 = tc::smem_u32(&bars[g][1]);
    const uint32_t bar_mma = tc::smem_u32(&bars[g][2]);
    uint32_t ph_in0 = 0, ph_in1 = 0, ph_mma = 0;
    bool pend0 = false, pend1 = false;  // loads in flight (for the drain on abort)
    const bool issuer = (t == 0);
    const int bar_id = 1 + g;

    int cn1[CPT], cn2[CPT];
#pragma unroll
    for (int j = 0; j < CPT; j++) chan_of(8 * j + wg, l, cn1[j], cn2[j]);

    const uint32_t id_mma = tc::idesc_f16(64, 0, 0);  // M 128, N 64, f16 operands
    const uint64_t bdesc = tc::sw128_kmajor_desc(sbase + OFF_B);
    uint64_t carry[CPT][NT - 1];
    bool ok = true;

    FJob a = L.one;   // the current job
    int cur = -1;     // its index (-1: none loaded)
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
    auto sync_group = [&]() { tc::named_barrier(bar_id, GTHREADS); };
    auto fail = [&]() {
        atomicExch(L.err, 1);
        abort_flag[g] = 1;
    };

    for (int w = blockIdx.x * GROUPS + g; w < L.nwork && ok; w += gridDim.x * GROUPS) {
        // the job of work item w (items are ascending, so the job index only grows)
        int j = cur < 0 ? 0 : cur;
        if (L.table)
            while (j + 1 < L.njobs && w >= L.table[j + 1].wk0) j++;
        if (j != cur) {
            if (L.table) a = L.table[j];
            cur = j;
            sync_group();  // the previous job's window is no longer read
            for (int i = t; i < N * 4; i += GTHREADS) {
                const int pr = i >> 10, c = i & (N - 1);
                const float w0 = 2 * pr < NT ? __ldg(a.win + 2 * pr * N + c) * a.scale : 0.0f;
                const float w1 = 2 * pr + 1 < NT ? __ldg(a.win + (2 * pr + 1) * N + c) * a.scale : 0.0f;
                wsp[pr * N + wpos(c)] = make_float2(w0, w1);
            }
            sync_group();
        }
        const int runs_per_e = (a.nsp + RUN - 1) / RUN;
        const int wl = w - a.wk0;
        const int e = wl / runs_per_e;
        const int s0 = (wl % runs_per_e) * RUN;
        const int s1 = min(s0 + RUN, a.nsp);
        const int nunits = (s1 - s0 + US - 1) / US;
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
        if (!tc::mbar_wait(bar_in1, ph_in1)) fail();
        ph_in1 ^= 1;
        pend1 = false;
#pragma unroll
        for (int j = 0; j < CPT; j++) {
            const uint32_t cb = (uint32_t)(2 * (32 * cn1[j] + cn2[j]));
#pragma unroll
            for (int i = 0; i < NT - 1; i++)
                carry[j][i] = iq_to_f2(lds_u16(gR + (uint32_t)(8 * ROWB + i * ROWB) + cb));
        }
        sync_group();
        if (abort_flag[g]) {
            ok = false;
            break;
        }
        if (issuer && nunits > 1) load_rows(1, s0 + US + NT - 1, unit_rows(1), e);
        pend1 = nunits > 1;

        for (int u = 0; u < nunits; u++) {
            const int slot = u & 1;
            const uint32_t ring = gR + (uint32_t)(slot * 8 * ROWB);
            if (!tc::mbar_wait(slot ? bar_in1 : bar_in0, slot ? ph_in1 : ph_in0)) fail();
            if (slot) {
                ph_in1 ^= 1;
                pend1 = false;
            } else {
                ph_in0 ^= 1;
                pend0 = false;
            }
            // ---- PFB: 8 spectra x 4 channels per thread -> A tiles (f16, scaled)
#pragma unroll
            for (int j = 0; j < CPT; j++) {
                const int n1 = cn1[j], n2 = cn2[j];
                const int c = 32 * n1 + n2;
                uint64_t w2[NT];
#pragma unroll
                for (int pr = 0; pr < NT / 2; pr++) {
                    const float2 wv = lds_f2(wsp_s + (uint32_t)((pr * N + wpos(c)) * 8));
                    w2[2 * pr] = pk2(wv.x, wv.x);
                    w2[2 * pr + 1] = pk2(wv.y, wv.y);
                }
                uint64_t xw[NT - 1 + US];
#pragma unroll
                for (int i = 0; i < NT - 1; i++) xw[i] = carry[j][i];
#pragma unroll
                for (int r = 0; r < US; r++)
                    xw[NT - 1 + r] = iq_to_f2(lds_u16(ring + (uint32_t)(r * ROWB + 2 * c)));
#pragma unroll
                for (int s = 0; s < US; s++) {
                    uint64_t acc = mul2(xw[s], w2[0]);
#pragma unroll
                    for (int i = 1; i < NT; i++) acc = fma2(xw[s + i], w2[i], acc);
                    const float2 p = up2(acc);
                    const int row = (s & 3) * 32 + n2;
                    sts_u32(gA + (uint32_t)(s >> 2) * TILE + tile_word(row, n1),
                            pack_h2<__half>(p.x, p.y));
                }
#pragma unroll
                for (int i = 0; i < NT - 1; i++) carry[j][i] = xw[US + i];
            }
            tc::fence_proxy_async();
            sync_group();
            if (abort_flag[g]) {
                ok = false;
                break;
            }
            if (issuer) {
                if (u + 2 < nunits) {
                    load_rows(slot, s0 + US * (u + 2) + NT - 1, unit_rows(u + 2), e);
                }
                tc::fence_after_sync();
#pragma unroll
                for (int tl = 0; tl < 2; tl++) {
                    const uint64_t ad = tc::sw128_kmajor_desc(gA + (uint32_t)tl * TILE);
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        tc::mma_f16(tmem + (uint32_t)(tl * 64), ad + 2 * k, bdesc + 2 * k, id_mma,
                                    k > 0);
                }
                tc::mma_commit(bar_mma);
            }
            if (u + 2 < nunits) {
                if (slot) pend1 = true;
                else pend0 = true;
            }
            // ---- twiddle: TMEM (row = (spectrum, n2), col = k1) -> A' (row = (spectrum, k1), K = n2)
            if (!tc::mbar_wait(bar_mma, ph_mma)) fail();
            ph_mma ^= 1;
            tc::fence_after_sync();
            {
                const int tl = wg >> 2, qd = wg & 3;
                const uint32_t tbase = tmem + lane_q + (uint32_t)(tl * 64);
                const uint32_t abase = gA + (uint32_t)tl * TILE;
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    uint32_t v[32];
                    tc::tmem_ld16(tbase + (uint32_t)(half * 32), *reinterpret_cast<uint32_t(*)[16]>(v));
                    tc::tmem_ld16(tbase + (uint32_t)(half * 32 + 16),
                                  *reinterpret_cast<uint32_t(*)[16]>(v + 16));
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int kk = 0; kk < 16; kk++) {
                        const int k1 = half * 16 + kk;
                        const float yr = __uint_as_float(v[2 * kk]), yi = __uint_as_float(v[2 * kk + 1]);
                        const float2 w = tw[k1 * 32 + l];
                        const float zr = fmaf(yr, w.x, -yi * w.y);
                        const float zi = fmaf(yr, w.y, yi * w.x);
                        sts_u32(abase + tile_word(qd * 32 + k1, l), pack_h2<__half>(zr, zi));
                    }
                }
            }
            tc::fence_proxy_async();
            tc::fence_before_sync();
            sync_group();
            if (issuer) {
                tc::fence_after_sync();
#pragma unroll
                for (int tl = 0; tl < 2; tl++) {
                    const uint64_t ad = tc::sw128_kmajor_desc(gA + (uint32_t)tl * TILE);
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        tc::mma_f16(tmem + (uint32_t)(tl * 64), ad + 2 * k, bdesc + 2 * k, id_mma,
                                    k > 0);
                }
                tc::mma_commit(bar_mma);
            }
            // ---- output: TMEM (row = (spectrum, k1), col = k2) -> staging [channel][spectrum]
            if (!tc::mbar_wait(bar_mma, ph_mma)) fail();
            ph_mma ^= 1;
            tc::fence_after_sync();
            {
                const int tl = wg >> 2, qd = wg & 3;
                const int su = tl * 4 + qd;  // spectrum within the unit
                const uint32_t tbase = tmem + lane_q + (uint32_t)(tl * 64);
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    uint32_t v[32];
                    tc::tmem_ld16(tbase + (uint32_t)(half * 32), *reinterpret_cast<uint32_t(*)[16]>(v));
                    tc::tmem_ld16(tbase + (uint32_t)(half * 32 + 16),
                                  *reinterpret_cast<uint32_t(*)[16]>(v + 16));
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int kk = 0; kk < 16; kk++) {
                        const int c = l + 32 * (half * 16 + kk);
                        const float qs = MODE == OUT_Q8 ? qs_s[c] : 1.0f;
                        sts_u32(gA + (uint32_t)(c * 32) + (uint32_t)((su ^ ((c >> 2) & 7)) << 2),
                                pack_out<MODE>(__uint_as_float(v[2 * kk]),
                                               __uint_as_float(v[2 * kk + 1]), qs));
                    }
                }
            }
            tc::fence_before_sync();
            sync_group();
            // ---- copy-out.  Units pair up into 16 spectra: the first unit's packed
            // 16-byte re and im chunks wait in TMEM, the second writes both units'
            // chunks as full 32-byte sectors (re chunks j, j+1 and im chunks 4+j,
            // 5+j of a row are sector neighbours under the row swizzle).
            {
                const int sabs = s0 + US * u;
                const int nvalid = min(US, a.nsp - sabs);
                const bool second = (u & 1) != 0;
                const bool lone = !second && u + 1 == nunits;  // first unit without a partner
                const uint32_t stash = tmem + lane_q + TMEM_STASH + (uint32_t)((wg >> 2) * 32);
                const int s_first = second ? sabs - US : sabs;
                const int kc = s_first >> 5, j0 = (s_first & 31) >> 3;  // j0 even
                const bool swap = (e & 1) != 0;  // the odd chunk comes first in the sector
                const uint32_t sre = (uint32_t)(((j0 ^ (e & 7)) & ~1) << 4);
                const uint32_t sim = (uint32_t)((((4 + j0) ^ (e & 7)) & ~1) << 4);
#pragma unroll
                for (int j = 0; j < CPT; j++) {
                    const int c = t + GTHREADS * j;
                    uint32_t wv[US];
#pragma unroll
                    for (int s = 0; s < US; s++) {
                        const uint32_t x = lds_u32(gA + (uint32_t)(c * 32) +
                                                   (uint32_t)((s ^ ((c >> 2) & 7)) << 2));
                        wv[s] = s < nvalid ? x : 0u;
                    }
                    uint32_t pk[8];  // re (4 words: 8 spectra) then im
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        pk[q] = __byte_perm(wv[2 * q], wv[2 * q + 1], 0x5410);
                        pk[4 + q] = __byte_perm(wv[2 * q], wv[2 * q + 1], 0x7632);
                    }
                    if (!second && !lone) {
                        tc::tmem_st8(stash + (uint32_t)(8 * j), pk);
                        continue;
                    }
                    uint32_t p0[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};  // first unit (zero if lone)
                    if (second) {
                        tc::tmem_ld8(stash + (uint32_t)(8 * j), p0);
                        tc::tmem_ld_wait();
                    }
                    const uint32_t *fw = second ? p0 : pk;  // first unit's words
                    const uint4 fr = make_uint4(fw[0], fw[1], fw[2], fw[3]);
                    const uint4 fi = make_uint4(fw[4], fw[5], fw[6], fw[7]);
                    const uint4 sr = second ? make_uint4(pk[0], pk[1], pk[2], pk[3])
                                            : make_uint4(0u, 0u, 0u, 0u);
                    const uint4 si = second ? make_uint4(pk[4], pk[5], pk[6], pk[7])
                                            : make_uint4(0u, 0u, 0u, 0u);
                    uint8_t *row = a.X16 + (((size_t)kc * N + c) * a.nep + e) * 128;
                    if (swap) {
                        stg32(row + sre, sr, fr);
                        stg32(row + sim, si, fi);
                    } else {
                        stg32(row + sre, fr, sr);
                        stg32(row + sim, fi, si);
                    }
                }
                if (!second && !lone) tc::tmem_st_wait();
            }
            sync_group();
        }
    }
    // drain copies still in flight (only after an abort), bounded
    if (!ok && t == 0) {
        if (pend0) tc::mbar_wait(bar_in0, ph_in0);
        if (pend1) tc::mbar_wait(bar_in1, ph_in1);
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
    const long blocks = std::max(1L, std::min<long>(nsm, ((long)L.nwork + ftc::GROUPS - 1) / ftc::GROUPS));
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
