// fengine.cu -- fused F-engine: int8 I/Q -> PFB tap sum -> FFT -> channel-major
// corner turn, in one kernel (the reference runs PpS_Batch, cufftExecC2C and
// ReorderFOutput as three passes over HBM, MDT_OneStation_client.cu:1083,
// 1105,1114).
//
// A block transforms ROWS rows (spectrum s, elements e0..e0+ROWS-1):
//  * the tap sum P[c] = sum_i W[i*Nch + c] * iq[s+i][e][c] is formed with
//    16-byte vector loads into shared memory, accumulated with fmaf from zero
//    in increasing i, the order of PpS_Batch (MDT_device_functions.cu:143-152),
//    so P is bit-identical to the drop-in kernel's output on the same samples;
//  * the FFT passes run in shared memory (fft_core.cuh), the last one leaves
//    the spectrum in natural order in shared memory;
//  * the block writes X[(c*Nsp + s)*NE + e] (ReorderFOutput's layout,
//    MDT_device_functions.cu:207): for each channel the ROWS elements are
//    contiguous.
// Input spectra may come from two buffers: the first `nhist` spectra from
// `hist` (the PFB history carried between integrations, reference
// MDT_OneStation_client.cu:1170) and the rest from `iq`.
#include <cuda_bf16.h>
#include <algorithm>
#include <cuda_fp16.h>

#include "fengine.cuh"
#include "fft_core.cuh"

namespace mdt {

// Rows (elements) per block of the FP32 F-engine and threads per row.
// Small blocks let several blocks share an SM, so one block's sample loads
// overlap another's FFT passes and barriers.
#ifndef MDT_FENG_ROWS
#define MDT_FENG_ROWS 4
#endif
#ifndef MDT_FENG_TPR
#define MDT_FENG_TPR 256
#endif
// Threads per SM the register budget is sized for (64K registers / this).
#ifndef MDT_FENG_SM_THREADS
#define MDT_FENG_SM_THREADS 1024
#endif

// Threads per row: N/8 capped at `cap`, but never fewer than N/16 (at most
// one radix-16 or two radix-8 butterflies per thread and pass).
constexpr int feng_tpr(int n, int cap)
{
    return (n / 8 < 1) ? 1 : (n / 8 <= cap ? n / 8 : (cap >= n / 16 ? cap : n / 16));
}

template <int N>
struct FengCfg {
    static constexpr int TPR = feng_tpr(N, MDT_FENG_TPR);
    static constexpr int RMAX = (1024 / TPR) < 1 ? 1 : 1024 / TPR;
    static constexpr int ROWS = MDT_FENG_ROWS < RMAX ? MDT_FENG_ROWS : RMAX;
    static constexpr int THREADS = ROWS * TPR;
    // resident blocks per SM requested from the register allocator
    static constexpr int MINB = (MDT_FENG_SM_THREADS / THREADS) < 1 ? 1 : (MDT_FENG_SM_THREADS / THREADS);
    static constexpr int RSTRIDE = fft::Shape<N>::PADN + 4;  // float2 per row (bank skew)
    static constexpr size_t SMEM = sizeof(float2) * (size_t)RSTRIDE * ROWS;
};

struct FengArgs {
    const char2 *hist;  // first nhist spectra (may be null when nhist == 0)
    const char2 *iq;    // remaining spectra
    int nhist;
    int ne, ntaps, nsp, ngroups;
    const float *win;
    const float2 *tw;
    float2 *X;
};

// Polyphase tap sum of the block's rows into shared memory (natural channel
// order, padded): each work item is 8 consecutive channels of one row, read
// as one 16-byte int8 I/Q vector and two float4 window vectors per tap;
// accumulation is fmaf from zero in increasing tap order.  Row r of the block
// is (spectrum s0, element e0 + r), or with SPECTRA_ROWS (spectrum s0 + r,
// element e0); rows past NE or Nsp are zero.
template <int N, int ROWS, int THREADS, bool SPECTRA_ROWS = false>
__device__ __forceinline__ void pfb_rows_to_smem(const FengArgs &a, int s0, int e0, float2 *smem,
                                                 int rstride)
{
    constexpr int ITEMS = ROWS * (N / 8);
    const long rowlen = (long)a.ne * N;
    for (int it = threadIdx.x; it < ITEMS; it += THREADS) {
        const int r = it / (N / 8);
        const int c0 = (it - r * (N / 8)) * 8;
        const int e = SPECTRA_ROWS ? e0 : e0 + r;
        const int s = SPECTRA_ROWS ? s0 + r : s0;
        float re[8], im[8];
#pragma unroll
        for (int k = 0; k < 8; k++) re[k] = im[k] = 0.0f;
        if (e < a.ne && s < a.nsp) {
            for (int i = 0; i < a.ntaps; i++) {
                const int sp = s + i;
                const char2 *src = (sp < a.nhist) ? a.hist + (long)sp * rowlen
                                                  : a.iq + (long)(sp - a.nhist) * rowlen;
                const int4 raw = __ldg(reinterpret_cast<const int4 *>(src + (long)e * N + c0));
                const float4 w0 = __ldg(reinterpret_cast<const float4 *>(a.win + (long)i * N + c0));
                const float4 w1 =
                    __ldg(reinterpret_cast<const float4 *>(a.win + (long)i * N + c0 + 4));
                const float w[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
                const int words[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int word = words[k >> 1];
                    const int sh = (k & 1) * 16;
                    const float xr = (float)(signed char)((word >> sh) & 0xff);
                    const float xi = (float)(signed char)((word >> (sh + 8)) & 0xff);
                    re[k] = __fmaf_rn(w[k], xr, re[k]);
                    im[k] = __fmaf_rn(w[k], xi, im[k]);
                }
            }
        }
        float2 *sx = smem + (size_t)r * rstride;
        const int p0 = fft::pad(c0);  // c0 % 8 == 0: pad(c0 + k) = p0 + k for k < 8
#pragma unroll
        for (int k = 0; k < 8; k++) sx[p0 + k] = make_float2(re[k], im[k]);
    }
}

template <int N>
__global__ void __launch_bounds__(FengCfg<N>::THREADS, FengCfg<N>::MINB) fengine_f32_kernel(FengArgs a)
{
    using C = FengCfg<N>;
    extern __shared__ float2 fsm[];
    const long blk = blockIdx.x;
    const int s = (int)(blk / a.ngroups);
    const int e0 = (int)(blk - (long)s * a.ngroups) * C::ROWS;
    const int lrow = threadIdx.x / C::TPR;
    const int t = threadIdx.x - lrow * C::TPR;

    pfb_rows_to_smem<N, C::ROWS, C::THREADS>(a, s, e0, fsm, C::RSTRIDE);
    __syncthreads();
    auto none_load = [](int) { return make_float2(0.f, 0.f); };
    auto none_store = [](int, float2) {};
    fft::transform_row<N, C::TPR, false, false>(fsm + (size_t)lrow * C::RSTRIDE, t, a.tw,
                                                none_load, none_store);

    // corner turn: ROWS contiguous elements per channel
    const int nrow = min(C::ROWS, a.ne - e0);
    float2 *dst = a.X + (long)s * a.ne + e0;
    const long cstride = (long)a.nsp * a.ne;
    for (int k = threadIdx.x; k < N * C::ROWS; k += C::THREADS) {
        const int c = k / C::ROWS, r = k - c * C::ROWS;
        if (r < nrow) dst[(long)c * cstride + r] = fsm[(size_t)r * C::RSTRIDE + fft::pad(c)];
    }
}

// ------------------------------------------------------------------------
// Spectrum-block F-engines (the plan's FP32 path and the tensor-core path).
// A block owns one element and 8 consecutive spectra s0..s0+7, the rows of
// its transform.  The tap sum keeps the window of the thread's channels in
// registers and converts each input spectrum from int8 once: input spectrum
// s0+j feeds row r at tap j-r, and the unrolled loop over j visits every
// row's taps in increasing order, so each output is the same fmaf chain as
// PpS_Batch (bit-identical).  NT is Ntaps as a compile-time constant (4 or
// 8); other tap counts use the per-row tap sum above.  Consecutive blocks
// are the four 8-spectrum groups of one (element, 32-spectrum chunk), so
// their inputs overlap in L2 and their partial output rows meet there.

// Threads per row and register budget of the spectrum-block kernels.
#ifndef MDT_FENG16_TPR
#define MDT_FENG16_TPR 64
#endif
#ifndef MDT_FENG16_SM_THREADS
#define MDT_FENG16_SM_THREADS 1024
#endif

constexpr int SB8 = 8;  // spectra per block

// Tap sums of the spectrum-block kernels convert int8 samples with integer
// and FP32 add instructions instead of the int-to-float conversion unit.
#ifndef MDT_FENG_I2F_MAGIC
#define MDT_FENG_I2F_MAGIC 1
#endif

template <int N>
struct FengBCfg {
    static constexpr int TPR = feng_tpr(N, MDT_FENG16_TPR);
    static constexpr int THREADS = SB8 * TPR;
    static constexpr int MINB =
        (MDT_FENG16_SM_THREADS / THREADS) < 1 ? 1 : (MDT_FENG16_SM_THREADS / THREADS);
    static constexpr int RSTRIDE = fft::Shape<N>::PADN + 4;
    // the transform's rows, the block's int8 input rows (up to 8 + 7), then
    // the FFT's compact twiddle table
    static constexpr size_t STAGE_OFF = (sizeof(float2) * (size_t)RSTRIDE * SB8 + 15) / 16 * 16;
    static constexpr size_t TW_OFF = STAGE_OFF + (size_t)(SB8 + 7) * 2 * N;
    static constexpr size_t SMEM = TW_OFF + sizeof(float2) * (size_t)fft::tw_compact_len<N>();
};

template <int CPI>
struct Samples;
template <>
struct Samples<1> {
    float re[1], im[1];
    __device__ __forceinline__ void load_shared(const uint8_t *p)
    {
        const char2 v = *reinterpret_cast<const char2 *>(p);
        re[0] = (float)v.x;
        im[0] = (float)v.y;
    }
    __device__ __forceinline__ void load(const char2 *p, bool ok)
    {
        const char2 v = ok ? __ldg(p) : make_char2(0, 0);
        re[0] = (float)v.x;
        im[0] = (float)v.y;
    }
};
template <>
struct Samples<2> {
    float re[2], im[2];
    __device__ __forceinline__ void load_shared(const uint8_t *p)
    {
        const char4 v = *reinterpret_cast<const char4 *>(p);
        re[0] = (float)v.x;
        im[0] = (float)v.y;
        re[1] = (float)v.z;
        im[1] = (float)v.w;
    }
    __device__ __forceinline__ void load(const char2 *p, bool ok)
    {
        const char4 v = ok ? __ldg(reinterpret_cast<const char4 *>(p)) : make_char4(0, 0, 0, 0);
        re[0] = (float)v.x;
        im[0] = (float)v.y;
        re[1] = (float)v.z;
        im[1] = (float)v.w;
    }
};

// 16-byte asynchronous global->shared copy; src_bytes 0 fills zeros.
__device__ __forceinline__ void cp_async16(void *dst, const void *src, int src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}

// The block's input rows (spectra s0 .. s0+7+NT-1 of element e) are copied
// into shared memory `stage` with cp.async, all in flight at once (rows past
// the input are zero-filled) and committed as one group.
template <int N, int NT, int THREADS>
__device__ __forceinline__ void stage_rows_async(const FengArgs &a, int s0, int e, uint8_t *stage)
{
    constexpr int NROW = SB8 + NT - 1;
    constexpr int RCHUNKS = 2 * N / 16;  // 16-byte chunks per input row
    const long rowlen = (long)a.ne * N;
    const int nin = a.nsp + NT - 1;  // input spectra of this integration
    for (int i = threadIdx.x; i < NROW * RCHUNKS; i += THREADS) {
        const int j = i / RCHUNKS, k = i - j * RCHUNKS;
        const int sp = s0 + j;
        const char2 *row = (sp < a.nhist) ? a.hist + (long)sp * rowlen
                                          : a.iq + (long)(sp - a.nhist) * rowlen;
        const bool in = sp < nin;
        cp_async16(stage + (size_t)j * 2 * N + 16 * k,
                   in ? reinterpret_cast<const uint8_t *>(row + (long)e * N) + 16 * k
                      : reinterpret_cast<const uint8_t *>(a.iq),
                   in ? 16 : 0);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Waits for the staged rows, then forms the block's 8 tap sums from them
// into the transform rows (no barrier after the sums).
template <int N, int NT, int THREADS>
__device__ __forceinline__ void tapsum_from_stage(const FengArgs &a, int s0, float2 *smem, int rstride,
                                                  const uint8_t *stage)
{
    constexpr int CPI = (N / THREADS >= 2) ? 2 : 1;  // channels per thread item
    constexpr int ITEMS = N / CPI;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    for (int it = threadIdx.x; it < ITEMS; it += THREADS) {
        const int c0 = it * CPI;
        if constexpr (CPI == 2 && MDT_FFT_F32X2) {
            // the two channels c0, c0 + 1 as one packed FP32 pair: one f32x2
            // fma per (row, tap) and component, each lane rounded as fmaf
            float2 w2[NT];
#pragma unroll
            for (int i = 0; i < NT; i++)
                w2[i] = __ldg(reinterpret_cast<const float2 *>(a.win + (long)i * N + c0));
            float2 ar[SB8], ai[SB8];
#pragma unroll
            for (int r = 0; r < SB8; r++) ar[r] = ai[r] = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < SB8 + NT - 1; j++) {
#if MDT_FENG_I2F_MAGIC
                // int8 -> float without the conversion unit: byte u = x + 128
                // placed in the mantissa of 2^23 gives 2^23 + u exactly, and
                // subtracting 2^23 + 128 leaves x exactly
                const uint32_t wv =
                    *reinterpret_cast<const uint32_t *>(stage + (size_t)j * 2 * N + 2 * c0) ^ 0x80808080u;
                constexpr float kOff = -8388736.0f;  // -(2^23 + 128)
                const float2 off = make_float2(kOff, kOff);
                const float2 xr = __fadd2_rn(make_float2(__uint_as_float(__byte_perm(wv, 0x4B000000u, 0x7540)),
                                                         __uint_as_float(__byte_perm(wv, 0x4B000000u, 0x7542))),
                                             off);
                const float2 xi = __fadd2_rn(make_float2(__uint_as_float(__byte_perm(wv, 0x4B000000u, 0x7541)),
                                                         __uint_as_float(__byte_perm(wv, 0x4B000000u, 0x7543))),
                                             off);
#else
                Samples<2> x;
                x.load_shared(stage + (size_t)j * 2 * N + 2 * c0);
                const float2 xr = make_float2(x.re[0], x.re[1]), xi = make_float2(x.im[0], x.im[1]);
#endif
#pragma unroll
                for (int r = 0; r < SB8; r++) {
                    const int i = j - r;
                    if (i >= 0 && i < NT) {
                        ar[r] = __ffma2_rn(w2[i], xr, ar[r]);
                        ai[r] = __ffma2_rn(w2[i], xi, ai[r]);
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < SB8; r++) {
                const bool live = s0 + r < a.nsp;
                float2 *row = smem + (size_t)r * rstride + fft::pad(c0);  // pad(c0 + 1) = pad(c0) + 1
                row[0] = live ? make_float2(ar[r].x, ai[r].x) : make_float2(0.f, 0.f);
                row[1] = live ? make_float2(ar[r].y, ai[r].y) : make_float2(0.f, 0.f);
            }
            continue;
        }
        float w[NT][CPI];
#pragma unroll
        for (int i = 0; i < NT; i++)
#pragma unroll
            for (int k = 0; k < CPI; k++) w[i][k] = __ldg(a.win + (long)i * N + c0 + k);
        float ar[SB8][CPI], ai[SB8][CPI];
#pragma unroll
        for (int r = 0; r < SB8; r++)
#pragma unroll
            for (int k = 0; k < CPI; k++) ar[r][k] = ai[r][k] = 0.0f;
#pragma unroll
        for (int j = 0; j < SB8 + NT - 1; j++) {
            Samples<CPI> x;
            x.load_shared(stage + (size_t)j * 2 * N + 2 * c0);
#pragma unroll
            for (int r = 0; r < SB8; r++) {
                const int i = j - r;
                if (i >= 0 && i < NT) {
#pragma unroll
                    for (int k = 0; k < CPI; k++) {
                        ar[r][k] = __fmaf_rn(w[i][k], x.re[k], ar[r][k]);
                        ai[r][k] = __fmaf_rn(w[i][k], x.im[k], ai[r][k]);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < SB8; r++) {
            const bool live = s0 + r < a.nsp;
#pragma unroll
            for (int k = 0; k < CPI; k++)
                smem[(size_t)r * rstride + fft::pad(c0 + k)] =
                    live ? make_float2(ar[r][k], ai[r][k]) : make_float2(0.f, 0.f);
        }
    }
}

// Stage, then tap sum; `mid()` runs while the copies are in flight.
template <int N, int NT, int THREADS, class Mid>
__device__ __forceinline__ void pfb_block8_to_smem(const FengArgs &a, int s0, int e, float2 *smem,
                                                   int rstride, uint8_t *stage, Mid &&mid)
{
    stage_rows_async<N, NT, THREADS>(a, s0, e, stage);
    mid();
    tapsum_from_stage<N, NT, THREADS>(a, s0, smem, rstride, stage);
}

// Block decode: blk = (kc * NE + e) * 4 + jsub, s0 = 32 kc + 8 jsub.
struct Block8 {
    int jsub, e, kc, s0;
    __device__ __forceinline__ Block8(int ne, int blk)
    {
        jsub = blk & 3;
        const int rest = blk >> 2;
        e = rest % ne;
        kc = rest / ne;
        s0 = kc * 32 + jsub * 8;
    }
    __device__ __forceinline__ explicit Block8(int ne) : Block8(ne, (int)blockIdx.x) {}
};

// Tap sum + FFT of the block's 8 rows; the spectra stay in shared memory
// (row r at fsm + r*RSTRIDE, channel c at pad(c)).  The FFT reads its
// twiddles from the compact table at TW_OFF (one 8-byte shared load per
// power instead of a scattered global load).
template <int N, int NT>
__device__ __forceinline__ void fengine_block8(const FengArgs &a, const Block8 &b, float2 *fsm)
{
    using C = FengBCfg<N>;
    float2 *tws = reinterpret_cast<float2 *>(reinterpret_cast<uint8_t *>(fsm) + C::TW_OFF);
    auto fill_tw = [&]() { fft::fill_tw_compact<N>(tws, a.tw, (int)threadIdx.x, C::THREADS); };
    if constexpr (NT > 0) {
        pfb_block8_to_smem<N, NT, C::THREADS>(a, b.s0, b.e, fsm, C::RSTRIDE,
                                              reinterpret_cast<uint8_t *>(fsm) + C::STAGE_OFF,
                                              fill_tw);
    } else {
        fill_tw();
        pfb_rows_to_smem<N, SB8, C::THREADS, true>(a, b.s0, b.e, fsm, C::RSTRIDE);
    }
    __syncthreads();
    const int lrow = threadIdx.x / C::TPR;
    const int t = threadIdx.x - lrow * C::TPR;
    auto none_load = [](int) { return make_float2(0.f, 0.f); };
    auto none_store = [](int, float2) {};
    fft::transform_row_tws<N, C::TPR, false, false>(fsm + (size_t)lrow * C::RSTRIDE, t, tws,
                                                    none_load, none_store);
}

// FP32 output in the 8-spectrum blocked layout of the plan's FP32 path (XB,
// fengine.cuh): one 64-byte run per channel for the block's (8 spectra,
// element).
template <int N>
__device__ __forceinline__ void store_c64b(const float2 *fsm, const Block8 &b, float2 *XB, int ne, int nsb)
{
    using C = FengBCfg<N>;
    float2 *base = XB + (size_t)(b.kc * 4 + b.jsub) * xb_block_stride(ne, N, nsb) + (size_t)b.e * SB8;
    const size_t cstride = (size_t)xb_chan_stride(ne, N, nsb);
    for (int it = threadIdx.x; it < N * 4; it += C::THREADS) {
        const int c = it >> 2, q = it & 3;  // q: pair of spectra
        const float2 v0 = fsm[(size_t)(2 * q) * C::RSTRIDE + fft::pad(c)];
        const float2 v1 = fsm[(size_t)(2 * q + 1) * C::RSTRIDE + fft::pad(c)];
        *reinterpret_cast<float4 *>(base + (size_t)c * cstride + 2 * q) =
            make_float4(v0.x, v0.y, v1.x, v1.y);
    }
}

// Work unit u decodes as blockIdx.x does in Block8; units whose 8-spectrum
// block lies past the last one (the tail of the last 32-spectrum chunk) hold
// no work.
__device__ __forceinline__ int next_c64b_unit(int u, int step, int nunits, int ne, int nsb)
{
    while (u < nunits && Block8(ne, u).kc * 4 + Block8(ne, u).jsub >= nsb) u += step;
    return u;
}

// Nch >= 1024 with NT = 4 or 8: persistent blocks (as many as fit on the GPU at once), each
// looping over units u = blockIdx.x, blockIdx.x + gridDim.x, ...  A unit's
// input rows are staged while the previous unit's FFT and stores run: the
// staging buffer is free once the tap sum has read it, so the next unit's
// copies are issued right after the tap-sum barrier.  The compact twiddle
// table is filled once per block.
// Otherwise one block per unit (smaller blocks already share an SM several
// at a time; NT = 0, other tap counts, forms the tap sums from global memory).
template <int N, int NT>
constexpr bool c64b_persistent()
{
    return NT > 0 && N >= 1024;
}

template <int N, int NT>
__global__ void __launch_bounds__(FengBCfg<N>::THREADS, FengBCfg<N>::MINB)
    fengine_c64b_kernel(FengArgs a, float2 *__restrict__ XB, int nsb, int nunits)
{
    using C = FengBCfg<N>;
    extern __shared__ float2 fsm[];
    if constexpr (!c64b_persistent<N, NT>()) {
        const Block8 b(a.ne);
        if (b.kc * 4 + b.jsub >= nsb) return;
        fengine_block8<N, NT>(a, b, fsm);
        store_c64b<N>(fsm, b, XB, a.ne, nsb);
    } else {
        uint8_t *stage = reinterpret_cast<uint8_t *>(fsm) + C::STAGE_OFF;
        float2 *tws = reinterpret_cast<float2 *>(reinterpret_cast<uint8_t *>(fsm) + C::TW_OFF);
        const int step = (int)gridDim.x;
        int u = next_c64b_unit((int)blockIdx.x, step, nunits, a.ne, nsb);
        if (u >= nunits) return;
        {
            const Block8 b(a.ne, u);
            stage_rows_async<N, NT, C::THREADS>(a, b.s0, b.e, stage);
        }
        fft::fill_tw_compact<N>(tws, a.tw, (int)threadIdx.x, C::THREADS);
        const int lrow = threadIdx.x / C::TPR;
        const int t = threadIdx.x - lrow * C::TPR;
        auto none_load = [](int) { return make_float2(0.f, 0.f); };
        auto none_store = [](int, float2) {};
        while (true) {
            const Block8 b(a.ne, u);
            // waits for the staged rows; its barrier also orders the previous
            // unit's stores (reads of the rows) before the new tap sums
            tapsum_from_stage<N, NT, C::THREADS>(a, b.s0, fsm, C::RSTRIDE, stage);
            __syncthreads();  // rows complete, staging buffer free
            const int un = next_c64b_unit(u + step, step, nunits, a.ne, nsb);
            if (un < nunits) {
                const Block8 bn(a.ne, un);
                stage_rows_async<N, NT, C::THREADS>(a, bn.s0, bn.e, stage);
            }
            fft::transform_row_tws<N, C::TPR, false, false>(fsm + (size_t)lrow * C::RSTRIDE, t, tws,
                                                            none_load, none_store);
            store_c64b<N>(fsm, b, XB, a.ne, nsb);
            if (un >= nunits) break;
            u = un;
        }
    }
}

// f16 / bf16 output (power-of-two scaled) in the tensor-core operand layout
// of xengine_tc.cu:  X16[kc][c][e][128 B], row = [re(32 spectra) | im(32
// spectra)], 16-byte chunk j stored at j ^ (e & 7).  The block's 8 spectra
// are one 16-byte chunk of re and one of im per channel, written straight
// from the transform's shared memory.
template <typename H>
__device__ __forceinline__ uint32_t pack2(float lo, float hi);
template <>
__device__ __forceinline__ uint32_t pack2<__half>(float lo, float hi)
{
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}
template <>
__device__ __forceinline__ uint32_t pack2<__nv_bfloat16>(float lo, float hi)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}

// QUANT: requantise each channel to integers in [-127, 127] with
// qscales[c] (rint, clamp) before the (exact) conversion to f16 -- the
// int8 operand of the exact int8 X-engine mode.
template <bool QUANT>
__device__ __forceinline__ float prep(float x, float sc)
{
    if constexpr (QUANT) {
        float v = rintf(x * sc);
        return fminf(fmaxf(v, -127.0f), 127.0f);
    } else {
        return x * sc;
    }
}

template <int N, int NT, typename H, bool QUANT>
__global__ void __launch_bounds__(FengBCfg<N>::THREADS, FengBCfg<N>::MINB)
    fengine_x16_kernel(FengArgs a, uint8_t *__restrict__ X16, int nep, int nkc, float scale,
                       const float *__restrict__ qscales)
{
    using C = FengBCfg<N>;
    extern __shared__ float2 fsm[];
    const Block8 b(a.ne);
    fengine_block8<N, NT>(a, b, fsm);

    // X16[kc][c][e][128 B]: rows of one (chunk, channel) are contiguous
    uint8_t *rowbase = X16 + ((size_t)b.kc * N * nep + b.e) * 128;
    const size_t cstride = (size_t)nep * 128;
    const int pre = (b.jsub ^ (b.e & 7)) << 4, pim = ((4 + b.jsub) ^ (b.e & 7)) << 4;
    for (int c = threadIdx.x; c < N; c += C::THREADS) {
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; r++) v[r] = fsm[(size_t)r * C::RSTRIDE + fft::pad(c)];
        const float sc = QUANT ? __ldg(qscales + c) : scale;
        uint4 ure, uim;
        ure.x = pack2<H>(prep<QUANT>(v[0].x, sc), prep<QUANT>(v[1].x, sc));
        ure.y = pack2<H>(prep<QUANT>(v[2].x, sc), prep<QUANT>(v[3].x, sc));
        ure.z = pack2<H>(prep<QUANT>(v[4].x, sc), prep<QUANT>(v[5].x, sc));
        ure.w = pack2<H>(prep<QUANT>(v[6].x, sc), prep<QUANT>(v[7].x, sc));
        uim.x = pack2<H>(prep<QUANT>(v[0].y, sc), prep<QUANT>(v[1].y, sc));
        uim.y = pack2<H>(prep<QUANT>(v[2].y, sc), prep<QUANT>(v[3].y, sc));
        uim.z = pack2<H>(prep<QUANT>(v[4].y, sc), prep<QUANT>(v[5].y, sc));
        uim.w = pack2<H>(prep<QUANT>(v[6].y, sc), prep<QUANT>(v[7].y, sc));
        uint8_t *row = rowbase + (size_t)c * cstride;
        *reinterpret_cast<uint4 *>(row + pre) = ure;
        *reinterpret_cast<uint4 *>(row + pim) = uim;
    }
}

// ------------------------------------------------------------------------
// Batched f16 F-engine: one launch for every job of a batch that shares
// (Nch, Ntaps).  Job j owns blocks [blk0[j], blk0[j+1]); within a job the
// blocks decode as in fengine_x16_kernel.
template <int N, int NT>
__global__ void __launch_bounds__(FengBCfg<N>::THREADS, FengBCfg<N>::MINB)
    fengine_x16_batched_kernel(const FJob *__restrict__ jobs, int njobs, const float2 *tw)
{
    using C = FengBCfg<N>;
    extern __shared__ float2 fsm[];
    int j = 0;
    while (j + 1 < njobs && (int)blockIdx.x >= jobs[j + 1].blk0) j++;
    const FJob jb = jobs[j];
    FengArgs a;
    a.hist = nullptr;
    a.iq = jb.iq;
    a.nhist = 0;
    a.ne = jb.ne;
    a.ntaps = NT;
    a.nsp = jb.nsp;
    a.ngroups = 0;
    a.win = jb.win;
    a.tw = tw;
    a.X = nullptr;
    const Block8 b(jb.ne, (int)blockIdx.x - jb.blk0);
    fengine_block8<N, NT>(a, b, fsm);

    uint8_t *rowbase = jb.X16 + ((size_t)b.kc * N * jb.nep + b.e) * 128;
    const size_t cstride = (size_t)jb.nep * 128;
    const int pre = (b.jsub ^ (b.e & 7)) << 4, pim = ((4 + b.jsub) ^ (b.e & 7)) << 4;
    const float sc = jb.scale;
    for (int c = threadIdx.x; c < N; c += C::THREADS) {
        float2 v[8];
#pragma unroll
        for (int r = 0; r < 8; r++) v[r] = fsm[(size_t)r * C::RSTRIDE + fft::pad(c)];
        uint4 ure, uim;
        ure.x = pack2<__half>(v[0].x * sc, v[1].x * sc);
        ure.y = pack2<__half>(v[2].x * sc, v[3].x * sc);
        ure.z = pack2<__half>(v[4].x * sc, v[5].x * sc);
        ure.w = pack2<__half>(v[6].x * sc, v[7].x * sc);
        uim.x = pack2<__half>(v[0].y * sc, v[1].y * sc);
        uim.y = pack2<__half>(v[2].y * sc, v[3].y * sc);
        uim.z = pack2<__half>(v[4].y * sc, v[5].y * sc);
        uim.w = pack2<__half>(v[6].y * sc, v[7].y * sc);
        uint8_t *row = rowbase + (size_t)c * cstride;
        *reinterpret_cast<uint4 *>(row + pre) = ure;
        *reinterpret_cast<uint4 *>(row + pim) = uim;
    }
}

// Per-channel mean power over the elements and spectra of an XB buffer
// (nsb blocks of 8 spectra, nsp valid): pw[c] = mean |X|^2.  Each thread sums
// its values in (block, element, spectrum) order whatever the layout's
// strides, so the result does not depend on them.
__global__ void channel_power_kernel(const float2 *__restrict__ XB, int ne, int nsb, int nsp,
                                     long cstride, long bstride, float *__restrict__ pw)
{
    const int c = blockIdx.x;
    const float2 *xc = XB + (size_t)c * cstride;
    const int run = ne * 8;  // complex64 values of one (block, channel)
    double acc = 0.0;
    for (long i = threadIdx.x; i < (long)nsb * run; i += blockDim.x) {
        const long sb = i / run;
        const float2 v = xc[sb * bstride + (i - sb * run)];
        acc += (double)v.x * v.x + (double)v.y * v.y;
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) pw[c] = (float)(red[0] / ((double)ne * nsp));
}

// scale[c] = target_rms / sqrt(power[c]) (1 when the channel carries no power).
__global__ void scales_from_power_kernel(const float *__restrict__ pw, int nch, float target_rms,
                                         float *__restrict__ scales)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nch) scales[c] = pw[c] > 0.0f ? target_rms / sqrtf(pw[c]) : 1.0f;
}

// Calls f.run<N, NT>() for the runtime (nch, ntaps).
template <class F>
static mdt_status dispatch_block8(int nch, int ntaps, F f)
{
#define MDT_NT_CASES(NV)                                                       \
    case NV:                                                                   \
        return ntaps == 4 ? f.template run<NV, 4>()                            \
                          : (ntaps == 8 ? f.template run<NV, 8>() : f.template run<NV, 0>());
    switch (nch) {
        MDT_NT_CASES(32)
        MDT_NT_CASES(64)
        MDT_NT_CASES(128)
        MDT_NT_CASES(256)
        MDT_NT_CASES(512)
        MDT_NT_CASES(1024)
        MDT_NT_CASES(2048)
        default: break;
    }
#undef MDT_NT_CASES
    set_error("F-engine: Nch must be a power of two in [32, 2048] for this path");
    return MDT_ERR_NOT_SUPPORTED;
}

template <typename H>
struct Feng16Run {
    FengArgs a;
    uint8_t *X16;
    int nep, nkc;
    float scale;
    cudaStream_t stream;
    const float *qscales = nullptr;  // non-null: requantise (exact int8 mode)
    template <int N, int NT>
    mdt_status run()
    {
        using C = FengBCfg<N>;
        static_assert(C::SMEM <= 232448, "F-engine shared memory");
        mdt_status st;
        a.tw = fft_twiddles(N, &st);
        if (!a.tw) return st;
        long blocks = (long)a.ne * nkc * 4;
        if (blocks > 0x7fffffffL) return invalid("fengine_x16: grid too large");
        auto kern = qscales ? fengine_x16_kernel<N, NT, H, true> : fengine_x16_kernel<N, NT, H, false>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)C::SMEM);
        if (e != cudaSuccess) return cuda_status(e, "fengine_x16 smem attribute");
        kern<<<(unsigned)blocks, C::THREADS, C::SMEM, stream>>>(a, X16, nep, nkc, scale, qscales);
        return launch_status("fengine_x16_kernel");
    }
};

struct FengBRun {
    FengArgs a;
    float2 *XB;
    int nsb;
    cudaStream_t stream;
    // optional caller-provided twiddles: the tables for N = 32, 64, ..., 2048
    // back to back (the table for N starts at entry N - 32); null = the
    // library's per-device tables
    const float2 *tw_concat = nullptr;
    template <int N, int NT>
    mdt_status run()
    {
        using C = FengBCfg<N>;
        static_assert(C::SMEM <= 232448, "F-engine shared memory");
        mdt_status st = MDT_SUCCESS;
        a.tw = tw_concat ? tw_concat + (N - 32) : fft_twiddles(N, &st);
        if (!a.tw) return st;
        cudaError_t e = cudaFuncSetAttribute(fengine_c64b_kernel<N, NT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)C::SMEM);
        if (e != cudaSuccess) return cuda_status(e, "fengine_c64b smem attribute");
        const long nkc = (nsb + 3) / 4;
        const long units = (long)a.ne * nkc * 4;
        if (units > 0x7fffffffL) return invalid("fengine_c64b: grid too large");
        long grid = units;
        if (c64b_persistent<N, NT>()) {  // the blocks that fit on the GPU at once
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fengine_c64b_kernel<N, NT>,
                                                              C::THREADS, C::SMEM);
            if (e != cudaSuccess) return cuda_status(e, "fengine_c64b occupancy");
            grid = std::min(units, (long)std::max(per_sm, 1) * sm_count());
        }
        if (grid == 0) return MDT_SUCCESS;
        fengine_c64b_kernel<N, NT><<<(unsigned)grid, C::THREADS, C::SMEM, stream>>>(a, XB, nsb,
                                                                                   (int)units);
        return launch_status("fengine_c64b_kernel");
    }
};

static FengArgs make_args(int ne, int ntaps, int nsp, const int8_t *hist, int nhist,
                          const int8_t *iq, const float *win)
{
    FengArgs a;
    a.hist = reinterpret_cast<const char2 *>(hist);
    a.iq = reinterpret_cast<const char2 *>(iq);
    a.nhist = nhist;
    a.ne = ne;
    a.ntaps = ntaps;
    a.nsp = nsp;
    a.win = win;
    a.X = nullptr;
    a.ngroups = 0;
    a.tw = nullptr;
    return a;
}

// ab_fmt 0 = f16, 1 = bf16; X16 sized nch * nkc * nep * 128 bytes, rows
// >= NE must already be zero (they are never written).
mdt_status fengine_x16(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                       const int8_t *iq, const float *win, void *X16, int nep, int nkc,
                       int ab_fmt, float scale, cudaStream_t stream)
{
    if (((uintptr_t)iq | (uintptr_t)hist | (uintptr_t)win | (uintptr_t)X16) & 15)
        return invalid("fengine_x16: buffers must be 16-byte aligned");
    FengArgs a = make_args(ne, ntaps, nsp, hist, nhist, iq, win);
    if (ab_fmt == 1)
        return dispatch_block8(nch, ntaps,
                               Feng16Run<__nv_bfloat16>{a, (uint8_t *)X16, nep, nkc, scale, stream});
    return dispatch_block8(nch, ntaps, Feng16Run<__half>{a, (uint8_t *)X16, nep, nkc, scale, stream});
}

struct FengBatchRun {
    const FJob *jobs;
    int njobs;
    long nblocks;
    cudaStream_t stream;
    template <int N, int NT>
    mdt_status run()
    {
        if constexpr (NT == 0) {
            return invalid("batched F-engine: Ntaps must be 4 or 8");
        } else {
            using C = FengBCfg<N>;
            mdt_status st;
            const float2 *tw = fft_twiddles(N, &st);
            if (!tw) return st;
            cudaError_t e = cudaFuncSetAttribute(fengine_x16_batched_kernel<N, NT>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)C::SMEM);
            if (e != cudaSuccess) return cuda_status(e, "batched F-engine smem attribute");
            if (nblocks > 0x7fffffffL) return invalid("batched F-engine: grid too large");
            fengine_x16_batched_kernel<N, NT><<<(unsigned)nblocks, C::THREADS, C::SMEM, stream>>>(
                jobs, njobs, tw);
            return launch_status("fengine_x16_batched_kernel");
        }
    }
};

// Batched f16 F-engine launch over jobs sharing (nch, ntaps in {4, 8});
// `jobs` is a device array of njobs FJob, `nblocks` the total block count.
mdt_status fengine_x16_batched(int nch, int ntaps, const FJob *jobs, int njobs, long nblocks,
                               cudaStream_t stream)
{
    return dispatch_block8(nch, ntaps, FengBatchRun{jobs, njobs, nblocks, stream});
}

// Per-channel int8 scales from the power of a blocked FP32 F-output:
// scale[c] = target_rms / rms_c.  pw: nch floats of workspace.
mdt_status channel_scales(const float2 *XB, int ne, int nch, int nsp, float target_rms, float *pw,
                          float *scales, cudaStream_t stream)
{
    const long nsb = (nsp + 7) / 8;
    channel_power_kernel<<<nch, 256, 0, stream>>>(XB, ne, (int)nsb, nsp, xb_chan_stride(ne, nch, nsb),
                                                  xb_block_stride(ne, nch, nsb), pw);
    mdt_status st = launch_status("channel_power_kernel");
    if (st != MDT_SUCCESS) return st;
    scales_from_power_kernel<<<(unsigned)cdiv(nch, 256), 256, 0, stream>>>(pw, nch, target_rms,
                                                                           scales);
    return launch_status("scales_from_power_kernel");
}

// Exact-int8 F-engine: X16 layout holding integers in [-127, 127] (f16),
// requantised per channel with qscales.
mdt_status fengine_q8(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                      const int8_t *iq, const float *win, void *X16, int nep, int nkc,
                      const float *qscales, cudaStream_t stream)
{
    if (((uintptr_t)iq | (uintptr_t)hist | (uintptr_t)win | (uintptr_t)X16) & 15)
        return invalid("fengine_q8: buffers must be 16-byte aligned");
    if (!qscales) return invalid("fengine_q8: null scales");
    FengArgs a = make_args(ne, ntaps, nsp, hist, nhist, iq, win);
    Feng16Run<__half> run{a, (uint8_t *)X16, nep, nkc, 1.0f, stream};
    run.qscales = qscales;
    return dispatch_block8(nch, ntaps, run);
}

// FP32 F-engine into the 8-spectrum blocked layout XB (fengine.cuh).
mdt_status fengine_c64b(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                        const int8_t *iq, const float *win, float2 *XB, cudaStream_t stream)
{
    if (((uintptr_t)iq | (uintptr_t)hist | (uintptr_t)win | (uintptr_t)XB) & 15)
        return invalid("fengine_c64b: buffers must be 16-byte aligned");
    FengArgs a = make_args(ne, ntaps, nsp, hist, nhist, iq, win);
    return dispatch_block8(nch, ntaps, FengBRun{a, XB, (nsp + 7) / 8, stream});
}

// As fengine_c64b, with the twiddle tables supplied by the caller (see
// FengBRun::tw_concat); allocates nothing.
mdt_status fengine_c64b_given_twiddles(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                       const float *win, float2 *XB, const float2 *tw_concat,
                                       cudaStream_t stream)
{
    if (((uintptr_t)iq | (uintptr_t)win | (uintptr_t)XB) & 15)
        return invalid("fengine_c64b: buffers must be 16-byte aligned");
    FengArgs a = make_args(ne, ntaps, nsp, nullptr, 0, iq, win);
    FengBRun run{a, XB, (nsp + 7) / 8, stream};
    run.tw_concat = tw_concat;
    return dispatch_block8(nch, ntaps, run);
}

// ------------------------------------------------------------------------
template <int N>
static mdt_status launch_feng(FengArgs a, cudaStream_t stream)
{
    using C = FengCfg<N>;
    mdt_status st;
    a.tw = fft_twiddles(N, &st);
    if (!a.tw) return st;
    if (C::SMEM > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fengine_f32_kernel<N>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)C::SMEM);
        if (e != cudaSuccess) return cuda_status(e, "fengine smem attribute");
    }
    a.ngroups = (int)cdiv(a.ne, C::ROWS);
    long blocks = (long)a.nsp * a.ngroups;
    if (blocks > 0x7fffffffL) return invalid("fengine: grid too large");
    fengine_f32_kernel<N><<<(unsigned)blocks, C::THREADS, C::SMEM, stream>>>(a);
    return launch_status("fengine_f32_kernel");
}

mdt_status fengine_f32(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                       const int8_t *iq, const float *win, float2 *X, cudaStream_t stream)
{
    // the tap sum reads 16-byte vectors of samples and window coefficients
    if (((uintptr_t)iq | (uintptr_t)hist | (uintptr_t)win) & 15)
        return invalid("fengine: sample and window buffers must be 16-byte aligned");
    FengArgs a;
    a.hist = reinterpret_cast<const char2 *>(hist);
    a.iq = reinterpret_cast<const char2 *>(iq);
    a.nhist = nhist;
    a.ne = ne;
    a.ntaps = ntaps;
    a.nsp = nsp;
    a.win = win;
    a.X = X;
    switch (nch) {
        case 32: return launch_feng<32>(a, stream);
        case 64: return launch_feng<64>(a, stream);
        case 128: return launch_feng<128>(a, stream);
        case 256: return launch_feng<256>(a, stream);
        case 512: return launch_feng<512>(a, stream);
        case 1024: return launch_feng<1024>(a, stream);
        case 2048: return launch_feng<2048>(a, stream);
        case 4096: return launch_feng<4096>(a, stream);
        case 8192: return launch_feng<8192>(a, stream);
        case 16384: return launch_feng<16384>(a, stream);
        default: break;
    }
    set_error("fengine: Nch must be a power of two in [32, 16384]");
    return MDT_ERR_NOT_SUPPORTED;
}

mdt_status check_dims(int ne, int nch, int ntaps, int nsp)
{
    if (ne < MDT_MIN_ELEMENTS || ne > MDT_MAX_ELEMENTS)
        return invalid("NE out of range [3, 2048]");
    if (nch < MDT_MIN_CHANNELS || nch > MDT_MAX_CHANNELS || !is_pow2(nch))
        return invalid("Nch must be a power of two in [32, 16384]");
    if (ntaps < MDT_MIN_TAPS || ntaps > MDT_MAX_TAPS) return invalid("Ntaps out of range [4, 128]");
    if (nsp < MDT_MIN_SPECTRA || nsp > MDT_MAX_SPECTRA)
        return invalid("Nspectra out of range [2, 16384]");
    return MDT_SUCCESS;
}

}  // namespace mdt

extern "C" MDT_API mdt_status mdt_fengine_x16(int ne, int nch, int ntaps, int nsp,
                                              const int8_t *iq, const float *window, void *X16,
                                              int ab_fmt, float scale, cudaStream_t stream)
{
    mdt_status st = mdt::check_dims(ne, nch, ntaps, nsp);
    if (st != MDT_SUCCESS) return st;
    if (!iq || !window || !X16 || (ab_fmt != 0 && ab_fmt != 1) || !(scale > 0.0f))
        return mdt::invalid("fengine_x16: bad arguments");
    const int nep = (ne + 15) / 16 * 16, nkc = (nsp + 31) / 32;
    return mdt::fengine_x16(ne, nch, ntaps, nsp, nullptr, 0, iq, window, X16, nep, nkc, ab_fmt,
                            scale, stream);
}

extern "C" MDT_API mdt_status mdt_fengine_q8(int ne, int nch, int ntaps, int nsp,
                                             const int8_t *iq, const float *window, void *X16,
                                             const float *qscales, cudaStream_t stream)
{
    mdt_status st = mdt::check_dims(ne, nch, ntaps, nsp);
    if (st != MDT_SUCCESS) return st;
    if (!iq || !window || !X16 || !qscales) return mdt::invalid("fengine_q8: null pointer");
    const int nep = (ne + 15) / 16 * 16, nkc = (nsp + 31) / 32;
    return mdt::fengine_q8(ne, nch, ntaps, nsp, nullptr, 0, iq, window, X16, nep, nkc, qscales,
                           stream);
}

extern "C" MDT_API mdt_status mdt_fengine_c64b(int ne, int nch, int ntaps, int nsp,
                                               const int8_t *iq, const float *window, void *XB,
                                               cudaStream_t stream)
{
    mdt_status st = mdt::check_dims(ne, nch, ntaps, nsp);
    if (st != MDT_SUCCESS) return st;
    if (!iq || !window || !XB) return mdt::invalid("fengine_c64b: null pointer");
    return mdt::fengine_c64b(ne, nch, ntaps, nsp, nullptr, 0, iq, window, (float2 *)XB, stream);
}

extern "C" MDT_API mdt_status mdt_fengine_f32(int ne, int nch, int ntaps, int nsp,
                                              const int8_t *iq, const float *window, void *X,
                                              cudaStream_t stream)
{
    mdt_status st = mdt::check_dims(ne, nch, ntaps, nsp);
    if (st != MDT_SUCCESS) return st;
    if (!iq || !window || !X) return mdt::invalid("fengine_f32: null pointer");
    return mdt::fengine_f32(ne, nch, ntaps, nsp, nullptr, 0, iq, window, (float2 *)X, stream);
}
