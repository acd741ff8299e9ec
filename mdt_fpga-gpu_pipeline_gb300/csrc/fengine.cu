// fengine.cu -- fused F-engine: int8 I/Q -> PFB tap sum -> FFT -> channel-major
// corner turn, in one kernel (the reference runs PpS_Batch, cufftExecC2C and
// ReorderFOutput as three passes over HBM, MDT_OneStation_client.cu:1083,
// 1105,1114).
//
// A block transforms ROWS rows (spectrum s, elements e0..e0+ROWS-1):
//  * the tap sum P[c] = sum_i W[i*Nch + c] * iq[s+i][e][c] is formed with
//    16-byte vector loads into shared memory, accumulated with fmaf from zero
//    in increasing i, the order of PpS_Batch (MDT_device_functions.cu:191-200),
//    so P is bit-identical to the drop-in kernel's output on the same samples;
//  * the FFT passes run in shared memory (fft_core.cuh), the last one leaves
//    the spectrum in natural order in shared memory;
//  * the block writes X[(c*Nsp + s)*NE + e] (ReorderFOutput's layout,
//    MDT_device_functions.cu:255): for each channel the ROWS elements are
//    contiguous.
// Input spectra may come from two buffers: the first `nhist` spectra from
// `hist` (the PFB history carried between integrations, reference
// MDT_OneStation_client.cu:1170) and the rest from `iq`.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fft_core.cuh"

namespace mdt {

// Rows (elements) per block of the FP32 F-engine.  Small blocks let several
// blocks share an SM, so one block's sample loads overlap another's FFT
// passes and barriers.
#ifndef MDT_FENG_ROWS
#define MDT_FENG_ROWS 4
#endif
// Threads per SM the register budget is sized for (64K registers / this).
#ifndef MDT_FENG_SM_THREADS
#define MDT_FENG_SM_THREADS 1536
#endif

template <int N>
struct FengCfg {
    static constexpr int TPR = fft::Shape<N>::TPR;
    static constexpr int RMAX = (1024 / TPR) < 1 ? 1 : 1024 / TPR;
    static constexpr int ROWS = MDT_FENG_ROWS < RMAX ? MDT_FENG_ROWS : RMAX;
    static constexpr int THREADS = ROWS * TPR;
    // resident blocks per SM requested from the register allocator
    static constexpr int MINB = (MDT_FENG_SM_THREADS / THREADS) < 1 ? 1 : (MDT_FENG_SM_THREADS / THREADS);
    static constexpr int RSTRIDE = 2 * fft::Shape<N>::PADN + 8;  // floats per row (bank skew)
    static constexpr size_t SMEM = sizeof(float) * (size_t)RSTRIDE * ROWS;
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

// Polyphase tap sum of the block's ROWS rows into shared memory (natural
// channel order, padded): each work item is 8 consecutive channels of one
// row, read as one 16-byte int8 I/Q vector and two float4 window vectors per
// tap; accumulation is fmaf from zero in increasing tap order.
// Row r of the block is (spectrum s0, element e0 + r), or with SPECTRA_ROWS
// (spectrum s0 + r, element e0); rows past NE or Nsp are zero.
template <int N, int ROWS, int THREADS, bool SPECTRA_ROWS = false>
__device__ __forceinline__ void pfb_rows_to_smem(const FengArgs &a, int s0, int e0, float *smem,
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
        float *sre = smem + (size_t)r * rstride;
        float *sim = sre + fft::Shape<N>::PADN;
        const int p0 = fft::pad(c0);  // c0 % 8 == 0: pad(c0 + k) = p0 + k
#pragma unroll
        for (int k = 0; k < 8; k++) {
            sre[p0 + k] = re[k];
            sim[p0 + k] = im[k];
        }
    }
}

template <int N>
__global__ void __launch_bounds__(FengCfg<N>::THREADS, FengCfg<N>::MINB) fengine_f32_kernel(FengArgs a)
{
    using C = FengCfg<N>;
    extern __shared__ float smem[];
    const long blk = blockIdx.x;
    const int s = (int)(blk / a.ngroups);
    const int e0 = (int)(blk - (long)s * a.ngroups) * C::ROWS;
    const int lrow = threadIdx.x / C::TPR;
    const int t = threadIdx.x - lrow * C::TPR;
    float *sre = smem + (size_t)lrow * C::RSTRIDE;
    float *sim = sre + fft::Shape<N>::PADN;

    pfb_rows_to_smem<N, C::ROWS, C::THREADS>(a, s, e0, smem, C::RSTRIDE);
    __syncthreads();
    auto none_load = [](int) { return make_float2(0.f, 0.f); };
    auto none_store = [](int, float2) {};
    fft::transform_row<N, C::TPR, false, false>(sre, sim, t, a.tw, none_load, none_store);

    // corner turn: ROWS contiguous elements per channel
    const int nrow = min(C::ROWS, a.ne - e0);
    float2 *dst = a.X + (long)s * a.ne + e0;
    const long cstride = (long)a.nsp * a.ne;
    for (int k = threadIdx.x; k < N * C::ROWS; k += C::THREADS) {
        const int c = k / C::ROWS, r = k - c * C::ROWS;
        if (r < nrow) {
            const float *rr = smem + (size_t)r * C::RSTRIDE;
            dst[(long)c * cstride + r] =
                make_float2(rr[fft::pad(c)], rr[fft::Shape<N>::PADN + fft::pad(c)]);
        }
    }
}

// ------------------------------------------------------------------------
// F-engine for the tensor-core X-engine: same tap sum and FFT, output scaled
// by a power of two and rounded to f16 / bf16 in the X16 operand layout of
// xengine_tc.cu:  X16[c][kc][e][128 B], row = [re(32 spectra) | im(32 spectra)],
// 16-byte chunk j stored at j ^ (e & 7).  A block owns one element and SB
// consecutive spectra (SB = 32 when Nch <= 1024), transforms them R rows at a
// time, stages the rounded values per channel in shared memory and writes
// whole swizzled chunks.
template <int N>
struct Feng16Cfg {
    static constexpr int TPR = fft::Shape<N>::TPR;
    static constexpr int SB = (32 * N * 4 <= 131072) ? 32 : 131072 / (N * 4);
    static constexpr int RMAX = (1024 / TPR) < 1 ? 1 : 1024 / TPR;
    static constexpr int R = SB < RMAX ? SB : RMAX;
    static constexpr int THREADS = R * TPR;
    static constexpr int RSTRIDE = 2 * fft::Shape<N>::PADN + 8;
    static constexpr int SROWW = SB + 1;  // staging words per channel row: 2*SB halves + pad
    static constexpr size_t FFT_SMEM = sizeof(float) * (size_t)RSTRIDE * R;
    static constexpr size_t SMEM = FFT_SMEM + sizeof(uint32_t) * (size_t)SROWW * N;
};

template <typename H>
__device__ __forceinline__ H to_half(float x);
template <>
__device__ __forceinline__ __half to_half<__half>(float x)
{
    return __float2half_rn(x);
}
template <>
__device__ __forceinline__ __nv_bfloat16 to_half<__nv_bfloat16>(float x)
{
    return __float2bfloat16_rn(x);
}

template <int N, typename H>
__global__ void __launch_bounds__(Feng16Cfg<N>::THREADS)
    fengine_x16_kernel(FengArgs a, uint8_t *__restrict__ X16, int nep, int nkc, float scale)
{
    using C = Feng16Cfg<N>;
    extern __shared__ float smem[];
    uint16_t *stage = reinterpret_cast<uint16_t *>(smem + C::FFT_SMEM / sizeof(float));
    const int nsblk = nkc * (32 / C::SB);
    const int e = blockIdx.x % a.ne;
    const int sblk = blockIdx.x / a.ne;
    const int s0 = sblk * C::SB;
    const int lrow = threadIdx.x / C::TPR;
    const int t = threadIdx.x - lrow * C::TPR;
    float *sre = smem + (size_t)lrow * C::RSTRIDE;
    float *sim = sre + fft::Shape<N>::PADN;
    auto none_load = [](int) { return make_float2(0.f, 0.f); };
    auto none_store = [](int, float2) {};
    (void)nsblk;

    for (int round = 0; round < C::SB / C::R; round++) {
        pfb_rows_to_smem<N, C::R, C::THREADS, true>(a, s0 + round * C::R, e, smem, C::RSTRIDE);
        __syncthreads();
        fft::transform_row<N, C::TPR, false, false>(sre, sim, t, a.tw, none_load, none_store);
        for (int it = threadIdx.x; it < N * C::R; it += C::THREADS) {
            const int r = it % C::R, c = it / C::R;
            const float *rr = smem + (size_t)r * C::RSTRIDE;
            const int sl = round * C::R + r;
            const H hr = to_half<H>(rr[fft::pad(c)] * scale);
            const H hi = to_half<H>(rr[fft::Shape<N>::PADN + fft::pad(c)] * scale);
            stage[(size_t)c * 2 * C::SROWW + sl] = *reinterpret_cast<const uint16_t *>(&hr);
            stage[(size_t)c * 2 * C::SROWW + C::SB + sl] = *reinterpret_cast<const uint16_t *>(&hi);
        }
        __syncthreads();
    }

    // swizzled 16-byte chunks: local chunk u covers halves 8u..8u+7 of the
    // staged row (re for u < SB/8, im otherwise)
    const int kc = s0 / 32, soff = s0 % 32;
    constexpr int NU = C::SB / 4;
    const uint32_t *sw = reinterpret_cast<const uint32_t *>(stage);
    uint8_t *rowbase = X16 + (size_t)kc * nep * 128 + (size_t)e * 128;
    const size_t cstride = (size_t)nkc * nep * 128;
    for (int it = threadIdx.x; it < N * NU; it += C::THREADS) {
        const int u = it % NU, c = it / NU;
        const int j = (u < C::SB / 8) ? (soff / 8 + u) : (4 + soff / 8 + (u - C::SB / 8));
        const uint32_t *w = sw + (size_t)c * C::SROWW + 4 * u;
        uint4 v = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4 *>(rowbase + (size_t)c * cstride + ((j ^ (e & 7)) << 4)) = v;
    }
}

template <int N, typename H>
static mdt_status launch_feng16(FengArgs a, uint8_t *X16, int nep, int nkc, float scale,
                                cudaStream_t stream)
{
    using C = Feng16Cfg<N>;
    static_assert(C::SMEM <= 232448, "F-engine X16 shared memory");
    mdt_status st;
    a.tw = fft_twiddles(N, &st);
    if (!a.tw) return st;
    cudaError_t e = cudaFuncSetAttribute(fengine_x16_kernel<N, H>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    if (e != cudaSuccess) return cuda_status(e, "fengine_x16 smem attribute");
    long blocks = (long)a.ne * nkc * (32 / C::SB);
    if (blocks > 0x7fffffffL) return invalid("fengine_x16: grid too large");
    fengine_x16_kernel<N, H><<<(unsigned)blocks, C::THREADS, C::SMEM, stream>>>(a, X16, nep, nkc,
                                                                              scale);
    return launch_status("fengine_x16_kernel");
}

template <typename H>
static mdt_status fengine_x16_dispatch(int nch, FengArgs a, uint8_t *X16, int nep, int nkc,
                                       float scale, cudaStream_t stream)
{
    switch (nch) {
        case 32: return launch_feng16<32, H>(a, X16, nep, nkc, scale, stream);
        case 64: return launch_feng16<64, H>(a, X16, nep, nkc, scale, stream);
        case 128: return launch_feng16<128, H>(a, X16, nep, nkc, scale, stream);
        case 256: return launch_feng16<256, H>(a, X16, nep, nkc, scale, stream);
        case 512: return launch_feng16<512, H>(a, X16, nep, nkc, scale, stream);
        case 1024: return launch_feng16<1024, H>(a, X16, nep, nkc, scale, stream);
        case 2048: return launch_feng16<2048, H>(a, X16, nep, nkc, scale, stream);
        case 4096: return launch_feng16<4096, H>(a, X16, nep, nkc, scale, stream);
        default: break;
    }
    set_error("fengine_x16: Nch must be a power of two in [32, 4096]");
    return MDT_ERR_NOT_SUPPORTED;
}

// ab_fmt 0 = f16, 1 = bf16; X16 sized nch * nkc * nep * 128 bytes, rows
// >= NE must already be zero (they are never written).
mdt_status fengine_x16(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                       const int8_t *iq, const float *win, void *X16, int nep, int nkc,
                       int ab_fmt, float scale, cudaStream_t stream)
{
    if (((uintptr_t)iq | (uintptr_t)hist | (uintptr_t)win | (uintptr_t)X16) & 15)
        return invalid("fengine_x16: buffers must be 16-byte aligned");
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
    if (ab_fmt == 1)
        return fengine_x16_dispatch<__nv_bfloat16>(nch, a, (uint8_t *)X16, nep, nkc, scale, stream);
    return fengine_x16_dispatch<__half>(nch, a, (uint8_t *)X16, nep, nkc, scale, stream);
}

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

extern "C" MDT_API mdt_status mdt_fengine_f32(int ne, int nch, int ntaps, int nsp,
                                              const int8_t *iq, const float *window, void *X,
                                              cudaStream_t stream)
{
    mdt_status st = mdt::check_dims(ne, nch, ntaps, nsp);
    if (st != MDT_SUCCESS) return st;
    if (!iq || !window || !X) return mdt::invalid("fengine_f32: null pointer");
    return mdt::fengine_f32(ne, nch, ntaps, nsp, nullptr, 0, iq, window, (float2 *)X, stream);
}
