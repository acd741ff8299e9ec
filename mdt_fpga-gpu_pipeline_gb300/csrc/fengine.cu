// fengine.cu -- fused F-engine: int8 I/Q -> PFB tap sum -> FFT -> channel-major
// corner turn, in one kernel (the reference runs PpS_Batch, cufftExecC2C and
// ReorderFOutput as three passes over HBM, MDT_OneStation_client.cu:1083,
// 1105,1114).
//
// A block transforms ROWS rows (spectrum s, elements e0..e0+ROWS-1):
//  * the first Stockham pass takes its inputs straight from the tap sum
//      P[c] = sum_i W[i*Nch + c] * iq[s+i][e][c]
//    accumulated with fmaf from zero in increasing i, the order of
//    PpS_Batch (MDT_device_functions.cu:191-200), so P is bit-identical to
//    the drop-in kernel's output on the same samples;
//  * the passes run in shared memory (fft_core.cuh), the last one leaves the
//    spectrum in natural order in shared memory;
//  * the block writes X[(c*Nsp + s)*NE + e] (ReorderFOutput's layout,
//    MDT_device_functions.cu:255): for each channel the ROWS elements are
//    contiguous.
// Input spectra may come from two buffers: the first `nhist` spectra from
// `hist` (the PFB history carried between integrations, reference
// MDT_OneStation_client.cu:1170) and the rest from `iq`.
#include "fft_core.cuh"

namespace mdt {

template <int N>
struct FengCfg {
    static constexpr int TPR = fft::Shape<N>::TPR;
    static constexpr int ROWS = (1024 / TPR) >= 4 ? 4 : ((1024 / TPR) < 1 ? 1 : 1024 / TPR);
    static constexpr int THREADS = ROWS * TPR;
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

template <int N>
__global__ void __launch_bounds__(FengCfg<N>::THREADS) fengine_f32_kernel(FengArgs a)
{
    using C = FengCfg<N>;
    extern __shared__ float smem[];
    const long blk = blockIdx.x;
    const int s = (int)(blk / a.ngroups);
    const int e0 = (int)(blk - (long)s * a.ngroups) * C::ROWS;
    const int lrow = threadIdx.x / C::TPR;
    const int t = threadIdx.x - lrow * C::TPR;
    const int e = e0 + lrow;
    const bool valid = e < a.ne;
    float *sre = smem + (size_t)lrow * C::RSTRIDE;
    float *sim = sre + fft::Shape<N>::PADN;
    const long rowlen = (long)a.ne * N;  // samples per spectrum

    auto load = [&](int c) -> float2 {
        float re = 0.0f, im = 0.0f;
        if (valid) {
            for (int i = 0; i < a.ntaps; i++) {
                const int sp = s + i;
                const char2 *src = (sp < a.nhist) ? a.hist + (long)sp * rowlen
                                                  : a.iq + (long)(sp - a.nhist) * rowlen;
                const char2 x = __ldg(src + (long)e * N + c);
                const float w = __ldg(a.win + (long)i * N + c);
                re = __fmaf_rn(w, (float)x.x, re);
                im = __fmaf_rn(w, (float)x.y, im);
            }
        }
        return make_float2(re, im);
    };
    auto store = [&](int c, float2 v) {
        sre[fft::pad(c)] = v.x;
        sim[fft::pad(c)] = v.y;
    };
    fft::transform_row<N, C::TPR>(sre, sim, t, a.tw, load, store);
    __syncthreads();

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
