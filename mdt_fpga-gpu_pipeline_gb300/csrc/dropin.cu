// dropin.cu -- the reference's three __global__ kernels with their exact
// signatures (reference MDT_device_functions.h:44-46), so that a caller that
// launches them with <<<grid, block, 0, stream>>> links against this library
// unchanged; plus C-ABI launchers and the library's error plumbing.
//
// Semantics follow the reference kernels (MDT_device_functions.cu), with two
// deliberate differences that only widen what works:
//  * every kernel walks its index space with grid-stride loops, so any grid
//    that covers the reference's implied sizes produces the same result
//    (NE and Nspectra are still taken from gridDim exactly as the reference
//    kernels take them);
//  * ReorderFOutput stages full 32x32 tiles with whatever block shape it is
//    given; the reference loads only blockDim.x channels of each tile
//    (:193,197) and writes 32, which is wrong for its documented NE < 32
//    geometry (:175).
#include <math.h>
#include <mutex>
#include <stdio.h>
#include <unordered_map>

#include "MDT_device_functions.h"
#include "mdt_common.cuh"

namespace mdt {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

mdt_status invalid(const std::string &msg)
{
    set_error(msg);
    return MDT_ERR_INVALID_VALUE;
}

mdt_status cuda_status(cudaError_t err, const char *what)
{
    if (err == cudaSuccess) return MDT_SUCCESS;
    set_error(std::string(what) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) +
              ")");
    return MDT_ERR_CUDA;
}

int sm_count()
{
    static std::mutex mu;
    static std::unordered_map<int, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
        n = 148;
    cache[dev] = n;
    return n;
}

}  // namespace mdt

// ----------------------------------------------------------------- kernels

// nvcc gives __global__ host stubs hidden visibility by default; the drop-in
// kernels are part of the library's interface, so their stubs are exported.
#define MDT_KERNEL_EXPORT __attribute__((visibility("default")))

// Minimum 4-term Blackman-Harris windowed sinc (reference :52-88), with the
// reference's float argument conventions; sinpif/cospif are CUDA's.
__global__ MDT_KERNEL_EXPORT void PFB_Window_min4term_BH(int Nchannels, int Ntaps, float *Window)
{
    const long total = (long)Ntaps * Nchannels;
    const long step = (long)gridDim.x * blockDim.x;
    for (long idx = threadIdx.x + (long)blockIdx.x * blockDim.x; idx < total; idx += step) {
        float arg = (idx - 0.5f * Ntaps * Nchannels) / Nchannels;
        float sinc = (arg == 0.0f) ? 1.0f : sinpif(arg) / (3.14159265358979323846f * arg);
        float x = 2.0f * idx / (Ntaps * Nchannels);
        float bh = 0.35875f - 0.48829f * cospif(x) + 0.14128f * cospif(2.0f * x) -
                   0.01168f * cospif(3.0f * x);
        Window[idx] = sinc * bh;
    }
}

// Polyphase structure (reference :113-161):
//   out[s][e][c] = sum_{i<Ntaps} W[i*Nch + c] * in[s+i][e][c]
// accumulated with fmaf in increasing i from zero (bit-exact with the
// reference).  NE = gridDim.z, spectrum s = blockIdx.y, element e = blockIdx.z.
__global__ MDT_KERNEL_EXPORT void PpS_Batch(int Nchannels, int Ntaps, float *Window, cuComplex *InSignal,
                          cufftComplex *PolyStruct)
{
    const long stride_spec = (long)gridDim.z * Nchannels;
    const long base = (long)blockIdx.y * stride_spec + (long)blockIdx.z * Nchannels;
    const float2 *__restrict__ in = reinterpret_cast<const float2 *>(InSignal) + base;
    const float *__restrict__ w = Window;
    float2 *__restrict__ out = reinterpret_cast<float2 *>(PolyStruct) + base;
    const int step = gridDim.x * blockDim.x;
    for (int c = threadIdx.x + blockIdx.x * blockDim.x; c < Nchannels; c += step) {
        float re = 0.0f, im = 0.0f;
        const float2 *p = in + c;
        const float *wp = w + c;
#pragma unroll 8
        for (int i = 0; i < Ntaps; i++) {
            float2 x = __ldg(p + (long)i * stride_spec);
            float wi = __ldg(wp + (long)i * Nchannels);
            re = __fmaf_rn(wi, x.x, re);
            im = __fmaf_rn(wi, x.y, im);
        }
        out[c] = make_float2(re, im);
    }
}

// Corner turn (reference :183-208):  X[(c*Nsp + s)*NE + e] = F[(s*NE + e)*Nch + c]
// with Nsp = gridDim.z and s = blockIdx.z.  32x32 tiles through shared memory
// (33-column rows), tiles walked grid-stride over (blockIdx.x -> elements,
// blockIdx.y -> channels), every tile fully staged whatever the block shape.
__global__ MDT_KERNEL_EXPORT void ReorderFOutput(int NpolsxNelements, int Nchannels, cufftComplex *FOutput,
                               cuComplex *XInput)
{
    __shared__ float2 tile[32][33];
    const int NE = NpolsxNelements;
    const long s = blockIdx.z;
    const long nsp = gridDim.z;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    const float2 *__restrict__ F = reinterpret_cast<const float2 *>(FOutput) + s * NE * (long)Nchannels;
    float2 *__restrict__ X = reinterpret_cast<float2 *>(XInput);
    for (int e0 = blockIdx.x * 32; e0 < NE; e0 += gridDim.x * 32) {
        for (int c0 = blockIdx.y * 32; c0 < Nchannels; c0 += gridDim.y * 32) {
            for (int k = tid; k < 1024; k += nthr) {
                const int le = k >> 5, lc = k & 31;
                if (e0 + le < NE && c0 + lc < Nchannels)
                    tile[le][lc] = F[(long)(e0 + le) * Nchannels + c0 + lc];
            }
            __syncthreads();
            for (int k = tid; k < 1024; k += nthr) {
                const int lc = k >> 5, le = k & 31;
                if (e0 + le < NE && c0 + lc < Nchannels)
                    X[((long)(c0 + lc) * nsp + s) * NE + e0 + le] = tile[le][lc];
            }
            __syncthreads();
        }
    }
}

// Hamming windowed sinc (no reference counterpart; see mdt_fx.h):
// evaluated in double per coefficient and rounded once to float.
__global__ void mdt_window_hamming_sinc_kernel(int nch, int ntaps, float *w)
{
    const long L = (long)ntaps * nch;
    for (long n = threadIdx.x + (long)blockIdx.x * blockDim.x; n < L;
         n += (long)gridDim.x * blockDim.x) {
        double t = ((double)n - 0.5 * (double)L) / (double)nch;
        double sinc = (t == 0.0) ? 1.0 : sinpi(t) / (3.141592653589793238462643383279502884 * t);
        double hw = 0.54 - 0.46 * cospi(2.0 * (double)n / (double)L);
        w[n] = (float)(sinc * hw);
    }
}

// ------------------------------------------------------------------- C ABI

extern "C" {

MDT_API int mdt_version(void) { return 1000; }

MDT_API const char *mdt_last_error(void) { return mdt::g_last_error.c_str(); }

MDT_API mdt_status mdt_launch_PFB_Window_min4term_BH(unsigned gx, unsigned gy, unsigned gz,
                                                     unsigned bx, unsigned by, unsigned bz,
                                                     cudaStream_t stream, int nchannels,
                                                     int ntaps, float *window)
{
    if (!window || nchannels <= 0 || ntaps <= 0) return mdt::invalid("window: bad arguments");
    PFB_Window_min4term_BH<<<dim3(gx, gy, gz), dim3(bx, by, bz), 0, stream>>>(nchannels, ntaps,
                                                                           window);
    return mdt::launch_status("PFB_Window_min4term_BH");
}

MDT_API mdt_status mdt_launch_PpS_Batch(unsigned gx, unsigned gy, unsigned gz, unsigned bx,
                                        unsigned by, unsigned bz, cudaStream_t stream,
                                        int nchannels, int ntaps, float *window, void *insignal,
                                        void *polystruct)
{
    if (!window || !insignal || !polystruct || nchannels <= 0 || ntaps <= 0)
        return mdt::invalid("PpS_Batch: bad arguments");
    PpS_Batch<<<dim3(gx, gy, gz), dim3(bx, by, bz), 0, stream>>>(
        nchannels, ntaps, window, (cuComplex *)insignal, (cufftComplex *)polystruct);
    return mdt::launch_status("PpS_Batch");
}

MDT_API mdt_status mdt_launch_ReorderFOutput(unsigned gx, unsigned gy, unsigned gz, unsigned bx,
                                             unsigned by, unsigned bz, cudaStream_t stream,
                                             int npolsxnelements, int nchannels, void *foutput,
                                             void *xinput)
{
    if (!foutput || !xinput || npolsxnelements <= 0 || nchannels <= 0)
        return mdt::invalid("ReorderFOutput: bad arguments");
    ReorderFOutput<<<dim3(gx, gy, gz), dim3(bx, by, bz), 0, stream>>>(
        npolsxnelements, nchannels, (cufftComplex *)foutput, (cuComplex *)xinput);
    return mdt::launch_status("ReorderFOutput");
}

MDT_API mdt_status mdt_window_hamming_sinc(int nchannels, int ntaps, float *window,
                                           cudaStream_t stream)
{
    if (!window || nchannels <= 0 || ntaps <= 0) return mdt::invalid("window: bad arguments");
    long L = (long)nchannels * ntaps;
    int blocks = (int)mdt::cdiv(L, 256);
    mdt_window_hamming_sinc_kernel<<<blocks, 256, 0, stream>>>(nchannels, ntaps, window);
    return mdt::launch_status("window_hamming_sinc");
}

}  // extern "C"
