// fft.cu -- batched C2C FFT on the shared-memory Stockham core
// (fft_core.cuh) and the cuFFT subset the reference client calls
// (cufftPlan1d / cufftSetStream / cufftExecC2C / cufftDestroy /
// cufftGetVersion, reference MDT_OneStation_client.cu:441-446,622-630,1105).
#include <cufft.h>
#include "mdt_cufft_cublas_shim.h"  // checks the exported signatures

#include <map>
#include <mutex>
#include <vector>

#include "fft_core.cuh"

namespace mdt {

// ------------------------------------------------------------ twiddles
const float2 *fft_twiddles(int n, mdt_status *st)
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, float2 *> tables;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(dev, n);
    auto it = tables.find(key);
    if (it != tables.end()) {
        *st = MDT_SUCCESS;
        return it->second;
    }
    std::vector<float2> h(n);
    for (int k = 0; k < n; k++) {
        double a = -2.0 * 3.141592653589793238462643383279502884 * (double)k / (double)n;
        h[k] = make_float2((float)cos(a), (float)sin(a));
    }
    float2 *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float2) * n);
    if (e != cudaSuccess) {
        *st = cuda_status(e, "twiddle table alloc");
        return nullptr;
    }
    e = cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        *st = cuda_status(e, "twiddle table copy");
        return nullptr;
    }
    tables[key] = d;
    *st = MDT_SUCCESS;
    return d;
}

// ------------------------------------------------------------ kernel
template <int N>
struct RowsCfg {
    static constexpr int TPR = fft::Shape<N>::TPR;
    static constexpr int ROWS = (256 / TPR) < 1 ? 1 : 256 / TPR;
    static constexpr int THREADS = ROWS * TPR;
    static constexpr size_t SMEM = sizeof(float2) * fft::Shape<N>::PADN * ROWS;
};

template <int N>
__global__ void __launch_bounds__(RowsCfg<N>::THREADS)
    fft_rows_kernel(const float2 *in, float2 *out, long rows, const float2 *__restrict__ tw,
                    int inverse)
{
    using C = RowsCfg<N>;
    extern __shared__ float2 smem2[];
    const int lrow = threadIdx.x / C::TPR;
    const int t = threadIdx.x - lrow * C::TPR;
    const long row = (long)blockIdx.x * C::ROWS + lrow;
    const bool valid = row < rows;
    float2 *sx = smem2 + (size_t)lrow * fft::Shape<N>::PADN;
    const float2 *src = in + (valid ? row : 0) * (long)N;
    float2 *dst = out + (valid ? row : 0) * (long)N;
    auto load = [&](int i) -> float2 {
        float2 v = valid ? src[i] : make_float2(0.f, 0.f);
        return inverse ? cconj(v) : v;
    };
    auto store = [&](int i, float2 v) {
        if (valid) dst[i] = inverse ? cconj(v) : v;
    };
    fft::transform_row<N, C::TPR, true, true>(sx, t, tw, load, store);
}

template <int N>
static mdt_status launch_rows(const float2 *in, float2 *out, long rows, int inverse,
                              cudaStream_t stream)
{
    using C = RowsCfg<N>;
    mdt_status st;
    const float2 *tw = fft_twiddles(N, &st);
    if (!tw) return st;
    if (C::SMEM > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fft_rows_kernel<N>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)C::SMEM);
        if (e != cudaSuccess) return cuda_status(e, "fft smem attribute");
    }
    long blocks = cdiv(rows, C::ROWS);
    if (blocks > 0x7fffffffL) return invalid("fft: too many rows");
    fft_rows_kernel<N><<<(unsigned)blocks, C::THREADS, C::SMEM, stream>>>(in, out, rows, tw,
                                                                        inverse);
    return launch_status("fft_rows_kernel");
}

mdt_status fft_c2c(const void *in, void *out, long rows, int n, int direction,
                   cudaStream_t stream)
{
    if (!in || !out || rows < 0) return invalid("fft: bad pointers or rows");
    if (direction != -1 && direction != 1) return invalid("fft: direction must be -1 or +1");
    if (rows == 0) return MDT_SUCCESS;
    const float2 *i2 = (const float2 *)in;
    float2 *o2 = (float2 *)out;
    int inv = direction == 1;
    switch (n) {
        case 2: return launch_rows<2>(i2, o2, rows, inv, stream);
        case 4: return launch_rows<4>(i2, o2, rows, inv, stream);
        case 8: return launch_rows<8>(i2, o2, rows, inv, stream);
        case 16: return launch_rows<16>(i2, o2, rows, inv, stream);
        case 32: return launch_rows<32>(i2, o2, rows, inv, stream);
        case 64: return launch_rows<64>(i2, o2, rows, inv, stream);
        case 128: return launch_rows<128>(i2, o2, rows, inv, stream);
        case 256: return launch_rows<256>(i2, o2, rows, inv, stream);
        case 512: return launch_rows<512>(i2, o2, rows, inv, stream);
        case 1024: return launch_rows<1024>(i2, o2, rows, inv, stream);
        case 2048: return launch_rows<2048>(i2, o2, rows, inv, stream);
        case 4096: return launch_rows<4096>(i2, o2, rows, inv, stream);
        case 8192: return launch_rows<8192>(i2, o2, rows, inv, stream);
        case 16384: return launch_rows<16384>(i2, o2, rows, inv, stream);
        default: break;
    }
    set_error("fft: n must be a power of two in [2, 16384]");
    return MDT_ERR_NOT_SUPPORTED;
}

// ------------------------------------------------------------ cuFFT subset
struct ShimPlan {
    int n = 0;
    long batch = 0;
    cudaStream_t stream = 0;
};
static std::mutex g_plan_mu;
static std::map<int, ShimPlan> g_plans;
static int g_next_plan = 1;

}  // namespace mdt

extern "C" {

MDT_API mdt_status mdt_fft_c2c(const void *in, void *out, long rows, int n, int direction,
                               cudaStream_t stream)
{
    return mdt::fft_c2c(in, out, rows, n, direction, stream);
}

// cufftPlan1d(&plan, Nch, CUFFT_C2C, Nspectra*Npols*Nelements)
// (reference MDT_OneStation_client.cu:622).  Supported: C2C, nx = 2^k in
// [2, 16384], batch >= 1.  The plan allocates nothing per batch; the
// twiddle table for nx is created here, outside any stream capture.
cufftResult CUFFTAPI cufftPlan1d(cufftHandle *plan, int nx, cufftType type, int batch)
{
    if (!plan) return CUFFT_INVALID_VALUE;
    if (type != CUFFT_C2C) return CUFFT_NOT_SUPPORTED;
    if (batch < 1) return CUFFT_INVALID_VALUE;
    if (!mdt::is_pow2(nx) || nx < 2 || nx > 16384) return CUFFT_INVALID_SIZE;
    mdt_status st;
    if (!mdt::fft_twiddles(nx, &st)) return CUFFT_ALLOC_FAILED;
    std::lock_guard<std::mutex> lk(mdt::g_plan_mu);
    int h = mdt::g_next_plan++;
    mdt::ShimPlan p;
    p.n = nx;
    p.batch = batch;
    mdt::g_plans[h] = p;
    *plan = h;
    return CUFFT_SUCCESS;
}

// cufftSetStream (reference :630)
cufftResult CUFFTAPI cufftSetStream(cufftHandle plan, cudaStream_t stream)
{
    std::lock_guard<std::mutex> lk(mdt::g_plan_mu);
    auto it = mdt::g_plans.find(plan);
    if (it == mdt::g_plans.end()) return CUFFT_INVALID_PLAN;
    it->second.stream = stream;
    return CUFFT_SUCCESS;
}

// cufftExecC2C(plan, d_FOutput, d_FOutput, CUFFT_FORWARD) (reference :1105);
// in place or out of place, forward or inverse, unnormalised.
cufftResult CUFFTAPI cufftExecC2C(cufftHandle plan, cufftComplex *idata, cufftComplex *odata,
                                  int direction)
{
    mdt::ShimPlan p;
    {
        std::lock_guard<std::mutex> lk(mdt::g_plan_mu);
        auto it = mdt::g_plans.find(plan);
        if (it == mdt::g_plans.end()) return CUFFT_INVALID_PLAN;
        p = it->second;
    }
    if (!idata || !odata) return CUFFT_INVALID_VALUE;
    if (direction != CUFFT_FORWARD && direction != CUFFT_INVERSE) return CUFFT_INVALID_VALUE;
    mdt_status st = mdt::fft_c2c(idata, odata, p.batch, p.n, direction, p.stream);
    if (st == MDT_SUCCESS) return CUFFT_SUCCESS;
    if (st == MDT_ERR_NOT_SUPPORTED) return CUFFT_NOT_SUPPORTED;
    if (st == MDT_ERR_INVALID_VALUE) return CUFFT_INVALID_VALUE;
    return CUFFT_EXEC_FAILED;
}

cufftResult CUFFTAPI cufftDestroy(cufftHandle plan)
{
    std::lock_guard<std::mutex> lk(mdt::g_plan_mu);
    auto it = mdt::g_plans.find(plan);
    if (it == mdt::g_plans.end()) return CUFFT_INVALID_PLAN;
    mdt::g_plans.erase(it);
    return CUFFT_SUCCESS;
}

// Reports this library's version code (mdt_version), not a cuFFT release:
// the reference only prints it (MDT_OneStation_client.cu:443,446).
cufftResult CUFFTAPI cufftGetVersion(int *version)
{
    if (!version) return CUFFT_INVALID_VALUE;
    *version = mdt_version();
    return CUFFT_SUCCESS;
}

}  // extern "C"
