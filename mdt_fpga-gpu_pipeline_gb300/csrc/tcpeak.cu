// tcpeak.cu -- measured dense throughput of tcgen05.mma kind::f16 (f16
// operands, FP32 accumulate, M = 128, K = 16, N = 128 or 256) with both
// operands resident in shared memory: the tensor-core ceiling the X-engine's
// instruction shape can reach on this GPU, measured rather than quoted.
// Also the FP32 FMA rate (packed fma.rn.f32x2 or scalar fma.rn.f32), the
// ceiling of the FP32 SIMT X-engine.
//
// Each CTA fills a 128-row A tile and an N-row B tile (K = 64 f16, the
// 128-byte-swizzled K-major layout the X-engine uses) with pseudo-random
// values in [-1, 1), allocates N TMEM columns, and one thread issues `iters`
// groups of four K = 16 MMAs into the same accumulator, then commits and
// waits (bounded).  Operand values matter: random data draws more power than
// constant data.
#include <cuda_fp16.h>

#include <algorithm>

#include "mdt_common.cuh"
#include "tc_ptx.cuh"

namespace mdt {

constexpr int PK_THREADS = 128;

__global__ void __launch_bounds__(PK_THREADS, 1) tc_peak_kernel(int n, int iters, int *err)
{
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t done;
    __shared__ uint32_t tmem_slot;
    const uint32_t sbase = tc::smem_u32(sm);
    if (sbase & 1023) {
        if (threadIdx.x == 0) atomicExch(err, 2);
        return;
    }
    // A: 128 rows, B: n rows, 128 bytes each (64 f16)
    const int rows = 128 + n;
    __half *h = reinterpret_cast<__half *>(sm);
    for (int i = threadIdx.x; i < rows * 64; i += PK_THREADS) {
        uint32_t x = (uint32_t)i * 2654435761u ^ (blockIdx.x * 40503u + 12345u);
        x ^= x >> 15;
        x *= 2246822519u;
        x ^= x >> 13;
        h[i] = __float2half_rn(((int)(x & 0xffff) - 32768) * (1.0f / 32768.0f));
    }
    if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_u32(&done), 1);
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) {
        tc::tmem_alloc(tc::smem_u32(&tmem_slot), (uint32_t)n);
        tc::tmem_relinquish();
        tc::fence_before_sync();
    }
    tc::fence_proxy_async();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    if (threadIdx.x == 0) {
        const uint64_t ad = tc::sw128_kmajor_desc(sbase);
        const uint64_t bd = tc::sw128_kmajor_desc(sbase + 128 * 128);
        const uint32_t id = tc::idesc_f16(n, 0, 0);
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int k = 0; k < 4; k++) tc::mma_f16(tmem, ad + 2 * k, bd + 2 * k, id, (it | k) != 0);
        }
        tc::mma_commit(tc::smem_u32(&done));
        if (!tc::mbar_wait(tc::smem_u32(&done), 0)) atomicExch(err, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, (uint32_t)n);
    }
}

constexpr int FP_THREADS = 1024;

// Each thread runs 8 independent chains of packed FP32 FMAs (PACKED) or 16
// of scalar ones, `iters` steps each: 32 flops per thread and step either way.
template <bool PACKED>
__global__ void __launch_bounds__(FP_THREADS, 1) fp32_peak_kernel(int iters, float *sink)
{
    const float t = (float)(threadIdx.x + blockIdx.x * FP_THREADS) * 1e-7f;
    float s = 0.0f;
    if constexpr (PACKED) {
        float2 v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = make_float2(t + (float)k, t - (float)k);
        const float2 m = make_float2(0.99999f, 1.00001f), c = make_float2(1e-6f, -1e-6f);
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = __ffma2_rn(v[k], m, c);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) s += v[k].x + v[k].y;
    } else {
        float v[16];
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = t + (float)k;
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] = __fmaf_rn(v[k], 0.99999f, 1e-6f);
        }
#pragma unroll
        for (int k = 0; k < 16; k++) s += v[k];
    }
    if (s == -1.0e30f) *sink = s;  // keeps the chains live; never true for these values
}

}  // namespace mdt

// Times `reps` launches of one 1024-thread CTA per SM running the FMA chains
// above; returns the best launch's time and its TFLOP/s (2 flops per FMA).
extern "C" MDT_API mdt_status mdt_fp32_peak(int packed, int iters, int reps, float *best_ms,
                                            double *tflops, cudaStream_t stream)
{
    if (iters < 1 || reps < 1 || !best_ms || !tflops) return mdt::invalid("fp32_peak: bad arguments");
    float *sink = nullptr;
    cudaError_t e = cudaMalloc(&sink, sizeof(float));
    if (e != cudaSuccess) return mdt::cuda_status(e, "fp32_peak alloc");
    const unsigned grid = (unsigned)mdt::sm_count();
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) {
        cudaFree(sink);
        return mdt::cuda_status(cudaGetLastError(), "fp32_peak event");
    }
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        cudaFree(sink);
        return mdt::cuda_status(cudaGetLastError(), "fp32_peak event");
    }
    float best = 0.0f;
    mdt_status st = MDT_SUCCESS;
    for (int r = 0; r <= reps && st == MDT_SUCCESS; r++) {  // launch 0 warms up
        cudaEventRecord(a, stream);
        if (packed)
            mdt::fp32_peak_kernel<true><<<grid, mdt::FP_THREADS, 0, stream>>>(iters, sink);
        else
            mdt::fp32_peak_kernel<false><<<grid, mdt::FP_THREADS, 0, stream>>>(iters, sink);
        st = mdt::launch_status("fp32_peak_kernel");
        cudaEventRecord(b, stream);
        if (st != MDT_SUCCESS) break;
        e = cudaEventSynchronize(b);
        if (e != cudaSuccess) {
            st = mdt::cuda_status(e, "fp32_peak sync");
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (r > 0 && (best == 0.0f || ms < best)) best = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (st != MDT_SUCCESS) return st;
    *best_ms = best;
    *tflops = 32.0 * iters * (double)mdt::FP_THREADS * grid / (best * 1e-3) / 1e12;
    return MDT_SUCCESS;
}

// Times `reps` launches of ctas_per_sm CTAs per SM, each issuing `iters` x 4
// MMAs of 128 x n x 16; returns the best launch's time and its TFLOP/s
// (2 * 128 * n * 16 flops per MMA).  n is 128 or 256; ctas_per_sm * n <= 512.
extern "C" MDT_API mdt_status mdt_tc_peak_f16(int n, int ctas_per_sm, int iters, int reps,
                                              float *best_ms, double *tflops, int *err,
                                              cudaStream_t stream)
{
    if ((n != 128 && n != 256) || ctas_per_sm < 1 || ctas_per_sm * n > 512 || iters < 1 ||
        reps < 1 || !best_ms || !tflops || !err)
        return mdt::invalid("tc_peak_f16: bad arguments");
    // the operands need (128 + n) x 128 bytes; the request is sized so that
    // exactly ctas_per_sm CTAs fit on an SM (228 KB, 1 KB reserved per CTA)
    const size_t need = (size_t)(128 + n) * 128;
    const size_t smem = std::max(need, (size_t)(200 * 1024) / (size_t)ctas_per_sm);
    cudaError_t e = cudaFuncSetAttribute(mdt::tc_peak_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return mdt::cuda_status(e, "tc_peak_f16 smem attribute");
    const unsigned grid = (unsigned)(mdt::sm_count() * ctas_per_sm);
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return mdt::cuda_status(cudaGetLastError(), "tc_peak_f16 event");
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return mdt::cuda_status(cudaGetLastError(), "tc_peak_f16 event");
    }
    float best = 0.0f;
    mdt_status st = MDT_SUCCESS;
    for (int r = 0; r <= reps && st == MDT_SUCCESS; r++) {  // launch 0 warms up
        cudaEventRecord(a, stream);
        mdt::tc_peak_kernel<<<grid, mdt::PK_THREADS, smem, stream>>>(n, iters, err);
        st = mdt::launch_status("tc_peak_kernel");
        cudaEventRecord(b, stream);
        if (st != MDT_SUCCESS) break;
        e = cudaEventSynchronize(b);
        if (e != cudaSuccess) {
            st = mdt::cuda_status(e, "tc_peak_f16 sync");
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (r > 0 && (best == 0.0f || ms < best)) best = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st != MDT_SUCCESS) return st;
    *best_ms = best;
    *tflops = 2.0 * 128.0 * n * 16.0 * 4.0 * iters * grid / (best * 1e-3) / 1e12;
    return MDT_SUCCESS;
}
