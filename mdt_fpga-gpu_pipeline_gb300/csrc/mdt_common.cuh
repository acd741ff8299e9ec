// mdt_common.cuh -- shared helpers of libmdtfx (status plumbing, complex
// arithmetic with pinned rounding).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "mdt_fx.h"

namespace mdt {

// Records a message for mdt_last_error() on the calling thread.
void set_error(const std::string &msg);
// Turns a CUDA error (if any) into MDT_ERR_CUDA with a message.
mdt_status cuda_status(cudaError_t err, const char *what);
// Peeks at the launch error of the kernel just enqueued.
inline mdt_status launch_status(const char *what) { return cuda_status(cudaGetLastError(), what); }
mdt_status invalid(const std::string &msg);

inline bool is_pow2(long n) { return n > 0 && (n & (n - 1)) == 0; }
inline int ilog2(long n)
{
    int l = 0;
    while ((1L << l) < n) l++;
    return l;
}
inline long cdiv(long a, long b) { return (a + b - 1) / b; }

// Number of SMs of the current device (cached per device).
int sm_count();

// Complex arithmetic with every rounding written out (no contraction), so
// that two kernels sharing these helpers produce bit-identical results.
__device__ __forceinline__ float2 cadd(float2 a, float2 b)
{
    return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
    return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}
// a * b
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)),
                       __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}
// a * (-i)
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

}  // namespace mdt
