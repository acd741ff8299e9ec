/*
 * mdt_cuda_emu.h -- just enough of the CUDA execution model to compile the
 * reference's kernel sources with g++ and run them on the CPU, so that the
 * oracle can be pinned against the reference's own code.  Used only by
 * oracle/build_ref.sh (test infrastructure).
 *
 * A block runs as one OpenMP team with one OpenMP thread per CUDA thread:
 *   threadIdx / blockIdx are thread-local, blockDim / gridDim are global,
 *   __shared__ becomes a function-local static (one copy, shared by the team
 *   because blocks run one after another), __syncthreads() is an omp barrier.
 * sinpif / cospif are evaluated in double from their definitions
 * sin(pi x), cos(pi x) and rounded to float (window generator only; the
 * bit-exact kernels do not call them).
 */
#pragma once
#include <math.h>

struct mdt_emu_uint3 { unsigned int x, y, z; };

extern thread_local mdt_emu_uint3 threadIdx;
extern thread_local mdt_emu_uint3 blockIdx;
extern mdt_emu_uint3 blockDim;
extern mdt_emu_uint3 gridDim;

#define __global__
#define __device__
#define __constant__
#define __host__
#define __shared__ static
#define __syncthreads() _Pragma("omp barrier")

static inline float sinpif(float x) { return (float)sin(3.14159265358979323846 * (double)x); }
static inline float cospif(float x) { return (float)cos(3.14159265358979323846 * (double)x); }
