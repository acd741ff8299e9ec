/*
 * MDT_device_functions.h -- drop-in replacement for the reference header of
 * the same name (MDT_OneStation_client/MDT_device_functions.h:31-48).
 *
 * Same includes, same __constant__ d_PI, same three kernel prototypes, so the
 * reference client's GPU stage compiles and links against libmdtfx.so without
 * source changes:
 *   PFB_Window_min4term_BH(Nchannels, Ntaps, Window)                      (:44)
 *   PpS_Batch(Nchannels, Ntaps, Window, InSignal, PolyStruct)              (:45)
 *   ReorderFOutput(NpolsxNelements, Nchannels, FOutput, XInput)            (:46)
 * The kernels are defined in libmdtfx.so; their <<<>>> launches go through
 * the shared CUDA runtime, so the caller and the library must both link
 * cudart as a shared library (nvcc -cudart shared).  The prototypes carry
 * default visibility because nvcc otherwise marks __global__ entities
 * hidden, which keeps a caller's launch from binding to a shared library.
 * The cufftExecC2C / cublasCgemmBatched calls that follow them in the
 * reference sequence resolve to libmdtfx.so as well when the client links it
 * instead of -lcufft -lcublas (see mdt_cufft_cublas_shim.h).
 */
#ifndef MDT_DEVICE_FUNC
#define MDT_DEVICE_FUNC

#include <cuda.h>
#include <cufft.h>
#include <cublas_v2.h>

/*  Constant for device code  */
__device__ __constant__ float d_PI = 3.141592653589793238462643383279502884f;

#define MDT_DROPIN_KERNEL __global__ __attribute__((visibility("default")))

/*  Device kernel prototypes  */
MDT_DROPIN_KERNEL void PFB_Window_min4term_BH(int, int, float *);
MDT_DROPIN_KERNEL void PpS_Batch(int, int, float *, cuComplex *, cufftComplex *);
MDT_DROPIN_KERNEL void ReorderFOutput(int, int, cufftComplex *, cuComplex *);

#endif
