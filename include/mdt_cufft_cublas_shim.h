/*
 * mdt_cufft_cublas_shim.h -- the cuFFT and cuBLAS entry points that
 * libmdtfx.so exports in place of NVIDIA's libraries, with the toolkit's own
 * signatures and status codes (types come from <cufft.h> / <cublas_v2.h>).
 * A client that links libmdtfx.so instead of -lcufft -lcublas runs the
 * reference's F- and X-engine library calls on this library's kernels; no
 * cuFFT or cuBLAS code is involved.
 *
 * Supported subset (anything else returns CUFFT_NOT_SUPPORTED /
 * CUFFT_INVALID_SIZE / CUBLAS_STATUS_NOT_SUPPORTED):
 *   cuFFT: 1-D C2C plans of size 2^k, 2 <= n <= 16384, any batch, forward or
 *          inverse, in place or out of place, on the plan's stream.
 *   cuBLAS: host pointer mode; cublasCgemmBatched for any transa/transb.
 *          OP_N x OP_C with Aarray == Barray and lda == ldb (the X-engine)
 *          runs the Hermitian lower-triangle kernel and mirrors the upper
 *          triangle; other patterns run a general batched CGEMM.
 */
#ifndef MDT_CUFFT_CUBLAS_SHIM_H
#define MDT_CUFFT_CUBLAS_SHIM_H

#include <cufft.h>
#include <cublas_v2.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDT_SHIM_API

/* cufftPlan1d(&plan, Nchannels, CUFFT_C2C, Nspectra*Npols*Nelements)
 * replaces reference MDT_OneStation_client.cu:622 */
MDT_SHIM_API cufftResult cufftPlan1d(cufftHandle *plan, int nx, cufftType type, int batch);
/* replaces reference MDT_OneStation_client.cu:630 */
MDT_SHIM_API cufftResult cufftSetStream(cufftHandle plan, cudaStream_t stream);
/* cufftExecC2C(plan, d_FOutput, d_FOutput, CUFFT_FORWARD)
 * replaces reference MDT_OneStation_client.cu:1105 */
MDT_SHIM_API cufftResult cufftExecC2C(cufftHandle plan, cufftComplex *idata, cufftComplex *odata,
                                      int direction);
MDT_SHIM_API cufftResult cufftDestroy(cufftHandle plan);
/* reports mdt_version(); replaces reference MDT_OneStation_client.cu:443 */
MDT_SHIM_API cufftResult cufftGetVersion(int *version);

/* cublasCreate (macro for cublasCreate_v2 in <cublas_v2.h>)
 * replaces reference MDT_OneStation_client.cu:690 */
MDT_SHIM_API cublasStatus_t cublasCreate_v2(cublasHandle_t *handle);
MDT_SHIM_API cublasStatus_t cublasDestroy_v2(cublasHandle_t handle);
/* replaces reference MDT_OneStation_client.cu:699 */
MDT_SHIM_API cublasStatus_t cublasSetStream_v2(cublasHandle_t handle, cudaStream_t streamId);
MDT_SHIM_API cublasStatus_t cublasGetStream_v2(cublasHandle_t handle, cudaStream_t *streamId);
/* cublasCgemmBatched(h, OP_N, OP_C, NE, NE, Nspectra, &alpha, XinPtr, NE, XinPtr, NE,
 *                    &beta, XoutPtr, NE, Nchannels)
 * replaces reference MDT_OneStation_client.cu:1128 */
MDT_SHIM_API cublasStatus_t cublasCgemmBatched(cublasHandle_t handle, cublasOperation_t transa,
                                               cublasOperation_t transb, int m, int n, int k,
                                               const cuComplex *alpha,
                                               const cuComplex *const Aarray[], int lda,
                                               const cuComplex *const Barray[], int ldb,
                                               const cuComplex *beta, cuComplex *const Carray[],
                                               int ldc, int batchCount);

#ifdef __cplusplus
}
#endif
#endif /* MDT_CUFFT_CUBLAS_SHIM_H */
