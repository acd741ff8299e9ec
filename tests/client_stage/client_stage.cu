// client_stage.cu -- a stand-in for the reference client's GPU stage (rank 2,
// MDT_OneStation_client.cu:546-713 set-up and :1071-1152 loop body), written
// against the drop-in header only.  It is compiled with nvcc and linked
// against libmdtfx.so alone (no -lcufft, no -lcublas), which is the claim
// under test: the reference's call sequence
//   PpS_Batch<<<>>> -> cufftExecC2C -> ReorderFOutput<<<>>> -> cublasCgemmBatched
// links and runs unchanged on this library.
//
// usage: client_stage NE NCH NTAPS NSP in.bin out.bin
//   in.bin : int8 I/Q [(NSP+NTAPS-1)][NE][NCH][2] then float window [NTAPS*NCH]
//   out.bin: complex64 visibilities [NCH][NE][NE] (cuBLAS column-major)
// Exit codes: 0 ok, 2 usage/IO, 12.. CUDA / library failures.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "MDT_device_functions.h"

static int check_cuda(const char *what, int code)
{
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "%s: CUDA error %d (%s)\n", what, (int)e, cudaGetErrorString(e));
        return code;
    }
    return 0;
}

int main(int argc, char **argv)
{
    if (argc != 7) {
        fprintf(stderr, "usage: %s NE NCH NTAPS NSP in.bin out.bin\n", argv[0]);
        return 2;
    }
    const int NE = atoi(argv[1]), Nch = atoi(argv[2]), Ntaps = atoi(argv[3]), Nsp = atoi(argv[4]);
    const long nin = (long)(Nsp + Ntaps - 1) * NE * Nch;
    std::vector<signed char> iq(2 * nin);
    std::vector<float> win((size_t)Ntaps * Nch);
    FILE *f = fopen(argv[5], "rb");
    if (!f || fread(iq.data(), 1, iq.size(), f) != iq.size() ||
        fread(win.data(), sizeof(float), win.size(), f) != win.size()) {
        fprintf(stderr, "cannot read %s\n", argv[5]);
        return 2;
    }
    fclose(f);
    std::vector<cuComplex> h_in(nin);
    for (long i = 0; i < nin; i++) h_in[i] = make_cuComplex((float)iq[2 * i], (float)iq[2 * i + 1]);

    cudaStream_t cu_Stream;
    cudaStreamCreate(&cu_Stream);
    float *d_Window;
    cuComplex *d_FInput, *d_XInput, *d_XOutput, **d_XInputPtr, **d_XOutputPtr;
    cufftComplex *d_FOutput;
    const long nout = (long)Nsp * NE * Nch;
    cudaMalloc((void **)&d_Window, sizeof(float) * win.size());
    cudaMalloc((void **)&d_FInput, sizeof(cuComplex) * nin);
    cudaMalloc((void **)&d_FOutput, sizeof(cufftComplex) * nout);
    cudaMalloc((void **)&d_XInput, sizeof(cuComplex) * nout);
    cudaMalloc((void **)&d_XOutput, sizeof(cuComplex) * (size_t)NE * NE * Nch);
    cudaMalloc((void **)&d_XInputPtr, sizeof(cuComplex *) * Nch);
    cudaMalloc((void **)&d_XOutputPtr, sizeof(cuComplex *) * Nch);
    if (int rc = check_cuda("allocation", 12)) return rc;
    cudaMemcpy(d_Window, win.data(), sizeof(float) * win.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(d_FInput, h_in.data(), sizeof(cuComplex) * nin, cudaMemcpyHostToDevice);

    // grids as the reference client computes them (:605-611, documented Reorder grid)
    const int thr = 1024;
    dim3 pps_grid(Nch / thr + (Nch % thr != 0), Nsp, NE), pps_block(thr, 1, 1);
    dim3 re_grid(NE / 32 + (NE % 32 != 0), Nch / 32 + (Nch % 32 != 0), Nsp), re_block(32, 32, 1);

    cufftHandle plan;
    if (cufftPlan1d(&plan, Nch, CUFFT_C2C, Nsp * NE) != CUFFT_SUCCESS) return 13;
    cufftSetStream(plan, cu_Stream);

    std::vector<cuComplex *> hin(Nch), hout(Nch);
    for (int i = 0; i < Nch; i++) {
        hin[i] = d_XInput + (long)i * NE * Nsp;
        hout[i] = d_XOutput + (long)i * NE * NE;
    }
    cudaMemcpy(d_XInputPtr, hin.data(), sizeof(cuComplex *) * Nch, cudaMemcpyHostToDevice);
    cudaMemcpy(d_XOutputPtr, hout.data(), sizeof(cuComplex *) * Nch, cudaMemcpyHostToDevice);
    cuComplex alpha = make_cuComplex(1.0f / Nsp, 0.0f), beta = make_cuComplex(0.0f, 0.0f);
    cublasHandle_t blas;
    if (cublasCreate(&blas) != CUBLAS_STATUS_SUCCESS) return 16;
    if (cublasSetStream(blas, cu_Stream) != CUBLAS_STATUS_SUCCESS) return 17;

    PpS_Batch<<<pps_grid, pps_block, 0, cu_Stream>>>(Nch, Ntaps, d_Window, d_FInput, d_FOutput);
    cudaStreamSynchronize(cu_Stream);
    if (int rc = check_cuda("PpS_Batch", 22)) return rc;
    if (cufftExecC2C(plan, d_FOutput, d_FOutput, CUFFT_FORWARD) != CUFFT_SUCCESS) return 18;
    ReorderFOutput<<<re_grid, re_block, 0, cu_Stream>>>(NE, Nch, d_FOutput, d_XInput);
    if (cublasCgemmBatched(blas, CUBLAS_OP_N, CUBLAS_OP_C, NE, NE, Nsp, &alpha,
                           (const cuComplex **)d_XInputPtr, NE, (const cuComplex **)d_XInputPtr,
                           NE, &beta, d_XOutputPtr, NE, Nch) != CUBLAS_STATUS_SUCCESS)
        return 23;
    cudaStreamSynchronize(cu_Stream);
    if (int rc = check_cuda("X-engine", 24)) return rc;

    std::vector<cuComplex> vis((size_t)NE * NE * Nch);
    cudaMemcpy(vis.data(), d_XOutput, sizeof(cuComplex) * vis.size(), cudaMemcpyDeviceToHost);
    if (int rc = check_cuda("copy back", 26)) return rc;
    f = fopen(argv[6], "wb");
    if (!f || fwrite(vis.data(), sizeof(cuComplex), vis.size(), f) != vis.size()) return 2;
    fclose(f);
    cufftDestroy(plan);
    cublasDestroy(blas);
    printf("client_stage ok: NE=%d Nch=%d Ntaps=%d Nsp=%d\n", NE, Nch, Ntaps, Nsp);
    return 0;
}
