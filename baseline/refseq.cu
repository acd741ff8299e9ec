// refseq.cu -- the reference's own GPU FX sequence, run as the reference
// client's rank 2 runs it, for comparison with this repository's library.
//
// NOT PART OF THE PRODUCT: libmdtfx.so never links this file, cuFFT or cuBLAS.
// It is the "library bar" and the second parity check: the reference's
// kernels, compiled from the reference source for sm_103a into
// baseline/_ref/mdt_ref_kernels.fatbin by baseline/build_ref_gpu.sh, loaded
// here with the CUDA driver API, and NVIDIA's cuFFT and cuBLAS, called with
// the argument patterns of the reference client:
//   PpS_Batch<<<(ceil(Nch/1024), Nsp, NE), 1024>>>   MDT_OneStation_client.cu:605-611,1083
//   cufftPlan1d(Nch, C2C, Nsp*NE), cufftExecC2C(FORWARD, in place)     :622,630,1105
//   ReorderFOutput<<<(ceil(NE/32), ceil(Nch/32), Nsp), (32,32)>>>
//       (the kernel's documented grid, MDT_device_functions.cu:175-180, with the
//        (32,32) block under which the kernel is correct for any NE)
//   cublasCgemmBatched(N, C, NE, NE, Nsp, 1/Nsp, A[], NE, A[], NE, 0, C[], NE, Nch)
//       with A[c] = XInput + c*NE*Nsp, C[c] = XOutput + c*NE*NE          :656-660,683,1128
//   history: copy the last Ntaps-1 spectra of FInput to its head         :1170
// The reference's input is complex64 (int32 samples x 2^-19, :896-907); this
// harness converts the same int8 I/Q the library reads to complex64 exactly.
//
// cuFFT and cuBLAS are opened with dlopen(RTLD_LOCAL | RTLD_DEEPBIND) and
// their entry points taken with dlsym from those handles: libmdtfx.so exports
// the same names (its drop-in shim), and when it is loaded into the process
// first with global visibility an ordinary link would bind this harness to
// the shim instead of NVIDIA's libraries.  refseq_libraries() reports the
// files the entry points come from and the libraries' versions.
//
// C ABI (ctypes, baseline/refseq.py); every function returns 0 on success
// and a nonzero code with refseq_last_error() text otherwise.
#include <dlfcn.h>

#include <cuda.h>
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cufft.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    return fail(2, std::string(what) + ": " + cudaGetErrorString(e));
}

int drv_fail(CUresult r, const char *what)
{
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    return fail(3, std::string(what) + ": " + (s ? s : "CUDA driver error"));
}

// NVIDIA's cuFFT and cuBLAS entry points, bound from their own libraries.
struct Vendor {
    bool ok = false;
    void *fft = nullptr, *blas = nullptr;
    cufftResult (*plan1d)(cufftHandle *, int, cufftType, int) = nullptr;
    cufftResult (*set_stream)(cufftHandle, cudaStream_t) = nullptr;
    cufftResult (*exec_c2c)(cufftHandle, cufftComplex *, cufftComplex *, int) = nullptr;
    cufftResult (*destroy)(cufftHandle) = nullptr;
    cufftResult (*fft_version)(int *) = nullptr;
    cublasStatus_t (*create)(cublasHandle_t *) = nullptr;
    cublasStatus_t (*blas_set_stream)(cublasHandle_t, cudaStream_t) = nullptr;
    cublasStatus_t (*blas_destroy)(cublasHandle_t) = nullptr;
    cublasStatus_t (*blas_version)(cublasHandle_t, int *) = nullptr;
    cublasStatus_t (*cgemm_batched)(cublasHandle_t, cublasOperation_t, cublasOperation_t, int,
                                    int, int, const cuComplex *, const cuComplex *const[], int,
                                    const cuComplex *const[], int, const cuComplex *,
                                    cuComplex *const[], int, int) = nullptr;
};
Vendor g_vendor;

void *open_first(const char *const *names)
{
    for (int i = 0; names[i]; i++) {
        void *h = dlopen(names[i], RTLD_NOW | RTLD_LOCAL | RTLD_DEEPBIND);
        if (h) return h;
    }
    return nullptr;
}

template <typename F>
bool bind(void *h, const char *name, F &f)
{
    f = reinterpret_cast<F>(dlsym(h, name));
    return f != nullptr;
}

int load_vendor()
{
    Vendor &v = g_vendor;
    if (v.ok) return 0;
    static const char *fft_names[] = {"libcufft.so.12", "libcufft.so", nullptr};
    static const char *blas_names[] = {"libcublas.so.13", "libcublas.so", nullptr};
    v.fft = open_first(fft_names);
    if (!v.fft) return fail(6, std::string("dlopen libcufft: ") + dlerror());
    v.blas = open_first(blas_names);
    if (!v.blas) return fail(6, std::string("dlopen libcublas: ") + dlerror());
    if (!bind(v.fft, "cufftPlan1d", v.plan1d) || !bind(v.fft, "cufftSetStream", v.set_stream) ||
        !bind(v.fft, "cufftExecC2C", v.exec_c2c) || !bind(v.fft, "cufftDestroy", v.destroy) ||
        !bind(v.fft, "cufftGetVersion", v.fft_version) ||
        !bind(v.blas, "cublasCreate_v2", v.create) ||
        !bind(v.blas, "cublasSetStream_v2", v.blas_set_stream) ||
        !bind(v.blas, "cublasDestroy_v2", v.blas_destroy) ||
        !bind(v.blas, "cublasGetVersion_v2", v.blas_version) ||
        !bind(v.blas, "cublasCgemmBatched", v.cgemm_batched))
        return fail(6, "dlsym: a cuFFT or cuBLAS entry point is missing");
    v.ok = true;
    return 0;
}

// Reference kernel symbols (C++ names of MDT_device_functions.h:44-46).
const char *kPpS = "_Z9PpS_BatchiiPfP6float2S1_";
const char *kReorder = "_Z14ReorderFOutputiiP6float2S0_";
const char *kWindowBH = "_Z22PFB_Window_min4term_BHiiPf";

__global__ void iq_to_c64(const char2 *__restrict__ iq, float2 *__restrict__ out, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        char2 v = iq[i];
        out[i] = make_float2((float)v.x, (float)v.y);
    }
}

}  // namespace

struct RefSeq {
    int ne = 0, nch = 0, ntaps = 0, nsp = 0;
    CUmodule mod = nullptr;
    CUfunction pps = nullptr, reorder = nullptr, window_bh = nullptr;
    cudaStream_t stream = nullptr;
    cufftHandle fft = 0;
    bool fft_ok = false;
    cublasHandle_t blas = nullptr;
    float *window = nullptr;
    float2 *finput = nullptr, *foutput = nullptr, *xinput = nullptr, *xoutput = nullptr;
    float2 **xin_ptr = nullptr, **xout_ptr = nullptr;
    int max_threads = 1024;
};

extern "C" {

const char *refseq_last_error() { return g_err.c_str(); }

// The files cuFFT's cufftExecC2C and cuBLAS's cublasCgemmBatched were bound
// from (dladdr), written as "<cufft file>|<cublas file>" into `buf`, and the
// two libraries' version numbers.
int refseq_libraries(char *buf, int len, int *cufft_version, int *cublas_version)
{
    if (int rc = load_vendor()) return rc;
    Dl_info a{}, b{};
    dladdr(reinterpret_cast<void *>(g_vendor.exec_c2c), &a);
    dladdr(reinterpret_cast<void *>(g_vendor.cgemm_batched), &b);
    snprintf(buf, (size_t)len, "%s|%s", a.dli_fname ? a.dli_fname : "?",
             b.dli_fname ? b.dli_fname : "?");
    *cufft_version = 0;
    *cublas_version = 0;
    g_vendor.fft_version(cufft_version);
    cublasHandle_t h = nullptr;
    if (g_vendor.create(&h) == CUBLAS_STATUS_SUCCESS) {
        g_vendor.blas_version(h, cublas_version);
        g_vendor.blas_destroy(h);
    }
    return 0;
}

void refseq_destroy(RefSeq *r)
{
    if (!r) return;
    if (r->stream) cudaStreamSynchronize(r->stream);
    if (r->blas) g_vendor.blas_destroy(r->blas);
    if (r->fft_ok) g_vendor.destroy(r->fft);
    cudaFree(r->window);
    cudaFree(r->finput);
    cudaFree(r->foutput);
    cudaFree(r->xinput);
    cudaFree(r->xoutput);
    cudaFree(r->xin_ptr);
    cudaFree(r->xout_ptr);
    if (r->stream) cudaStreamDestroy(r->stream);
    if (r->mod) cuModuleUnload(r->mod);
    delete r;
}

// Loads the reference kernels from `fatbin` and sets up the buffers, the
// cuFFT plan and the cuBLAS handle of one integration of the given shape on
// the current device.
int refseq_create(const char *fatbin, int ne, int nch, int ntaps, int nsp, RefSeq **out)
{
    *out = nullptr;
    if (ne <= 0 || nch <= 0 || ntaps <= 0 || nsp <= 0) return fail(1, "bad shape");
    if (int rc = load_vendor()) return rc;
    RefSeq *r = new RefSeq;
    r->ne = ne;
    r->nch = nch;
    r->ntaps = ntaps;
    r->nsp = nsp;
    cudaError_t e = cudaFree(nullptr);  // the runtime's primary context becomes current
    if (e != cudaSuccess) { refseq_destroy(r); return cuda_fail(e, "context"); }
    CUresult cr = cuModuleLoad(&r->mod, fatbin);
    if (cr != CUDA_SUCCESS) { refseq_destroy(r); return drv_fail(cr, "load reference kernels"); }
    if ((cr = cuModuleGetFunction(&r->pps, r->mod, kPpS)) != CUDA_SUCCESS ||
        (cr = cuModuleGetFunction(&r->reorder, r->mod, kReorder)) != CUDA_SUCCESS ||
        (cr = cuModuleGetFunction(&r->window_bh, r->mod, kWindowBH)) != CUDA_SUCCESS) {
        refseq_destroy(r);
        return drv_fail(cr, "reference kernel symbol");
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&r->max_threads, cudaDevAttrMaxThreadsPerBlock, dev);
    const size_t nin = (size_t)(nsp + ntaps - 1) * ne * nch, nout = (size_t)nsp * ne * nch;
    if ((e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&r->window, sizeof(float) * (size_t)ntaps * nch)) != cudaSuccess ||
        (e = cudaMalloc(&r->finput, sizeof(float2) * nin)) != cudaSuccess ||
        (e = cudaMalloc(&r->foutput, sizeof(float2) * nout)) != cudaSuccess ||
        (e = cudaMalloc(&r->xinput, sizeof(float2) * nout)) != cudaSuccess ||
        (e = cudaMalloc(&r->xoutput, sizeof(float2) * (size_t)nch * ne * ne)) != cudaSuccess ||
        (e = cudaMalloc(&r->xin_ptr, sizeof(float2 *) * nch)) != cudaSuccess ||
        (e = cudaMalloc(&r->xout_ptr, sizeof(float2 *) * nch)) != cudaSuccess) {
        refseq_destroy(r);
        return cuda_fail(e, "allocation");
    }
    std::vector<float2 *> hin(nch), hout(nch);
    for (int c = 0; c < nch; c++) {
        hin[c] = r->xinput + (size_t)c * ne * nsp;
        hout[c] = r->xoutput + (size_t)c * ne * ne;
    }
    if ((e = cudaMemcpy(r->xin_ptr, hin.data(), sizeof(float2 *) * nch, cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMemcpy(r->xout_ptr, hout.data(), sizeof(float2 *) * nch, cudaMemcpyHostToDevice)) !=
            cudaSuccess) {
        refseq_destroy(r);
        return cuda_fail(e, "pointer arrays");
    }
    cufftResult fr = g_vendor.plan1d(&r->fft, nch, CUFFT_C2C, nsp * ne);
    if (fr != CUFFT_SUCCESS) { refseq_destroy(r); return fail(4, "cufftPlan1d: " + std::to_string(fr)); }
    r->fft_ok = true;
    g_vendor.set_stream(r->fft, r->stream);
    cublasStatus_t bs = g_vendor.create(&r->blas);
    if (bs != CUBLAS_STATUS_SUCCESS) { refseq_destroy(r); return fail(5, "cublasCreate: " + std::to_string(bs)); }
    g_vendor.blas_set_stream(r->blas, r->stream);
    *out = r;
    return 0;
}

// Device pointer of buffer `which`: 0 FInput (complex64, Nsp+Ntaps-1 spectra),
// 1 FOutput (PpS_Batch output, FFT'd in place), 2 XInput (reordered),
// 3 XOutput (visibilities, column-major NE x NE per channel), 4 window.
void *refseq_ptr(RefSeq *r, int which)
{
    switch (which) {
        case 0: return r->finput;
        case 1: return r->foutput;
        case 2: return r->xinput;
        case 3: return r->xoutput;
        case 4: return r->window;
        default: return nullptr;
    }
}

// Copies `bytes` of buffer `which` (see refseq_ptr) into device memory `dst`.
int refseq_read(RefSeq *r, int which, void *dst, size_t bytes)
{
    void *src = refseq_ptr(r, which);
    if (!src || !dst) return fail(1, "bad buffer");
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, r->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "read");
}

// FInput <- complex64(iq) (exact), window <- win; both device pointers.
int refseq_set_input(RefSeq *r, const void *iq, const float *win)
{
    const long n = (long)(r->nsp + r->ntaps - 1) * r->ne * r->nch;
    iq_to_c64<<<1216, 256, 0, r->stream>>>((const char2 *)iq, r->finput, n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "iq_to_c64");
    e = cudaMemcpyAsync(r->window, win, sizeof(float) * (size_t)r->ntaps * r->nch,
                        cudaMemcpyDeviceToDevice, r->stream);
    if (e != cudaSuccess) return cuda_fail(e, "window copy");
    e = cudaStreamSynchronize(r->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "set_input");
}

// One stage on the harness stream: 0 PpS_Batch, 1 cufftExecC2C, 2 ReorderFOutput,
// 3 cublasCgemmBatched, 4 history copy.
int refseq_stage(RefSeq *r, int stage)
{
    int ne = r->ne, nch = r->nch, ntaps = r->ntaps, nsp = r->nsp;
    if (stage == 0) {
        unsigned thr = (unsigned)r->max_threads;
        void *args[] = {&nch, &ntaps, &r->window, &r->finput, &r->foutput};
        CUresult cr = cuLaunchKernel(r->pps, (nch + thr - 1) / thr, nsp, ne, thr, 1, 1, 0,
                                     (CUstream)r->stream, args, nullptr);
        return cr == CUDA_SUCCESS ? 0 : drv_fail(cr, "PpS_Batch launch");
    }
    if (stage == 1) {
        cufftResult fr = g_vendor.exec_c2c(r->fft, (cufftComplex *)r->foutput,
                                      (cufftComplex *)r->foutput, CUFFT_FORWARD);
        return fr == CUFFT_SUCCESS ? 0 : fail(4, "cufftExecC2C: " + std::to_string(fr));
    }
    if (stage == 2) {
        void *args[] = {&ne, &nch, &r->foutput, &r->xinput};
        CUresult cr = cuLaunchKernel(r->reorder, (ne + 31) / 32, (nch + 31) / 32, nsp, 32, 32, 1,
                                     0, (CUstream)r->stream, args, nullptr);
        return cr == CUDA_SUCCESS ? 0 : drv_fail(cr, "ReorderFOutput launch");
    }
    if (stage == 3) {
        cuComplex alpha = make_cuComplex(1.0f / nsp, 0.0f), beta = make_cuComplex(0.0f, 0.0f);
        cublasStatus_t bs = g_vendor.cgemm_batched(
            r->blas, CUBLAS_OP_N, CUBLAS_OP_C, ne, ne, nsp, &alpha,
            (const cuComplex *const *)r->xin_ptr, ne, (const cuComplex *const *)r->xin_ptr, ne,
            &beta, (cuComplex *const *)r->xout_ptr, ne, nch);
        return bs == CUBLAS_STATUS_SUCCESS ? 0 : fail(5, "cublasCgemmBatched: " + std::to_string(bs));
    }
    if (stage == 4) {
        if (ntaps < 2) return 0;
        const size_t stride = (size_t)ne * nch;
        cudaError_t e = cudaMemcpyAsync(r->finput, r->finput + (size_t)nsp * stride,
                                        sizeof(float2) * (size_t)(ntaps - 1) * stride,
                                        cudaMemcpyDeviceToDevice, r->stream);
        return e == cudaSuccess ? 0 : cuda_fail(e, "history copy");
    }
    return fail(1, "bad stage");
}

int refseq_sync(RefSeq *r)
{
    cudaError_t e = cudaStreamSynchronize(r->stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, "sync");
}

// `reps` integrations back to back (PpS, FFT, Reorder, CGEMM; with
// `history`, the history copy too), timed with events on the harness stream:
// stage_ms[0..4] = summed per-stage times / reps, *total_ms = whole time / reps.
int refseq_run(RefSeq *r, int reps, int history, float *stage_ms, float *total_ms)
{
    for (int k = 0; k < 5; k++) stage_ms[k] = 0.f;
    *total_ms = 0.f;
    if (reps <= 0) return fail(1, "reps must be positive");
    const int nst = history ? 5 : 4;
    std::vector<cudaEvent_t> ev((size_t)reps * (nst + 1), nullptr);
    int rc = 0;
    for (auto &e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) { rc = fail(2, "event"); break; }
    for (int it = 0; it < reps && rc == 0; it++) {
        cudaEvent_t *E = ev.data() + (size_t)it * (nst + 1);
        cudaEventRecord(E[0], r->stream);
        for (int s = 0; s < nst && rc == 0; s++) {
            rc = refseq_stage(r, s);
            cudaEventRecord(E[s + 1], r->stream);
        }
    }
    cudaError_t e = cudaStreamSynchronize(r->stream);
    if (rc == 0 && e != cudaSuccess) rc = cuda_fail(e, "run");
    if (rc == 0) {
        for (int it = 0; it < reps; it++) {
            cudaEvent_t *E = ev.data() + (size_t)it * (nst + 1);
            for (int s = 0; s < nst; s++) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, E[s], E[s + 1]);
                stage_ms[s] += ms / reps;
            }
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[0], ev[(size_t)(reps - 1) * (nst + 1) + nst]);
        *total_ms = ms / reps;
    }
    for (auto &x : ev)
        if (x) cudaEventDestroy(x);
    return rc;
}

// The reference's window kernel with its documented grid
// (MDT_device_functions.cu:44-49) into `out` (Ntaps*Nch floats, device).
int refseq_window_bh(RefSeq *r, float *out)
{
    int nch = r->nch, ntaps = r->ntaps;
    unsigned thr = (unsigned)r->max_threads, n = (unsigned)(ntaps * nch);
    void *args[] = {&nch, &ntaps, &out};
    CUresult cr = cuLaunchKernel(r->window_bh, (n + thr - 1) / thr, 1, 1, thr, 1, 1, 0,
                                 (CUstream)r->stream, args, nullptr);
    if (cr != CUDA_SUCCESS) return drv_fail(cr, "PFB_Window_min4term_BH launch");
    return refseq_sync(r);
}

}  // extern "C"
