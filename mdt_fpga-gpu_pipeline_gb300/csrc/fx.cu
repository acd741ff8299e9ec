// fx.cu -- the plan API (mdt_fx_*): fused F-engine + X-engine over one or
// many integrations, with the PFB history of Ntaps-1 spectra carried between
// streamed integrations.  This is the reference's rank-2 loop
// (MDT_OneStation_client.cu:1071-1152: PpS_Batch -> cufftExecC2C ->
// ReorderFOutput -> cublasCgemmBatched, then the rank-3 history shift at
// :1170) as two kernels per integration on one stream.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <new>
#include <string>
#include <vector>

#include "fengine.cuh"
#include "mdt_common.cuh"

namespace mdt {
mdt_status check_dims(int ne, int nch, int ntaps, int nsp);
mdt_status fengine_f32(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                       const int8_t *iq, const float *win, float2 *X, cudaStream_t stream);
mdt_status xengine_herm_f32(int ne, long nbatch, int nsp, const float2 *X,
                            const float2 *const *Xptrs, long ld, long xstride, float2 *V,
                            float2 *const *Vptrs, long ldv, long vstride, float2 alpha,
                            float2 beta, bool beta_zero, cudaStream_t stream, int blocked);
mdt_status fengine_c64b(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                        const int8_t *iq, const float *win, float2 *XB, cudaStream_t stream);
const float2 *fft_twiddles(int n, mdt_status *st);
mdt_status fengine_x16(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                       const int8_t *iq, const float *win, void *X16, int nep, int nkc,
                       int ab_fmt, float scale, cudaStream_t stream);
mdt_status xengine_tc(int ne, int nch, int nsp, const void *X16, int ab_fmt, float scale,
                      float2 *V, double2 *Vacc, int *err, cudaStream_t stream);
int x16_padded_rows(int ne);
int x16_chunks(int nsp);
mdt_status fengine_q8(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                      const int8_t *iq, const float *win, void *X16, int nep, int nkc,
                      const float *qscales, cudaStream_t stream);
mdt_status xengine_q8(int ne, int nch, int nsp, const void *X16, const float *qscales, float2 *V,
                      double2 *Vacc, int2 *raw, int *err, cudaStream_t stream);
mdt_status channel_scales(const float2 *XB, int ne, int nch, int nsp, float target_rms, float *pw,
                          float *scales, cudaStream_t stream);
mdt_status fengine_tc(int ne, int nch, int ntaps, int nsp, const int8_t *hist, int nhist,
                      const int8_t *iq, const float *win, void *X16, int nep, int nkc, int ab_fmt,
                      float scale, int *err, cudaStream_t stream, const float *qscales);

// Vacc[i] += V[i] (complex64 -> complex128), the cross-integration sum of the
// FP32 path.
__global__ void accumulate_f64_kernel(const float2 *__restrict__ V, double2 *__restrict__ acc,
                                      long n)
{
    for (long i = threadIdx.x + (long)blockIdx.x * blockDim.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        float2 v = V[i];
        double2 a = acc[i];
        acc[i] = make_double2(a.x + (double)v.x, a.y + (double)v.y);
    }
}
}  // namespace mdt

struct mdt_fx_plan_s {
    mdt_fx_desc d;
    cudaStream_t stream = 0;
    float *window = nullptr;
    bool window_set = false;
    float2 *X = nullptr;       // F-engine output, one integration (FP32 path)
    void *X16 = nullptr;       // F-engine output in the tensor-core operand layout
    int nep = 0, nkc = 0;      // X16 padded rows and K-chunks
    float scale = 1.0f;        // power-of-two F-output scale of the f16/bf16 path
    int *err = nullptr;        // device flag set by a timed-out wait
    double2 *acc = nullptr;    // optional FP64 cross-integration accumulator
    bool tc_fengine = true;    // f16/bf16 path: tensor-core F-engine where it applies
    // exact int8 path: per-channel requantisation scales, calibrated from the
    // first integration's first spectra unless set by the caller
    float *qscales = nullptr, *qpower = nullptr;
    float2 *calib = nullptr;   // FP32 F-output of the calibration spectra
    bool qscales_valid = false;
    int8_t *hist[2] = {nullptr, nullptr};  // PFB history (double-buffered)
    int cur = 0;
    bool streaming = false;
    size_t bytes = 0;
    // host pipeline (mdt_fx_execute_host), allocated on first use
    cudaStream_t copy_stream = nullptr;  // host -> device input copies
    cudaStream_t out_stream = nullptr;   // device -> host visibility copies
    int8_t *stage_in[2] = {nullptr, nullptr};
    float2 *stage_vis[2] = {nullptr, nullptr};
    cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr},
                ev_out[2] = {nullptr, nullptr};
    // stage timing (mdt_fx_set_timing): events around each kernel, per integration
    bool timing = false;
    std::vector<cudaEvent_t> tev;  // triples: before F, between F and X, after X
    size_t tused = 0;
};

namespace {

size_t spectrum_bytes(const mdt_fx_desc &d) { return (size_t)d.nelements * d.nchannels * 2; }

void release(mdt_fx_plan p)
{
    if (!p) return;
    cudaFree(p->window);
    cudaFree(p->X);
    cudaFree(p->X16);
    cudaFree(p->err);
    cudaFree(p->qscales);
    cudaFree(p->qpower);
    cudaFree(p->calib);
    cudaFree(p->hist[0]);
    cudaFree(p->hist[1]);
    for (int i = 0; i < 2; i++) {
        cudaFree(p->stage_in[i]);
        cudaFree(p->stage_vis[i]);
        if (p->ev_in[i]) cudaEventDestroy(p->ev_in[i]);
        if (p->ev_done[i]) cudaEventDestroy(p->ev_done[i]);
        if (p->ev_out[i]) cudaEventDestroy(p->ev_out[i]);
    }
    if (p->copy_stream) cudaStreamDestroy(p->copy_stream);
    if (p->out_stream) cudaStreamDestroy(p->out_stream);
    for (cudaEvent_t e : p->tev) cudaEventDestroy(e);
    delete p;
}

// Next timing event (grown on demand, outside any capture).
cudaEvent_t timing_event(mdt_fx_plan p)
{
    if (p->tused == p->tev.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        p->tev.push_back(e);
    }
    return p->tev[p->tused++];
}

mdt_status one_integration(mdt_fx_plan p, const int8_t *hist, int nhist, const int8_t *iq,
                           void *vis)
{
    const mdt_fx_desc &d = p->d;
    cudaEvent_t t0 = nullptr, t1 = nullptr, t2 = nullptr;
    if (p->timing) {
        t0 = timing_event(p);
        t1 = timing_event(p);
        t2 = timing_event(p);
        if (!t0 || !t1 || !t2) return MDT_ERR_ALLOC;
        cudaEventRecord(t0, p->stream);
    }
    mdt_status st;
    if (d.precision == MDT_PREC_FP32) {
        // F-output in the 8-spectrum blocked layout XB (fengine.cuh)
        const long nsb = (d.nspectra + 7) / 8;
        if (d.nchannels <= 2048)
            st = mdt::fengine_c64b(d.nelements, d.nchannels, d.ntaps, d.nspectra, hist, nhist, iq,
                                   p->window, p->X, p->stream);
        else
            st = MDT_ERR_NOT_SUPPORTED;
        if (st == MDT_ERR_NOT_SUPPORTED) {
            // Nch > 2048: the element-row F-engine in the ReorderFOutput layout
            st = mdt::fengine_f32(d.nelements, d.nchannels, d.ntaps, d.nspectra, hist, nhist,
                                  iq, p->window, p->X, p->stream);
            if (st != MDT_SUCCESS) return st;
            if (t1) cudaEventRecord(t1, p->stream);
            st = mdt::xengine_herm_f32(d.nelements, d.nchannels, d.nspectra, p->X, nullptr,
                                       d.nelements, (long)d.nspectra * d.nelements,
                                       (float2 *)vis, nullptr, d.nelements,
                                       (long)d.nelements * d.nelements,
                                       make_float2(1.0f / d.nspectra, 0.f), make_float2(0.f, 0.f),
                                       true, p->stream, 0);
        } else {
            if (st != MDT_SUCCESS) return st;
            if (t1) cudaEventRecord(t1, p->stream);
            st = mdt::xengine_herm_f32(d.nelements, d.nchannels, d.nspectra, p->X, nullptr,
                                       mdt::xb_block_stride(d.nelements, d.nchannels, nsb),
                                       mdt::xb_chan_stride(d.nelements, d.nchannels, nsb),
                                       (float2 *)vis, nullptr,
                                       d.nelements, (long)d.nelements * d.nelements,
                                       make_float2(1.0f / d.nspectra, 0.f), make_float2(0.f, 0.f),
                                       true, p->stream, 1);
        }
        if (st == MDT_SUCCESS && p->acc) {
            long n = (long)d.nchannels * d.nelements * d.nelements;
            mdt::accumulate_f64_kernel<<<(unsigned)std::min<long>(mdt::cdiv(n, 256),
                                                                  (long)mdt::sm_count() * 16),
                                         256, 0, p->stream>>>((const float2 *)vis, p->acc, n);
            st = mdt::launch_status("accumulate_f64_kernel");
        }
    } else if (d.precision == MDT_PREC_INT8) {
        if (!p->qscales_valid) {
            // calibration: FP32 F-engine over the first spectra of this
            // integration, scale[c] = 20 / rms_c (int8 clips at 6.3 sigma)
            const int ncal = std::min(d.nspectra, 64);
            st = mdt::fengine_c64b(d.nelements, d.nchannels, d.ntaps, ncal, hist, nhist, iq,
                                   p->window, p->calib, p->stream);
            if (st == MDT_SUCCESS)
                st = mdt::channel_scales(p->calib, d.nelements, d.nchannels, ncal, 20.0f,
                                         p->qpower, p->qscales, p->stream);
            if (st != MDT_SUCCESS) return st;
            p->qscales_valid = true;
        }
        if (p->tc_fengine && d.nchannels == 1024 && (d.ntaps == 4 || d.ntaps == 8))
            st = mdt::fengine_tc(d.nelements, d.nchannels, d.ntaps, d.nspectra, hist, nhist, iq,
                                 p->window, p->X16, p->nep, p->nkc, 0, 1.0f, p->err, p->stream,
                                 p->qscales);
        else
            st = mdt::fengine_q8(d.nelements, d.nchannels, d.ntaps, d.nspectra, hist, nhist, iq,
                                 p->window, p->X16, p->nep, p->nkc, p->qscales, p->stream);
        if (st != MDT_SUCCESS) return st;
        if (t1) cudaEventRecord(t1, p->stream);
        st = mdt::xengine_q8(d.nelements, d.nchannels, d.nspectra, p->X16, p->qscales,
                             (float2 *)vis, p->acc, nullptr, p->err, p->stream);
    } else {
        const int fmt = (d.precision == MDT_PREC_BF16) ? 1 : 0;
        if (p->tc_fengine && d.nchannels == 1024 && (d.ntaps == 4 || d.ntaps == 8))
            st = mdt::fengine_tc(d.nelements, d.nchannels, d.ntaps, d.nspectra, hist, nhist, iq,
                                 p->window, p->X16, p->nep, p->nkc, fmt, p->scale, p->err,
                                 p->stream, nullptr);
        else
            st = mdt::fengine_x16(d.nelements, d.nchannels, d.ntaps, d.nspectra, hist, nhist, iq,
                                  p->window, p->X16, p->nep, p->nkc, fmt, p->scale, p->stream);
        if (st != MDT_SUCCESS) return st;
        if (t1) cudaEventRecord(t1, p->stream);
        st = mdt::xengine_tc(d.nelements, d.nchannels, d.nspectra, p->X16, fmt, p->scale,
                             (float2 *)vis, p->acc, p->err, p->stream);
    }
    if (st == MDT_SUCCESS && t2) cudaEventRecord(t2, p->stream);
    return st;
}

}  // namespace

extern "C" {

MDT_API mdt_status mdt_fx_create(const mdt_fx_desc *desc, mdt_fx_plan *plan)
{
    if (!desc || !plan) return mdt::invalid("fx_create: null argument");
    *plan = nullptr;
    mdt_status st = mdt::check_dims(desc->nelements, desc->nchannels, desc->ntaps,
                                    desc->nspectra);
    if (st != MDT_SUCCESS) return st;
    if (desc->precision != MDT_PREC_FP32 && desc->precision != MDT_PREC_FP16 &&
        desc->precision != MDT_PREC_BF16 && desc->precision != MDT_PREC_INT8) {
        mdt::set_error("fx_create: precision not supported by this library");
        return MDT_ERR_NOT_SUPPORTED;
    }
    if (desc->precision != MDT_PREC_FP32 && desc->nchannels > 2048) {
        mdt::set_error("fx_create: the f16/bf16 path supports Nch <= 2048");
        return MDT_ERR_NOT_SUPPORTED;
    }
    mdt_fx_plan p = new (std::nothrow) mdt_fx_plan_s;
    if (!p) return MDT_ERR_ALLOC;
    p->d = *desc;
    {
        // MDT_FENGINE=simt keeps the f16/bf16 path on the SIMT FFT F-engine
        const char *fe = std::getenv("MDT_FENGINE");
        p->tc_fengine = !(fe && std::string(fe) == "simt");
    }
    const mdt_fx_desc &d = p->d;
    size_t wbytes = sizeof(float) * (size_t)d.ntaps * d.nchannels;
    size_t xbytes = 0;
    size_t hbytes = spectrum_bytes(d) * (size_t)(d.ntaps - 1);
    cudaError_t e = cudaMalloc(&p->window, wbytes);
    if (d.precision == MDT_PREC_FP32) {
        // room for either layout: blocked pads Nsp up to a multiple of 8
        xbytes = sizeof(float2) * (size_t)((d.nspectra + 7) / 8 * 8) * d.nelements * d.nchannels;
        if (e == cudaSuccess) e = cudaMalloc(&p->X, xbytes);
    } else {
        p->nep = mdt::x16_padded_rows(d.nelements);
        p->nkc = mdt::x16_chunks(d.nspectra);
        xbytes = (size_t)d.nchannels * p->nkc * p->nep * 128;
        if (e == cudaSuccess) e = cudaMalloc(&p->X16, xbytes);
        // padding rows (elements NE..NEp-1) are never written: zero them once
        if (e == cudaSuccess) e = cudaMemset(p->X16, 0, xbytes);
        if (d.precision == MDT_PREC_INT8) {
            const size_t cal = sizeof(float2) * (size_t)d.nchannels * 64 * d.nelements;
            if (e == cudaSuccess) e = cudaMalloc(&p->qscales, sizeof(float) * d.nchannels);
            if (e == cudaSuccess) e = cudaMalloc(&p->qpower, sizeof(float) * d.nchannels);
            if (e == cudaSuccess) e = cudaMalloc(&p->calib, cal);
            xbytes += cal + 2 * sizeof(float) * d.nchannels;
        }
    }
    if (e == cudaSuccess) e = cudaMalloc(&p->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&p->hist[0], hbytes);
    if (e == cudaSuccess) e = cudaMalloc(&p->hist[1], hbytes);
    if (e != cudaSuccess) {
        release(p);
        mdt::cuda_status(e, "fx_create: workspace");
        return MDT_ERR_ALLOC;
    }
    p->bytes = wbytes + xbytes + 2 * hbytes;
    if (!mdt::fft_twiddles(d.nchannels, &st)) {
        release(p);
        return st;
    }
    *plan = p;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_destroy(mdt_fx_plan plan)
{
    if (!plan) return mdt::invalid("fx_destroy: null plan");
    release(plan);
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_set_stream(mdt_fx_plan plan, cudaStream_t stream)
{
    if (!plan) return mdt::invalid("fx_set_stream: null plan");
    plan->stream = stream;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_set_window(mdt_fx_plan plan, const float *window)
{
    if (!plan || !window) return mdt::invalid("fx_set_window: null argument");
    size_t n = (size_t)plan->d.ntaps * plan->d.nchannels;
    mdt_status st = mdt::cuda_status(cudaMemcpyAsync(plan->window, window, sizeof(float) * n,
                                                     cudaMemcpyDeviceToDevice, plan->stream),
                                     "fx_set_window");
    if (st != MDT_SUCCESS) return st;
    if (plan->d.precision == MDT_PREC_FP16 || plan->d.precision == MDT_PREC_BF16) {
        // F-output bound for int8 samples: |X| <= 127 sqrt(2) sum |W|; the
        // f16 scale is the power of two that keeps that bound under 60000.
        std::vector<float> h(n);
        st = mdt::cuda_status(cudaMemcpy(h.data(), plan->window, sizeof(float) * n,
                                         cudaMemcpyDeviceToHost),
                              "fx_set_window: window bound");
        if (st != MDT_SUCCESS) return st;
        double sum = 0;
        for (float w : h) sum += fabs((double)w);
        double bound = 127.0 * 1.4142135623730951 * sum;
        int ex = 0;
        while (bound * std::ldexp(1.0, -ex) > 60000.0 && ex < 60) ex++;
        plan->scale = (float)std::ldexp(1.0, -ex);
    }
    plan->window_set = true;
    return st;
}

MDT_API mdt_status mdt_fx_set_accumulator(mdt_fx_plan plan, void *acc)
{
    if (!plan) return mdt::invalid("fx_set_accumulator: null plan");
    if (((uintptr_t)acc & 15) != 0) return mdt::invalid("fx_set_accumulator: misaligned buffer");
    plan->acc = (double2 *)acc;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_set_channel_scales(mdt_fx_plan plan, const float *scales)
{
    if (!plan) return mdt::invalid("fx_set_channel_scales: null plan");
    if (plan->d.precision != MDT_PREC_INT8) {
        mdt::set_error("fx_set_channel_scales: plan precision is not INT8");
        return MDT_ERR_STATE;
    }
    if (!scales) {  // recalibrate at the next integration
        plan->qscales_valid = false;
        return MDT_SUCCESS;
    }
    mdt_status st = mdt::cuda_status(
        cudaMemcpyAsync(plan->qscales, scales, sizeof(float) * plan->d.nchannels,
                        cudaMemcpyDeviceToDevice, plan->stream),
        "fx_set_channel_scales");
    if (st == MDT_SUCCESS) plan->qscales_valid = true;
    return st;
}

MDT_API mdt_status mdt_fx_get_channel_scales(mdt_fx_plan plan, float *scales)
{
    if (!plan || !scales) return mdt::invalid("fx_get_channel_scales: null argument");
    if (plan->d.precision != MDT_PREC_INT8 || !plan->qscales_valid) {
        mdt::set_error("fx_get_channel_scales: no INT8 scales yet");
        return MDT_ERR_STATE;
    }
    return mdt::cuda_status(cudaMemcpyAsync(scales, plan->qscales,
                                            sizeof(float) * plan->d.nchannels,
                                            cudaMemcpyDeviceToDevice, plan->stream),
                            "fx_get_channel_scales");
}

MDT_API mdt_status mdt_fx_get_scale(mdt_fx_plan plan, float *scale)
{
    if (!plan || !scale) return mdt::invalid("fx_get_scale: null argument");
    *scale = plan->scale;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_check(mdt_fx_plan plan)
{
    if (!plan) return mdt::invalid("fx_check: null plan");
    mdt_status st = mdt::cuda_status(cudaStreamSynchronize(plan->stream), "fx_check");
    if (st != MDT_SUCCESS) return st;
    int flag = 0;
    st = mdt::cuda_status(cudaMemcpy(&flag, plan->err, sizeof(int), cudaMemcpyDeviceToHost),
                          "fx_check");
    if (st != MDT_SUCCESS) return st;
    if (flag) {
        cudaMemset(plan->err, 0, sizeof(int));
        mdt::set_error("fx_check: a device-side wait timed out");
        return MDT_ERR_TIMEOUT;
    }
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_workspace_bytes(mdt_fx_plan plan, size_t *bytes)
{
    if (!plan || !bytes) return mdt::invalid("fx_workspace_bytes: null argument");
    *bytes = plan->bytes;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_execute(mdt_fx_plan plan, const int8_t *iq, int nint, void *vis)
{
    if (!plan || !iq || !vis || nint < 0) return mdt::invalid("fx_execute: bad arguments");
    if (!plan->window_set) {
        mdt::set_error("fx_execute: no window set");
        return MDT_ERR_STATE;
    }
    const mdt_fx_desc &d = plan->d;
    const size_t sb = spectrum_bytes(d);
    const size_t vb = sizeof(float2) * (size_t)d.nchannels * d.nelements * d.nelements;
    for (int j = 0; j < nint; j++) {
        mdt_status st = one_integration(plan, nullptr, 0, iq + (size_t)j * d.nspectra * sb,
                                        (char *)vis + (size_t)j * vb);
        if (st != MDT_SUCCESS) return st;
    }
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_stream_reset(mdt_fx_plan plan)
{
    if (!plan) return mdt::invalid("fx_stream_reset: null plan");
    plan->streaming = false;
    plan->cur = 0;
    return MDT_SUCCESS;
}

static mdt_status stream_push(mdt_fx_plan plan, const int8_t *iq, void *vis)
{
    const mdt_fx_desc &d = plan->d;
    const size_t sb = spectrum_bytes(d);
    const int nh = d.ntaps - 1;
    mdt_status st;
    int8_t *next = plan->hist[plan->cur ^ 1];
    if (!plan->streaming) {
        // first block: Nsp + Ntaps - 1 spectra, lead-in included
        st = one_integration(plan, nullptr, 0, iq, vis);
        if (st != MDT_SUCCESS) return st;
        st = mdt::cuda_status(cudaMemcpyAsync(next, iq + (size_t)d.nspectra * sb, sb * nh,
                                              cudaMemcpyDeviceToDevice, plan->stream),
                              "fx_stream_push: history");
    } else {
        const int8_t *h = plan->hist[plan->cur];
        st = one_integration(plan, h, nh, iq, vis);
        if (st != MDT_SUCCESS) return st;
        // new history = last nh spectra of [h (nh) | iq (Nsp)]
        const int from_h = nh > d.nspectra ? nh - d.nspectra : 0;
        if (from_h > 0)
            st = mdt::cuda_status(cudaMemcpyAsync(next, h + (size_t)(nh - from_h) * sb,
                                                  sb * from_h, cudaMemcpyDeviceToDevice,
                                                  plan->stream),
                                  "fx_stream_push: history");
        if (st == MDT_SUCCESS)
            st = mdt::cuda_status(
                cudaMemcpyAsync(next + (size_t)from_h * sb,
                                iq + (size_t)(d.nspectra - (nh - from_h)) * sb,
                                sb * (nh - from_h), cudaMemcpyDeviceToDevice, plan->stream),
                "fx_stream_push: history");
    }
    if (st != MDT_SUCCESS) return st;
    plan->cur ^= 1;
    plan->streaming = true;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_stream_push(mdt_fx_plan plan, const int8_t *iq, void *vis)
{
    if (!plan || !iq || !vis) return mdt::invalid("fx_stream_push: bad arguments");
    if (!plan->window_set) {
        mdt::set_error("fx_stream_push: no window set");
        return MDT_ERR_STATE;
    }
    return stream_push(plan, iq, vis);
}

// Creates what the host pipeline still lacks (a failed call leaves what it
// made, and the next call completes it); ready when the last event exists.
static mdt_status host_pipeline_init(mdt_fx_plan p)
{
    if (p->ev_out[1]) return MDT_SUCCESS;
    const mdt_fx_desc &d = p->d;
    const size_t in_bytes = spectrum_bytes(d) * (size_t)(d.nspectra + d.ntaps - 1);
    const size_t vb = sizeof(float2) * (size_t)d.nchannels * d.nelements * d.nelements;
    cudaError_t e = cudaSuccess;
    if (!p->copy_stream) e = cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && !p->out_stream)
        e = cudaStreamCreateWithFlags(&p->out_stream, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        if (!p->stage_in[i]) {
            void *q = nullptr;
            e = cudaMalloc(&q, in_bytes);
            if (e == cudaSuccess) {
                p->stage_in[i] = static_cast<int8_t *>(q);
                p->bytes += in_bytes;
            }
        }
        if (e == cudaSuccess && !p->stage_vis[i]) {
            void *q = nullptr;
            e = cudaMalloc(&q, vb);
            if (e == cudaSuccess) {
                p->stage_vis[i] = static_cast<float2 *>(q);
                p->bytes += vb;
            }
        }
        if (e == cudaSuccess && !p->ev_in[i])
            e = cudaEventCreateWithFlags(&p->ev_in[i], cudaEventDisableTiming);
        if (e == cudaSuccess && !p->ev_done[i])
            e = cudaEventCreateWithFlags(&p->ev_done[i], cudaEventDisableTiming);
        if (e == cudaSuccess && !p->ev_out[i])
            e = cudaEventCreateWithFlags(&p->ev_out[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        mdt::cuda_status(e, "fx_execute_host: staging buffers");
        return MDT_ERR_ALLOC;
    }
    return MDT_SUCCESS;
}

// Host-memory pipeline: integration j's samples are copied host->device on a
// copy stream while integration j-1 is processed and j-2's visibilities are
// copied back on a third stream (so the input copies, which bound the
// pipeline, run back to back); the PFB history is carried on the device
// between integrations (the reference's rank 1 -> rank 2 -> rank 3 chain,
// MDT_OneStation_client.cu :1048, :1083-1128, :1170, :1199).  Returns after
// the last copy completes.
MDT_API mdt_status mdt_fx_execute_host(mdt_fx_plan plan, const int8_t *h_iq, int nint,
                                       void *h_vis)
{
    if (!plan || !h_iq || !h_vis || nint < 0) return mdt::invalid("fx_execute_host: bad arguments");
    if (!plan->window_set) {
        mdt::set_error("fx_execute_host: no window set");
        return MDT_ERR_STATE;
    }
    if (nint == 0) return MDT_SUCCESS;
    mdt_status st = host_pipeline_init(plan);
    if (st != MDT_SUCCESS) return st;
    const mdt_fx_desc &d = plan->d;
    const size_t sb = spectrum_bytes(d);
    const size_t vb = sizeof(float2) * (size_t)d.nchannels * d.nelements * d.nelements;
    const int nh = d.ntaps - 1;
    cudaStream_t cs = plan->copy_stream, os = plan->out_stream, ks = plan->stream;
    plan->streaming = false;
    plan->cur = 0;
    auto cuda = [&](cudaError_t e, const char *w) { return mdt::cuda_status(e, w); };
    // the copy streams start after everything already queued on the compute stream
    cudaEvent_t start = plan->ev_out[1];
    if ((st = cuda(cudaEventRecord(start, ks), "record")) != MDT_SUCCESS) return st;
    if ((st = cuda(cudaStreamWaitEvent(cs, start, 0), "wait")) != MDT_SUCCESS) return st;
    if ((st = cuda(cudaStreamWaitEvent(os, start, 0), "wait")) != MDT_SUCCESS) return st;
    auto upload = [&](int j) -> mdt_status {
        const int b = j & 1;
        const size_t off = (j == 0) ? 0 : ((size_t)j * d.nspectra + nh) * sb;
        const size_t len = (j == 0) ? (size_t)(d.nspectra + nh) * sb : (size_t)d.nspectra * sb;
        if (j >= 2) {  // stage_in[b] was read by integration j-2
            mdt_status s2 = cuda(cudaStreamWaitEvent(cs, plan->ev_done[b], 0), "wait");
            if (s2 != MDT_SUCCESS) return s2;
        }
        mdt_status s2 = cuda(cudaMemcpyAsync(plan->stage_in[b], h_iq + off, len,
                                             cudaMemcpyHostToDevice, cs), "H2D");
        if (s2 == MDT_SUCCESS) s2 = cuda(cudaEventRecord(plan->ev_in[b], cs), "record");
        return s2;
    };
    if ((st = upload(0)) != MDT_SUCCESS) return st;
    for (int j = 0; j < nint; j++) {
        const int b = j & 1;
        if (j + 1 < nint && (st = upload(j + 1)) != MDT_SUCCESS) return st;
        if ((st = cuda(cudaStreamWaitEvent(ks, plan->ev_in[b], 0), "wait")) != MDT_SUCCESS)
            return st;
        if (j >= 2 && (st = cuda(cudaStreamWaitEvent(ks, plan->ev_out[b], 0), "wait")) !=
                          MDT_SUCCESS)
            return st;
        if ((st = stream_push(plan, plan->stage_in[b], plan->stage_vis[b])) != MDT_SUCCESS)
            return st;
        if ((st = cuda(cudaEventRecord(plan->ev_done[b], ks), "record")) != MDT_SUCCESS) return st;
        if ((st = cuda(cudaStreamWaitEvent(os, plan->ev_done[b], 0), "wait")) != MDT_SUCCESS)
            return st;
        if ((st = cuda(cudaMemcpyAsync((char *)h_vis + (size_t)j * vb, plan->stage_vis[b], vb,
                                       cudaMemcpyDeviceToHost, os), "D2H")) != MDT_SUCCESS)
            return st;
        if ((st = cuda(cudaEventRecord(plan->ev_out[b], os), "record")) != MDT_SUCCESS) return st;
    }
    if ((st = cuda(cudaStreamSynchronize(cs), "fx_execute_host: sync")) != MDT_SUCCESS) return st;
    return cuda(cudaStreamSynchronize(os), "fx_execute_host: sync");
}

MDT_API mdt_status mdt_fx_set_timing(mdt_fx_plan plan, int enable)
{
    if (!plan) return mdt::invalid("fx_set_timing: null plan");
    plan->timing = enable != 0;
    plan->tused = 0;
    return MDT_SUCCESS;
}

// Sums the recorded F-engine and X-engine kernel durations (ms) since
// timing was enabled, synchronising on the last event; resets the record.
MDT_API mdt_status mdt_fx_get_timing(mdt_fx_plan plan, double *fengine_ms, double *xengine_ms,
                                     int *count)
{
    if (!plan || !fengine_ms || !xengine_ms || !count) return mdt::invalid("fx_get_timing: null");
    *fengine_ms = *xengine_ms = 0.0;
    *count = (int)(plan->tused / 3);
    if (plan->tused) {
        mdt_status st = mdt::cuda_status(cudaEventSynchronize(plan->tev[plan->tused - 1]),
                                         "fx_get_timing");
        if (st != MDT_SUCCESS) return st;
    }
    for (size_t i = 0; i + 2 < plan->tused; i += 3) {
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, plan->tev[i], plan->tev[i + 1]);
        cudaEventElapsedTime(&b, plan->tev[i + 1], plan->tev[i + 2]);
        *fengine_ms += a;
        *xengine_ms += b;
    }
    plan->tused = 0;
    return MDT_SUCCESS;
}

}  // extern "C"
