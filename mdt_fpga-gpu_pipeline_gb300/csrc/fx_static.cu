// fx_static.cu -- one FP32 FX integration that allocates no device memory.
//
// Some callers cannot allocate device memory themselves: a real-time ingest
// loop in which cudaMalloc's implicit device synchronisation would stall the
// other streams, a plugin host that gives the library a fixed device-memory
// budget up front, or a foreign-language runtime that owns every device
// allocation.  For them mdt_fx_integrate_static runs the plan's FP32 path
// (spectrum-block F-engine -> Hermitian X-engine) with its F-engine output
// in a file-scope device array instead of a plan workspace, and its FFT
// twiddle tables in a second file-scope array.  The caller passes only the
// samples, the window and the visibility buffer.
//
// The arrays are static __device__ storage: every GPU that loads the library
// holds them (MDT_STATIC_SCRATCH_BYTES + 32.5 KB) until the process exits.
// In host code their names are host-side stand-ins, not device addresses, so
// the first call on each device, with that device current, looks their
// device addresses up with cudaGetSymbolAddress and fills the twiddle tables
// (a host-to-device copy); that first call should therefore come before any
// stream capture.  Under CUDA's default lazy module loading the device
// memory of the arrays is committed when this file's module is first used,
// that is, by the first call on each device (with CUDA_MODULE_LOADING=EAGER,
// when the context is created).  A real-time caller therefore makes one
// warm-up call per device outside its loop.  Every call on a device shares the same scratch and
// overwrites all of the part it uses before reading it, so nothing needs
// clearing between calls; calls whose work overlaps on the GPU (different
// streams, or the same array used from two threads) race on the scratch.
#include <cmath>
#include <mutex>
#include <vector>

#include "fengine.cuh"
#include "mdt_common.cuh"

namespace mdt {
mdt_status check_dims(int ne, int nch, int ntaps, int nsp);
mdt_status fengine_c64b_given_twiddles(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                       const float *win, float2 *XB, const float2 *tw_concat,
                                       cudaStream_t stream);
mdt_status xengine_herm_f32(int ne, long nbatch, int nsp, const float2 *X,
                            const float2 *const *Xptrs, long ld, long xstride, float2 *V,
                            float2 *const *Vptrs, long ldv, long vstride, float2 alpha,
                            float2 beta, bool beta_zero, cudaStream_t stream, int blocked);
}  // namespace mdt

namespace {

// F-engine output of one integration in the 8-spectrum blocked layout:
// Nch * ceil(Nsp/8) * 8 * NE complex64 values must fit.
constexpr size_t kScratchBytes = (size_t)MDT_STATIC_SCRATCH_BYTES;
constexpr int kTwiddleEntries = 2048 * 2 - 32;  // tables for N = 32..2048, back to back

static __device__ __align__(256) float2 g_fx_scratch[kScratchBytes / sizeof(float2)];
static __device__ __align__(256) float2 g_fx_twiddles[kTwiddleEntries];

struct DeviceSlots {
    bool ready = false;
    float2 *scratch = nullptr;
    float2 *twiddles = nullptr;
};
std::mutex g_mu;
std::vector<DeviceSlots> g_slots;

// Once per device, with the device current: device addresses of the two
// arrays and the twiddle tables exp(-2 pi i k / N) (double, rounded to float,
// the same values as the library's per-device tables).  The two addresses
// are copied out while the lock is held: a first call on a higher device
// index grows g_slots and may move its elements, so no reference into the
// table outlives the lock.
mdt_status setup_current_device(float2 **scratch, float2 **twiddles)
{
    int dev = 0;
    mdt_status st = mdt::cuda_status(cudaGetDevice(&dev), "fx_integrate_static: device");
    if (st != MDT_SUCCESS) return st;
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_slots.size() <= dev) g_slots.resize(dev + 1);
    DeviceSlots &d = g_slots[dev];
    if (!d.ready) {
        float2 *sp = nullptr, *tp = nullptr;
        st = mdt::cuda_status(cudaGetSymbolAddress((void **)&sp, g_fx_scratch),
                              "fx_integrate_static: scratch address");
        if (st != MDT_SUCCESS) return st;
        st = mdt::cuda_status(cudaGetSymbolAddress((void **)&tp, g_fx_twiddles),
                              "fx_integrate_static: twiddle address");
        if (st != MDT_SUCCESS) return st;
        std::vector<float2> h(kTwiddleEntries);
        for (int n = 32; n <= 2048; n *= 2)
            for (int k = 0; k < n; k++) {
                double a = -2.0 * 3.141592653589793238462643383279502884 * (double)k / (double)n;
                h[n - 32 + k] = make_float2((float)cos(a), (float)sin(a));
            }
        st = mdt::cuda_status(cudaMemcpy(tp, h.data(), sizeof(float2) * h.size(),
                                         cudaMemcpyHostToDevice),
                              "fx_integrate_static: twiddle upload");
        if (st != MDT_SUCCESS) return st;
        d.scratch = sp;
        d.twiddles = tp;
        d.ready = true;
    }
    *scratch = d.scratch;
    *twiddles = d.twiddles;
    return MDT_SUCCESS;
}

}  // namespace

extern "C" MDT_API mdt_status mdt_fx_integrate_static(int ne, int nch, int ntaps, int nsp,
                                                      const int8_t *iq, const float *window,
                                                      void *vis, cudaStream_t stream)
{
    mdt_status st = mdt::check_dims(ne, nch, ntaps, nsp);
    if (st != MDT_SUCCESS) return st;
    if (!iq || !window || !vis) return mdt::invalid("fx_integrate_static: null pointer");
    if (nch > 2048) return mdt::invalid("fx_integrate_static: Nch must be <= 2048");
    const size_t need = sizeof(float2) * (size_t)nch * (size_t)((nsp + 7) / 8 * 8) * (size_t)ne;
    if (need > kScratchBytes)
        return mdt::invalid("fx_integrate_static: the F-engine output needs " +
                            std::to_string(need) + " bytes (Nch * ceil(Nsp/8)*8 * NE * 8), more "
                            "than the static scratch of " + std::to_string(kScratchBytes) +
                            " bytes");
    float2 *scratch = nullptr, *twiddles = nullptr;
    st = setup_current_device(&scratch, &twiddles);
    if (st != MDT_SUCCESS) return st;
    st = mdt::fengine_c64b_given_twiddles(ne, nch, ntaps, nsp, iq, window, scratch, twiddles,
                                          stream);
    if (st != MDT_SUCCESS) return st;
    const long nsb = (nsp + 7) / 8;
    return mdt::xengine_herm_f32(ne, nch, nsp, scratch, nullptr, mdt::xb_block_stride(ne, nch, nsb),
                                 mdt::xb_chan_stride(ne, nch, nsb),
                                 (float2 *)vis, nullptr, ne, (long)ne * ne,
                                 make_float2(1.0f / nsp, 0.f), make_float2(0.f, 0.f), true,
                                 stream, 1);
}
