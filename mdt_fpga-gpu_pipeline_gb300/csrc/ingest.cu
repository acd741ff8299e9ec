// ingest.cu -- streaming ingest pipeline (mdt_ingest_*): host packets ->
// pinned ring -> GPU depacketiser -> F-engine + X-engine -> (formatter) ->
// pinned output ring, one integration after another with the PFB history
// carried on the device.
//
// It stands in for the reference client's whole per-integration chain on one
// GPU: rank 1's depacketise-and-stack loop and its H2D copies
// (MDT_OneStation_client.cu:846-1050), rank 2's F/X processing (:1071-1152),
// rank 3's history shift and result copy (:1160-1199) and the MPI handshakes
// between them (:1022,1048,1075,1100,1121,1150,1170,1187,1234).
//
// Windows.  Integration n reads element-samples [sample0(n), sample0(n) +
// nspectra(n)*Nch): window 0 holds Nsp + Ntaps - 1 spectra from sample 0
// (the reference's first stack plus its Ntaps-1 lead-in spectra,
// :846-913); window n >= 1 holds the Nsp spectra after that.  Two windows are
// open at a time (the reference's two stacks).  A packet for window
// cur + 2 or later closes the oldest open window: its missing packets are
// zero-filled (counted), and it is processed.  Packets for closed windows are
// counted as late and dropped.
//
// Streams.  Packet batches are copied on a copy stream from a double-buffered
// pinned staging area; depacketising, closing and the F/X work run on the
// compute stream; results go back on the copy stream into a ring of pinned
// output slots that mdt_ingest_pop drains.  From the third integration on,
// the per-integration F/X (+ formatter) work is replayed as one CUDA graph per
// buffer parity.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "mdt_common.cuh"

namespace {

constexpr int OUT_SLOTS = 3;

struct WinGeom {
    long long sample0;
    int nspectra;
};

}  // namespace

struct mdt_ingest_s {
    mdt_fx_desc d{};
    mdt_packet_format fmt{};
    int formatted = 0;
    int max_packets = 0;
    mdt_fx_plan plan = nullptr;
    cudaStream_t s = nullptr, cs = nullptr;
    // packet staging
    unsigned char *h_pk[2] = {nullptr, nullptr}, *d_pk[2] = {nullptr, nullptr};
    cudaEvent_t ev_used[2] = {nullptr, nullptr};
    bool pk_busy[2] = {false, false};
    int pk_next = 0;
    // open windows (slot = window & 1)
    int8_t *win_iq[2] = {nullptr, nullptr};
    unsigned int *seen[2] = {nullptr, nullptr};
    mdt_depack_stats *d_stats = nullptr;  // [2]
    long long recv[2] = {0, 0};           // packets sent to each open window
    long long cur = 0;
    // results
    void *d_vis[2] = {nullptr, nullptr}, *d_fmt[2] = {nullptr, nullptr};
    size_t vis_bytes = 0, out_bytes = 0;
    void *h_out[OUT_SLOTS] = {};
    mdt_depack_stats *h_stats = nullptr;  // pinned [OUT_SLOTS]
    cudaEvent_t ev_comp[2] = {nullptr, nullptr}, ev_par[2] = {nullptr, nullptr};
    bool par_used[2] = {false, false};
    cudaEvent_t ev_out[OUT_SLOTS] = {};
    long long out_int[OUT_SLOTS] = {};
    int out_head = 0, out_count = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool window_set = false;
    long long late = 0, bad = 0;
};

namespace {

WinGeom window_geom(const mdt_fx_desc &d, long long n)
{
    if (n == 0) return {0, d.nspectra + d.ntaps - 1};
    return {((long long)d.ntaps - 1 + n * d.nspectra) * d.nchannels, d.nspectra};
}

long long window_of(const mdt_fx_desc &d, long long x)
{
    const long long spec = x / d.nchannels;
    if (spec < (long long)d.ntaps - 1 + d.nspectra) return 0;
    return (spec - (d.ntaps - 1)) / d.nspectra;
}

void release(mdt_ingest ing)
{
    if (!ing) return;
    if (ing->s) cudaStreamSynchronize(ing->s);
    if (ing->cs) cudaStreamSynchronize(ing->cs);
    if (ing->plan) mdt_fx_destroy(ing->plan);
    for (int i = 0; i < 2; i++) {
        cudaFreeHost(ing->h_pk[i]);
        cudaFree(ing->d_pk[i]);
        cudaFree(ing->win_iq[i]);
        cudaFree(ing->seen[i]);
        cudaFree(ing->d_vis[i]);
        cudaFree(ing->d_fmt[i]);
        if (ing->ev_used[i]) cudaEventDestroy(ing->ev_used[i]);
        if (ing->ev_comp[i]) cudaEventDestroy(ing->ev_comp[i]);
        if (ing->ev_par[i]) cudaEventDestroy(ing->ev_par[i]);
        if (ing->graph[i]) cudaGraphExecDestroy(ing->graph[i]);
    }
    for (int k = 0; k < OUT_SLOTS; k++) {
        cudaFreeHost(ing->h_out[k]);
        if (ing->ev_out[k]) cudaEventDestroy(ing->ev_out[k]);
    }
    cudaFree(ing->d_stats);
    cudaFreeHost(ing->h_stats);
    if (ing->s) cudaStreamDestroy(ing->s);
    if (ing->cs) cudaStreamDestroy(ing->cs);
    delete ing;
}

// The per-integration F/X (+ formatter) work on the compute stream.
mdt_status fx_body(mdt_ingest ing, int slot)
{
    mdt_status st = mdt_fx_stream_push(ing->plan, ing->win_iq[slot], ing->d_vis[slot]);
    if (st == MDT_SUCCESS && ing->formatted)
        st = mdt_format_baselines(ing->d.nelements, 1, ing->d.nchannels, ing->d_vis[slot],
                                  ing->d_fmt[slot], 1, ing->s);
    return st;
}

// Closes the oldest open window: zero-fill its gaps, run it, queue its result.
mdt_status close_window(mdt_ingest ing)
{
    auto cuda = [](cudaError_t e, const char *w) { return mdt::cuda_status(e, w); };
    const long long n = ing->cur;
    const int slot = (int)(n & 1);
    const int k = (ing->out_head + ing->out_count) % OUT_SLOTS;
    const WinGeom g = window_geom(ing->d, n);
    mdt_status st = mdt_depacketise_finish(&ing->fmt, ing->d.nelements, ing->d.nchannels,
                                           g.sample0, g.nspectra, ing->win_iq[slot],
                                           ing->seen[slot], ing->d_stats + slot, ing->s);
    if (st != MDT_SUCCESS) return st;
    // the visibility buffer of this parity was last read by the copy-back of n-2
    if (ing->par_used[slot] &&
        (st = cuda(cudaStreamWaitEvent(ing->s, ing->ev_par[slot], 0), "ingest: wait")) !=
            MDT_SUCCESS)
        return st;
    if (n < 2) {
        st = fx_body(ing, slot);
    } else {
        if (!ing->graph[slot]) {
            cudaGraph_t gr = nullptr;
            st = cuda(cudaStreamBeginCapture(ing->s, cudaStreamCaptureModeThreadLocal),
                      "ingest: begin capture");
            if (st != MDT_SUCCESS) return st;
            mdt_status body = fx_body(ing, slot);
            cudaError_t e = cudaStreamEndCapture(ing->s, &gr);
            if (body != MDT_SUCCESS) {
                if (gr) cudaGraphDestroy(gr);
                return body;
            }
            if ((st = cuda(e, "ingest: end capture")) != MDT_SUCCESS) return st;
            e = cudaGraphInstantiate(&ing->graph[slot], gr, 0);
            cudaGraphDestroy(gr);
            if ((st = cuda(e, "ingest: graph instantiate")) != MDT_SUCCESS) return st;
        }
        st = cuda(cudaGraphLaunch(ing->graph[slot], ing->s), "ingest: graph launch");
    }
    if (st != MDT_SUCCESS) return st;
    // this window's counters go with its result; the slot's counters restart
    if ((st = cuda(cudaMemcpyAsync(ing->h_stats + k, ing->d_stats + slot, sizeof(mdt_depack_stats),
                                   cudaMemcpyDeviceToHost, ing->s),
                   "ingest: stats")) != MDT_SUCCESS)
        return st;
    if ((st = cuda(cudaMemsetAsync(ing->d_stats + slot, 0, sizeof(mdt_depack_stats), ing->s),
                   "ingest: stats")) != MDT_SUCCESS)
        return st;
    if ((st = cuda(cudaEventRecord(ing->ev_comp[slot], ing->s), "ingest: record")) != MDT_SUCCESS)
        return st;
    if ((st = cuda(cudaStreamWaitEvent(ing->cs, ing->ev_comp[slot], 0), "ingest: wait")) !=
        MDT_SUCCESS)
        return st;
    const void *src = ing->formatted ? ing->d_fmt[slot] : ing->d_vis[slot];
    if ((st = cuda(cudaMemcpyAsync(ing->h_out[k], src, ing->out_bytes, cudaMemcpyDeviceToHost,
                                   ing->cs),
                   "ingest: D2H")) != MDT_SUCCESS)
        return st;
    if ((st = cuda(cudaEventRecord(ing->ev_out[k], ing->cs), "ingest: record")) != MDT_SUCCESS)
        return st;
    if ((st = cuda(cudaEventRecord(ing->ev_par[slot], ing->cs), "ingest: record")) != MDT_SUCCESS)
        return st;
    ing->par_used[slot] = true;
    ing->out_int[k] = n;
    ing->out_count++;
    ing->recv[slot] = 0;
    ing->cur++;
    return MDT_SUCCESS;
}

}  // namespace

extern "C" {

MDT_API mdt_status mdt_ingest_create(const mdt_fx_desc *desc, const mdt_packet_format *fmt,
                                     int max_packets, int formatted, mdt_ingest *out)
{
    if (!desc || !fmt || !out || max_packets < 1) return mdt::invalid("ingest_create: bad arguments");
    *out = nullptr;
    if (fmt->sample_bits != 8) {
        mdt::set_error("ingest_create: the pipeline consumes int8 I/Q packets (sample_bits 8); "
                       "32-bit packets feed the drop-in path through mdt_depacketise");
        return MDT_ERR_NOT_SUPPORTED;
    }
    if ((long long)fmt->sper_element > (long long)desc->nspectra * desc->nchannels)
        return mdt::invalid("ingest_create: a packet must not span more than two windows");
    size_t words = 0;
    mdt_status st = mdt_depacketise_seen_words(fmt, desc->nelements, desc->nchannels, 0,
                                               desc->nspectra + desc->ntaps - 1, &words);
    if (st != MDT_SUCCESS) return st;
    // window n >= 1 can touch one slot more than its length in packets
    const size_t groups = (size_t)mdt::cdiv(desc->nelements, fmt->inputs_per_station) * fmt->nsnap;
    words = std::max(words, groups * (size_t)(mdt::cdiv((long)desc->nspectra * desc->nchannels,
                                                        fmt->sper_element) + 1));
    mdt_ingest ing = new (std::nothrow) mdt_ingest_s;
    if (!ing) return MDT_ERR_ALLOC;
    ing->d = *desc;
    ing->fmt = *fmt;
    ing->formatted = formatted ? 1 : 0;
    ing->max_packets = max_packets;
    if ((st = mdt_fx_create(desc, &ing->plan)) != MDT_SUCCESS) {
        release(ing);
        return st;
    }
    const mdt_fx_desc &d = ing->d;
    const size_t stage = (size_t)2 * max_packets * fmt->packet_bytes;  // straddling packets twice
    const size_t win_bytes = (size_t)(d.nspectra + d.ntaps - 1) * d.nelements * d.nchannels * 2;
    ing->vis_bytes = sizeof(float2) * (size_t)d.nchannels * d.nelements * d.nelements;
    long nbl = 0;
    mdt_num_baselines(d.nelements, 1, &nbl);
    ing->out_bytes = ing->formatted ? sizeof(float2) * (size_t)nbl * d.nchannels : ing->vis_bytes;
    cudaError_t e = cudaStreamCreateWithFlags(&ing->s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ing->cs, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaHostAlloc(&ing->h_pk[i], stage, cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaMalloc(&ing->d_pk[i], stage);
        if (e == cudaSuccess) e = cudaMalloc(&ing->win_iq[i], win_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&ing->seen[i], sizeof(unsigned int) * words);
        if (e == cudaSuccess) e = cudaMemset(ing->seen[i], 0, sizeof(unsigned int) * words);
        if (e == cudaSuccess) e = cudaMalloc(&ing->d_vis[i], ing->vis_bytes);
        if (e == cudaSuccess && ing->formatted) e = cudaMalloc(&ing->d_fmt[i], ing->out_bytes);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ing->ev_used[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ing->ev_comp[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ing->ev_par[i], cudaEventDisableTiming);
    }
    for (int k = 0; k < OUT_SLOTS && e == cudaSuccess; k++) {
        e = cudaHostAlloc(&ing->h_out[k], ing->out_bytes, cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ing->ev_out[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaMalloc(&ing->d_stats, 2 * sizeof(mdt_depack_stats));
    if (e == cudaSuccess) e = cudaMemset(ing->d_stats, 0, 2 * sizeof(mdt_depack_stats));
    if (e == cudaSuccess)
        e = cudaHostAlloc(&ing->h_stats, OUT_SLOTS * sizeof(mdt_depack_stats), cudaHostAllocDefault);
    if (e != cudaSuccess) {
        mdt::cuda_status(e, "ingest_create: buffers");
        release(ing);
        return MDT_ERR_ALLOC;
    }
    if ((st = mdt_fx_set_stream(ing->plan, ing->s)) != MDT_SUCCESS) {
        release(ing);
        return st;
    }
    *out = ing;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_ingest_destroy(mdt_ingest ing)
{
    if (!ing) return mdt::invalid("ingest_destroy: null");
    release(ing);
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_ingest_set_window(mdt_ingest ing, const float *window)
{
    if (!ing || !window) return mdt::invalid("ingest_set_window: null argument");
    mdt_status st = mdt_fx_set_window(ing->plan, window);
    if (st == MDT_SUCCESS) ing->window_set = true;
    return st;
}

MDT_API mdt_status mdt_ingest_push(mdt_ingest ing, const void *packets, int npackets)
{
    if (!ing || npackets < 0 || (npackets && !packets)) return mdt::invalid("ingest_push: bad arguments");
    if (!ing->window_set) {
        mdt::set_error("ingest_push: no window set");
        return MDT_ERR_STATE;
    }
    if (npackets > ing->max_packets) return mdt::invalid("ingest_push: more packets than max_packets");
    if (npackets == 0) return MDT_SUCCESS;
    const mdt_fx_desc &d = ing->d;
    const mdt_packet_format &f = ing->fmt;
    const unsigned char *pk = (const unsigned char *)packets;
    const int nstation = (int)mdt::cdiv(d.nelements, f.inputs_per_station);
    // host scan of the headers: which open window(s) each packet belongs to
    std::vector<std::vector<int>> per;  // index w - cur
    long long bad = 0, late = 0, maxw = ing->cur - 1;
    for (int p = 0; p < npackets; p++) {
        uint32_t h[3];
        std::memcpy(h, pk + (size_t)p * f.packet_bytes, sizeof h);
        if (h[1] >= (uint32_t)f.nsnap || h[0] >= (uint32_t)nstation) {
            bad++;
            continue;
        }
        long e0 = (long)h[0] * f.inputs_per_station;
        for (uint32_t k = 0; k < h[1]; k++) e0 += f.inputs_per_snap[k];
        if (e0 + f.inputs_per_snap[h[1]] > d.nelements || f.inputs_per_snap[h[1]] == 0) {
            bad++;
            continue;
        }
        const long long first = (long long)h[2] * f.sper_element;
        const long long w0 = window_of(d, first), w1 = window_of(d, first + f.sper_element - 1);
        if (w1 < ing->cur) {
            late++;
            continue;
        }
        for (long long w = std::max(w0, ing->cur); w <= w1; w++) {
            const size_t i = (size_t)(w - ing->cur);
            if (per.size() <= i) per.resize(i + 1);
            per[i].push_back(p);
            maxw = std::max(maxw, w);
        }
    }
    const long long closes = std::max(0LL, maxw - (ing->cur + 1));
    if (ing->out_count + closes > OUT_SLOTS) {
        mdt::set_error("ingest_push: the output ring is full; pop results first");
        return MDT_ERR_STATE;
    }
    ing->bad += bad;
    ing->late += late;
    if (maxw < ing->cur) return MDT_SUCCESS;
    auto cuda = [](cudaError_t e, const char *w) { return mdt::cuda_status(e, w); };
    // stage the accepted packets, grouped by window
    const int b = ing->pk_next;
    mdt_status st;
    if (ing->pk_busy[b] &&
        (st = cuda(cudaEventSynchronize(ing->ev_used[b]), "ingest: staging")) != MDT_SUCCESS)
        return st;
    std::vector<size_t> off(per.size() + 1, 0);
    size_t n = 0;
    for (size_t i = 0; i < per.size(); i++) {
        off[i] = n;
        for (int p : per[i])
            std::memcpy(ing->h_pk[b] + (n++) * f.packet_bytes, pk + (size_t)p * f.packet_bytes,
                        f.packet_bytes);
    }
    off[per.size()] = n;
    if ((st = cuda(cudaMemcpyAsync(ing->d_pk[b], ing->h_pk[b], n * f.packet_bytes,
                                   cudaMemcpyHostToDevice, ing->cs),
                   "ingest: H2D")) != MDT_SUCCESS)
        return st;
    cudaEvent_t ev_h2d = ing->ev_used[b];  // reused: recorded again after the depacketise
    if ((st = cuda(cudaEventRecord(ev_h2d, ing->cs), "ingest: record")) != MDT_SUCCESS) return st;
    if ((st = cuda(cudaStreamWaitEvent(ing->s, ev_h2d, 0), "ingest: wait")) != MDT_SUCCESS)
        return st;
    const long long base = ing->cur;
    for (size_t i = 0; i < per.size(); i++) {
        const long long w = base + (long long)i;
        while (w >= ing->cur + 2)
            if ((st = close_window(ing)) != MDT_SUCCESS) return st;
        const size_t cnt = off[i + 1] - off[i];
        if (!cnt) continue;
        const int slot = (int)(w & 1);
        const WinGeom g = window_geom(d, w);
        if ((st = mdt_depacketise(&f, ing->d_pk[b] + off[i] * f.packet_bytes, (int)cnt,
                                  d.nelements, d.nchannels, g.sample0, g.nspectra,
                                  ing->win_iq[slot], ing->seen[slot], ing->d_stats + slot,
                                  ing->s)) != MDT_SUCCESS)
            return st;
        ing->recv[slot] += (long long)cnt;
    }
    if ((st = cuda(cudaEventRecord(ing->ev_used[b], ing->s), "ingest: record")) != MDT_SUCCESS)
        return st;
    ing->pk_busy[b] = true;
    ing->pk_next ^= 1;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_ingest_flush(mdt_ingest ing)
{
    if (!ing) return mdt::invalid("ingest_flush: null");
    const int open = (ing->recv[ing->cur & 1] > 0 || ing->recv[(ing->cur + 1) & 1] > 0) +
                     (ing->recv[(ing->cur + 1) & 1] > 0);
    if (ing->out_count + open > OUT_SLOTS) {
        mdt::set_error("ingest_flush: the output ring is full; pop results first");
        return MDT_ERR_STATE;
    }
    mdt_status st = MDT_SUCCESS;
    for (int i = 0; i < open && st == MDT_SUCCESS; i++) st = close_window(ing);
    return st;
}

MDT_API mdt_status mdt_ingest_pop(mdt_ingest ing, void *out, long long *integration,
                                  mdt_depack_stats *stats, int wait)
{
    if (!ing || !integration) return mdt::invalid("ingest_pop: bad arguments");
    *integration = -1;
    if (ing->out_count == 0) return MDT_SUCCESS;
    const int k = ing->out_head;
    cudaError_t e = wait ? cudaEventSynchronize(ing->ev_out[k]) : cudaEventQuery(ing->ev_out[k]);
    if (!wait && e == cudaErrorNotReady) return MDT_SUCCESS;
    mdt_status st = mdt::cuda_status(e, "ingest_pop");
    if (st != MDT_SUCCESS) return st;
    if ((st = mdt_fx_check(ing->plan)) != MDT_SUCCESS) return st;
    if (out) std::memcpy(out, ing->h_out[k], ing->out_bytes);
    if (stats) *stats = ing->h_stats[k];
    *integration = ing->out_int[k];
    ing->out_head = (k + 1) % OUT_SLOTS;
    ing->out_count--;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_ingest_counters(mdt_ingest ing, long long *late, long long *bad,
                                       long long *next_window, size_t *out_bytes)
{
    if (!ing) return mdt::invalid("ingest_counters: null");
    if (late) *late = ing->late;
    if (bad) *bad = ing->bad;
    if (next_window) *next_window = ing->cur;
    if (out_bytes) *out_bytes = ing->out_bytes;
    return MDT_SUCCESS;
}

}  // extern "C"
