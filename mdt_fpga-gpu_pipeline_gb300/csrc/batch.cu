// batch.cu -- many independent correlator jobs of uneven shape (elements,
// channels, taps, spectra) processed together: one f16 F-engine launch per
// (Nch, Ntaps) group of jobs, one persistent tensor-core X-engine launch over
// a work list that spans every job, all captured once in a CUDA graph and
// replayed.  The X-engine's column-chunk width and the order of its work
// list come from an autotuner that times the candidates on the batch itself
// and caches the choice per batch shape (in memory, and in the file named by
// MDT_AUTOTUNE_CACHE when that variable is set).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "fengine.cuh"
#include "xengine_tc.cuh"

extern "C" mdt_status mdt_window_hamming_sinc(int nchannels, int ntaps, float *window,
                                              cudaStream_t stream);

namespace {

struct Group {
    int nch, ntaps;
    int first, count;  // FJob entries [first, first + count)
    long nblocks;      // blocks of the SIMT F-engine launch
    long nwork;        // work items of the tensor-core F-engine launch
    bool tc;           // tensor-core F-engine (Nch 1024, Ntaps 4 or 8)
};

struct TuneChoice {
    int maxw;
    int lpt;  // 1: work list sorted by cost, largest first; 0: job order
};

std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune_cache;
bool g_tune_file_read = false;

void read_tune_file()
{
    if (g_tune_file_read) return;
    g_tune_file_read = true;
    const char *path = getenv("MDT_AUTOTUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    char key[4096];
    int maxw, lpt;
    while (fscanf(f, "%4095s %d %d", key, &maxw, &lpt) == 3) g_tune_cache[key] = {maxw, lpt};
    fclose(f);
}

void append_tune_file(const std::string &key, TuneChoice c)
{
    const char *path = getenv("MDT_AUTOTUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%s %d %d\n", key.c_str(), c.maxw, c.lpt);
    fclose(f);
}

}  // namespace

struct mdt_fx_batch_s {
    int njobs = 0;
    std::vector<mdt_fx_desc> d;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    float *windows = nullptr;
    std::vector<size_t> win_off;
    uint8_t *x16 = nullptr;
    std::vector<size_t> x16_off;
    std::vector<int> nep, nkc;
    std::vector<float> scale;
    std::vector<Group> groups;
    std::vector<int> fjob_of;  // job of each FJob entry
    std::vector<mdt::FJob> h_fjobs;
    std::vector<mdt::XJob> h_xjobs;
    mdt::FJob *d_fjobs = nullptr;
    mdt::XJob *d_xjobs = nullptr;
    mdt::XWork *d_work = nullptr;
    int nwork = 0, work_cap = 0;
    int *d_err = nullptr;
    bool tuned = false;
    TuneChoice choice{mdt::TCB_MAXW, 1};
    cudaGraphExec_t exec = nullptr;
    size_t bytes = 0;
};

namespace {

void release(mdt_fx_batch b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    cudaFree(b->windows);
    cudaFree(b->x16);
    cudaFree(b->d_fjobs);
    cudaFree(b->d_xjobs);
    cudaFree(b->d_work);
    cudaFree(b->d_err);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Power-of-two f16 scale keeping 127 sqrt(2) sum|W| under 60000 (as the plan).
float window_scale(const std::vector<float> &w)
{
    double sum = 0;
    for (float x : w) sum += fabs((double)x);
    const double bound = 127.0 * 1.4142135623730951 * sum;
    int ex = 0;
    while (bound * std::ldexp(1.0, -ex) > 60000.0 && ex < 60) ex++;
    return (float)std::ldexp(1.0, -ex);
}

mdt_status refresh_scale(mdt_fx_batch b, int j)
{
    const mdt_fx_desc &d = b->d[j];
    std::vector<float> h((size_t)d.ntaps * d.nchannels);
    mdt_status st = mdt::cuda_status(cudaMemcpy(h.data(), b->windows + b->win_off[j],
                                                sizeof(float) * h.size(), cudaMemcpyDeviceToHost),
                                     "batch: window");
    if (st != MDT_SUCCESS) return st;
    b->scale[j] = window_scale(h);
    return MDT_SUCCESS;
}

std::vector<mdt::XWork> build_work(mdt_fx_batch b, TuneChoice c)
{
    std::vector<mdt::XWork> work;
    std::vector<long> cost;
    mdt::TcTile tiles[160];
    for (int j = 0; j < b->njobs; j++) {
        const mdt_fx_desc &d = b->d[j];
        const int nt = mdt::make_tiles(d.nelements, b->nep[j], c.maxw, tiles);
        for (int ch = 0; ch < d.nchannels; ch++)
            for (int t = 0; t < nt; t++) {
                work.push_back({j, ch, tiles[t]});
                cost.push_back((long)b->nkc[j] * (tiles[t].n + (tiles[t].a_sep ? 128 : 0)));
            }
    }
    if (c.lpt) {
        std::vector<size_t> idx(work.size());
        for (size_t i = 0; i < idx.size(); i++) idx[i] = i;
        std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
        std::vector<mdt::XWork> sorted;
        sorted.reserve(work.size());
        for (size_t i : idx) sorted.push_back(work[i]);
        work.swap(sorted);
    }
    return work;
}

mdt_status upload_work(mdt_fx_batch b, const std::vector<mdt::XWork> &work)
{
    if ((int)work.size() > b->work_cap) {
        cudaFree(b->d_work);
        b->d_work = nullptr;
        cudaError_t e = cudaMalloc(&b->d_work, sizeof(mdt::XWork) * work.size());
        if (e != cudaSuccess) return mdt::cuda_status(e, "batch: work list");
        b->work_cap = (int)work.size();
    }
    b->nwork = (int)work.size();
    return mdt::cuda_status(cudaMemcpy(b->d_work, work.data(), sizeof(mdt::XWork) * work.size(),
                                       cudaMemcpyHostToDevice),
                            "batch: work list upload");
}

mdt_status upload_tables(mdt_fx_batch b)
{
    for (size_t i = 0; i < b->h_fjobs.size(); i++) b->h_fjobs[i].scale = b->scale[b->fjob_of[i]];
    for (int j = 0; j < b->njobs; j++)
        b->h_xjobs[j].alpha = 1.0f / ((float)b->d[j].nspectra * b->scale[j] * b->scale[j]);
    mdt_status st = mdt::cuda_status(
        cudaMemcpyAsync(b->d_fjobs, b->h_fjobs.data(), sizeof(mdt::FJob) * b->h_fjobs.size(),
                        cudaMemcpyHostToDevice, b->stream),
        "batch: job table");
    if (st != MDT_SUCCESS) return st;
    return mdt::cuda_status(
        cudaMemcpyAsync(b->d_xjobs, b->h_xjobs.data(), sizeof(mdt::XJob) * b->h_xjobs.size(),
                        cudaMemcpyHostToDevice, b->stream),
        "batch: job table");
}

std::string tune_key(mdt_fx_batch b)
{
    std::string k = "sm" + std::to_string(mdt::sm_count());
    for (const mdt_fx_desc &d : b->d)
        k += "_" + std::to_string(d.nelements) + "x" + std::to_string(d.nchannels) + "x" +
             std::to_string(d.nspectra);
    return k;
}

// Times every candidate (maxw in {64, 128}) x (order in {cost, job}) on the
// batch's own X-engine launch and keeps the fastest.
mdt_status autotune(mdt_fx_batch b)
{
    const std::string key = tune_key(b);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        read_tune_file();
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            b->choice = it->second;
            b->tuned = true;
            return upload_work(b, build_work(b, b->choice));
        }
    }
    mdt_status st = upload_tables(b);
    if (st != MDT_SUCCESS) return st;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return mdt::cuda_status(cudaGetLastError(), "batch: autotune events");
    float best = 1e30f;
    TuneChoice bestc{mdt::TCB_MAXW, 1};
    const TuneChoice cands[4] = {{128, 1}, {64, 1}, {128, 0}, {64, 0}};
    for (TuneChoice c : cands) {
        st = upload_work(b, build_work(b, c));
        if (st != MDT_SUCCESS) break;
        st = mdt::xengine_tc_batched(b->d_xjobs, b->d_work, b->nwork, b->d_err, b->stream);
        if (st != MDT_SUCCESS) break;
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < 3 && st == MDT_SUCCESS; r++)
            st = mdt::xengine_tc_batched(b->d_xjobs, b->d_work, b->nwork, b->d_err, b->stream);
        cudaEventRecord(e1, b->stream);
        if (st != MDT_SUCCESS) break;
        st = mdt::cuda_status(cudaEventSynchronize(e1), "batch: autotune");
        if (st != MDT_SUCCESS) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            bestc = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != MDT_SUCCESS) return st;
    b->choice = bestc;
    b->tuned = true;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = bestc;
        append_tune_file(key, bestc);
    }
    return upload_work(b, build_work(b, bestc));
}

mdt_status launch_all(mdt_fx_batch b)
{
    for (const Group &g : b->groups) {
        mdt_status st = g.tc ? mdt::fengine_tc_batched(g.ntaps, b->d_fjobs + g.first, g.count,
                                                       g.nwork, b->d_err, b->stream)
                             : mdt::fengine_x16_batched(g.nch, g.ntaps, b->d_fjobs + g.first,
                                                        g.count, g.nblocks, b->stream);
        if (st != MDT_SUCCESS) return st;
    }
    return mdt::xengine_tc_batched(b->d_xjobs, b->d_work, b->nwork, b->d_err, b->stream);
}

}  // namespace

extern "C" {

MDT_API mdt_status mdt_fx_batch_create(const mdt_fx_desc *descs, int njobs, mdt_fx_batch *out)
{
    if (!descs || !out || njobs < 1 || njobs > 4096) return mdt::invalid("fx_batch_create: bad arguments");
    *out = nullptr;
    for (int j = 0; j < njobs; j++) {
        const mdt_fx_desc &d = descs[j];
        mdt_status st = mdt::check_dims(d.nelements, d.nchannels, d.ntaps, d.nspectra);
        if (st != MDT_SUCCESS) return st;
        if (d.precision != MDT_PREC_FP16 || d.nchannels > 2048 || (d.ntaps != 4 && d.ntaps != 8)) {
            mdt::set_error("fx_batch_create: batched jobs take FP16 precision, Nch <= 2048 and "
                           "Ntaps 4 or 8");
            return MDT_ERR_NOT_SUPPORTED;
        }
    }
    mdt_fx_batch b = new (std::nothrow) mdt_fx_batch_s;
    if (!b) return MDT_ERR_ALLOC;
    b->njobs = njobs;
    b->d.assign(descs, descs + njobs);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    b->own_stream = true;
    size_t wtot = 0, xtot = 0;
    for (int j = 0; j < njobs; j++) {
        const mdt_fx_desc &d = b->d[j];
        b->win_off.push_back(wtot);
        wtot += (size_t)d.ntaps * d.nchannels;
        wtot = (wtot + 3) / 4 * 4;  // 16-byte aligned windows
        b->nep.push_back(mdt::x16_padded_rows(d.nelements));
        b->nkc.push_back(mdt::x16_chunks(d.nspectra));
        b->x16_off.push_back(xtot);
        xtot += (size_t)d.nchannels * b->nkc[j] * b->nep[j] * 128;
    }
    b->scale.assign(njobs, 1.0f);
    if (e == cudaSuccess) e = cudaMalloc(&b->windows, sizeof(float) * wtot);
    if (e == cudaSuccess) e = cudaMalloc(&b->x16, xtot);
    if (e == cudaSuccess) e = cudaMemset(b->x16, 0, xtot);  // padding rows stay zero
    if (e == cudaSuccess) e = cudaMalloc(&b->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_fjobs, sizeof(mdt::FJob) * njobs);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_xjobs, sizeof(mdt::XJob) * njobs);
    if (e != cudaSuccess) {
        release(b);
        mdt::cuda_status(e, "fx_batch_create");
        return MDT_ERR_ALLOC;
    }
    b->bytes = sizeof(float) * wtot + xtot;
    mdt_status st = MDT_SUCCESS;
    // default windows: the Hamming windowed sinc; twiddle tables made now,
    // outside any capture
    for (int j = 0; j < njobs && st == MDT_SUCCESS; j++) {
        st = mdt_window_hamming_sinc(b->d[j].nchannels, b->d[j].ntaps, b->windows + b->win_off[j],
                                     b->stream);
        if (st == MDT_SUCCESS && !mdt::fft_twiddles(b->d[j].nchannels, &st)) break;
    }
    if (st == MDT_SUCCESS) st = mdt::cuda_status(cudaStreamSynchronize(b->stream), "fx_batch_create");
    for (int j = 0; j < njobs && st == MDT_SUCCESS; j++) st = refresh_scale(b, j);
    if (st != MDT_SUCCESS) {
        release(b);
        return st;
    }
    // F-engine groups by (Nch, Ntaps), job tables; MDT_FENGINE=simt keeps
    // every group on the SIMT FFT F-engine
    const char *fe = getenv("MDT_FENGINE");
    const bool use_tc = !(fe && std::string(fe) == "simt");
    std::vector<int> order(njobs);
    for (int j = 0; j < njobs; j++) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return std::make_pair(b->d[x].nchannels, b->d[x].ntaps) <
               std::make_pair(b->d[y].nchannels, b->d[y].ntaps);
    });
    for (int idx = 0; idx < njobs; idx++) {
        const int j = order[idx];
        const mdt_fx_desc &d = b->d[j];
        if (b->groups.empty() || b->groups.back().nch != d.nchannels ||
            b->groups.back().ntaps != d.ntaps)
            b->groups.push_back({d.nchannels, d.ntaps, idx, 0, 0, 0,
                                 use_tc && mdt::fengine_tc_shape(d.nchannels, d.ntaps)});
        Group &g = b->groups.back();
        mdt::FJob f;
        f.iq = nullptr;
        f.win = b->windows + b->win_off[j];
        f.X16 = b->x16 + b->x16_off[j];
        f.ne = d.nelements;
        f.nsp = d.nspectra;
        f.nep = b->nep[j];
        f.nkc = b->nkc[j];
        f.scale = b->scale[j];
        f.blk0 = (int)g.nblocks;
        f.wk0 = (int)g.nwork;
        g.nblocks += mdt::fjob_blocks(d.nelements, b->nkc[j]);
        g.nwork += mdt::fjob_tc_items(d.nelements, d.nspectra);
        g.count++;
        b->h_fjobs.push_back(f);
        b->fjob_of.push_back(j);
    }
    for (int j = 0; j < njobs; j++) {
        const mdt_fx_desc &d = b->d[j];
        mdt::XJob x;
        x.X = b->x16 + b->x16_off[j];
        x.chan_bytes = (long)b->nep[j] * 128;
        x.chunk_bytes = (long)d.nchannels * x.chan_bytes;
        x.ne = d.nelements;
        x.nep = b->nep[j];
        x.nkc = b->nkc[j];
        x.alpha = 1.0f;
        x.V = nullptr;
        b->h_xjobs.push_back(x);
    }
    *out = b;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_batch_destroy(mdt_fx_batch b)
{
    if (!b) return mdt::invalid("fx_batch_destroy: null batch");
    if (b->stream) cudaStreamSynchronize(b->stream);
    release(b);
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_batch_set_window(mdt_fx_batch b, int job, const float *window)
{
    if (!b || !window || job < 0 || job >= b->njobs) return mdt::invalid("fx_batch_set_window: bad arguments");
    const mdt_fx_desc &d = b->d[job];
    mdt_status st = mdt::cuda_status(
        cudaMemcpyAsync(b->windows + b->win_off[job], window, sizeof(float) * d.ntaps * d.nchannels,
                        cudaMemcpyDeviceToDevice, b->stream),
        "fx_batch_set_window");
    if (st == MDT_SUCCESS) st = mdt::cuda_status(cudaStreamSynchronize(b->stream), "fx_batch_set_window");
    if (st == MDT_SUCCESS) st = refresh_scale(b, job);
    return st;
}

MDT_API mdt_status mdt_fx_batch_get_stream(mdt_fx_batch b, cudaStream_t *stream)
{
    if (!b || !stream) return mdt::invalid("fx_batch_get_stream: null argument");
    *stream = b->stream;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_batch_autotune(mdt_fx_batch b, int *maxw, int *cost_order)
{
    if (!b) return mdt::invalid("fx_batch_autotune: null batch");
    if (!b->tuned) {
        mdt_status st = autotune(b);
        if (st != MDT_SUCCESS) return st;
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
    }
    if (maxw) *maxw = b->choice.maxw;
    if (cost_order) *cost_order = b->choice.lpt;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_fx_batch_execute(mdt_fx_batch b, const int8_t *const *iq, void *const *vis,
                                        int use_graph)
{
    if (!b || !iq || !vis) return mdt::invalid("fx_batch_execute: null argument");
    for (int j = 0; j < b->njobs; j++)
        if (!iq[j] || !vis[j] || ((uintptr_t)iq[j] & 15))
            return mdt::invalid("fx_batch_execute: every job needs 16-byte aligned samples and "
                                "a visibility buffer");
    for (size_t i = 0; i < b->h_fjobs.size(); i++)
        b->h_fjobs[i].iq = reinterpret_cast<const char2 *>(iq[b->fjob_of[i]]);
    for (int j = 0; j < b->njobs; j++) b->h_xjobs[j].V = (float2 *)vis[j];
    mdt_status st = mdt_fx_batch_autotune(b, nullptr, nullptr);
    if (st != MDT_SUCCESS) return st;
    st = upload_tables(b);
    if (st != MDT_SUCCESS) return st;
    if (!use_graph) return launch_all(b);
    if (!b->exec) {
        // the kernels read every pointer from the device job tables, so the
        // captured graph stays valid when the caller's buffers change
        cudaGraph_t graph = nullptr;
        st = mdt::cuda_status(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal),
                              "fx_batch_execute: capture");
        if (st != MDT_SUCCESS) return st;
        mdt_status lst = launch_all(b);
        st = mdt::cuda_status(cudaStreamEndCapture(b->stream, &graph), "fx_batch_execute: capture");
        if (lst != MDT_SUCCESS) st = lst;
        if (st == MDT_SUCCESS)
            st = mdt::cuda_status(cudaGraphInstantiate(&b->exec, graph, 0), "fx_batch_execute: graph");
        if (graph) cudaGraphDestroy(graph);
        if (st != MDT_SUCCESS) return st;
    }
    return mdt::cuda_status(cudaGraphLaunch(b->exec, b->stream), "fx_batch_execute: graph launch");
}

MDT_API mdt_status mdt_fx_batch_check(mdt_fx_batch b)
{
    if (!b) return mdt::invalid("fx_batch_check: null batch");
    mdt_status st = mdt::cuda_status(cudaStreamSynchronize(b->stream), "fx_batch_check");
    if (st != MDT_SUCCESS) return st;
    int flag = 0;
    st = mdt::cuda_status(cudaMemcpy(&flag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost),
                          "fx_batch_check");
    if (st != MDT_SUCCESS) return st;
    if (flag) {
        cudaMemset(b->d_err, 0, sizeof(int));
        mdt::set_error("fx_batch_check: a device-side wait timed out");
        return MDT_ERR_TIMEOUT;
    }
    return MDT_SUCCESS;
}

}  // extern "C"
