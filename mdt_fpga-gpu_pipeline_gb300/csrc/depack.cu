// depack.cu -- GPU depacketiser: SNAP packets -> [spectrum][element][channel]
// samples, with packet-gap detection.
//
// Replaces the host loop of the reference client's rank 1
// (MDT_OneStation_client.cu:846-907).  A packet is `words_header` 32-bit
// header words -- [0] station, [1] SNAP board, [2] packet counter -- then
// `sper_element` samples for each of InputsPerSNAP[snap] inputs, sample-major
// (payload sample (i, j) = input j of sample i).  Element-sample index of
// sample i is counter * sper_element + i; its spectrum is index / Nch and its
// channel index % Nch.  Element = station * inputs_per_station +
// sum_{k < snap} InputsPerSNAP[k] + j.
//
// Samples are either the reference's int32 fixed point (two words, re and im,
// scaled by 2^-19 into complex64) or int8 I/Q pairs (two bytes, copied to the
// int8 I/Q layout of the fused path).  The int32 conversion follows the
// reference bit for bit, including its mapping of 0x80000000 to +4096.0
// (the reference negates 2^32 - w through an int, which wraps for w = 2^31).
//
// The output window is element-samples [sample0, sample0 + nspectra * Nch)
// (sample0 a multiple of Nch); packets outside it are counted and skipped.
// Arrivals are counted per (station, SNAP, packet slot) in `seen`; the finish
// step zero-fills the samples of slots that never arrived, counts them, and
// clears `seen` for the next window.
#include <algorithm>

#include "mdt_common.cuh"

namespace mdt {

struct DepackGeom {
    int hdr_words, sper, ips, nsnap, nstation, bits;
    long pkt_bytes;
    int ne, nch, nspectra;
    long long sample0, c0;  // first packet counter touching the window
    long nslots;
    int snap_off[MDT_MAX_SNAPS + 1];
    int snap_n[MDT_MAX_SNAPS];
};

__device__ __forceinline__ float fixed19_to_float(uint32_t w)
{
    // reference: w >= 2^31 -> -2^-19 * (int)(2^32 - w), else 2^-19 * (int)w,
    // both in double, then rounded to float.
    if (w == 0x80000000u) return 4096.0f;
    return __int2float_rn((int)w) * 1.9073486328125e-06f;
}

__global__ void depacketise_kernel(DepackGeom g, const unsigned char *__restrict__ pkts,
                                   void *__restrict__ out, unsigned int *__restrict__ seen,
                                   mdt_depack_stats *__restrict__ stats)
{
    const unsigned char *p = pkts + (long)blockIdx.x * g.pkt_bytes;
    const uint32_t *hdr = (const uint32_t *)p;
    const uint32_t station = hdr[0], snap = hdr[1], counter = hdr[2];
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        if (snap >= (uint32_t)g.nsnap || station >= (uint32_t)g.nstation ||
            (long)station * g.ips + g.snap_off[snap] + g.snap_n[snap] > g.ne) {
            atomicAdd(&stats->bad, 1ull);
            ok = 0;
        } else {
            const long long slot = (long long)counter - g.c0;
            if (slot < 0 || slot >= g.nslots) {
                atomicAdd(&stats->outside, 1ull);
                ok = 0;
            } else {
                const unsigned int prev =
                    atomicAdd(&seen[((long)station * g.nsnap + snap) * g.nslots + slot], 1u);
                if (prev) atomicAdd(&stats->duplicate, 1ull);
                atomicAdd(&stats->accepted, 1ull);
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) return;
    const int nin = g.snap_n[snap];
    const long elem0 = (long)station * g.ips + g.snap_off[snap];
    const long long first = (long long)counter * g.sper - g.sample0;
    const long long wlen = (long long)g.nspectra * g.nch;
    const int total = g.sper * nin;
    // consecutive threads take consecutive samples of one input, so the
    // stores run along channels
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int j = idx / g.sper, i = idx - j * g.sper;
        const long long s = first + i;
        if (s < 0 || s >= wlen) continue;
        const long long spec = s / g.nch;
        const int chan = (int)(s - spec * g.nch);
        const long o = ((long)spec * g.ne + elem0 + j) * g.nch + chan;
        if (g.bits == 32) {
            const uint32_t *w = hdr + g.hdr_words + 2 * (i * nin + j);
            ((float2 *)out)[o] = make_float2(fixed19_to_float(w[0]), fixed19_to_float(w[1]));
        } else {
            const char2 *w = (const char2 *)(p + 4 * g.hdr_words) + (i * nin + j);
            ((char2 *)out)[o] = *w;
        }
    }
}

// One thread per (station, SNAP, slot): zero-fill slots that never arrived,
// count them, clear the arrival counts.
__global__ void depack_finish_kernel(DepackGeom g, void *__restrict__ out,
                                     unsigned int *__restrict__ seen,
                                     mdt_depack_stats *__restrict__ stats)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long ngrp = (long)g.nstation * g.nsnap;
    if (t >= ngrp * g.nslots) return;
    const long grp = t / g.nslots, slot = t - grp * g.nslots;
    const int station = (int)(grp / g.nsnap), snap = (int)(grp - (long)station * g.nsnap);
    const long elem0 = (long)station * g.ips + g.snap_off[snap];
    const int nin = g.snap_n[snap];
    const unsigned int n = seen[t];
    seen[t] = 0;
    if (n || elem0 + nin > g.ne || nin == 0) return;
    atomicAdd(&stats->missing, 1ull);
    const long long first = (g.c0 + slot) * g.sper - g.sample0;
    const long long wlen = (long long)g.nspectra * g.nch;
    for (int i = 0; i < g.sper; i++) {
        const long long s = first + i;
        if (s < 0 || s >= wlen) continue;
        const long long spec = s / g.nch;
        const int chan = (int)(s - spec * g.nch);
        for (int j = 0; j < nin; j++) {
            const long o = ((long)spec * g.ne + elem0 + j) * g.nch + chan;
            if (g.bits == 32)
                ((float2 *)out)[o] = make_float2(0.f, 0.f);
            else
                ((char2 *)out)[o] = make_char2(0, 0);
        }
    }
}

static mdt_status make_geom(const mdt_packet_format *f, int ne, int nch, long long sample0,
                            int nspectra, DepackGeom *g)
{
    if (!f) return invalid("depacketise: null packet format");
    if (f->words_header < 3 || f->sper_element < 1 || f->inputs_per_station < 1 ||
        f->nsnap < 1 || f->nsnap > MDT_MAX_SNAPS || (f->sample_bits != 32 && f->sample_bits != 8))
        return invalid("depacketise: bad packet format");
    if (ne < 1 || nch < 1 || nspectra < 1 || sample0 < 0 || sample0 % nch)
        return invalid("depacketise: bad window (sample0 must be a multiple of Nch)");
    g->hdr_words = f->words_header;
    g->sper = f->sper_element;
    g->ips = f->inputs_per_station;
    g->nsnap = f->nsnap;
    g->bits = f->sample_bits;
    int off = 0, maxn = 0;
    for (int k = 0; k < f->nsnap; k++) {
        if (f->inputs_per_snap[k] < 0) return invalid("depacketise: negative inputs_per_snap");
        g->snap_off[k] = off;
        g->snap_n[k] = f->inputs_per_snap[k];
        off += f->inputs_per_snap[k];
        maxn = std::max(maxn, f->inputs_per_snap[k]);
    }
    g->snap_off[f->nsnap] = off;
    if (off > f->inputs_per_station) return invalid("depacketise: SNAP inputs exceed a station");
    const long need = 4L * f->words_header +
                      (long)f->sper_element * maxn * (f->sample_bits == 32 ? 8 : 2);
    g->pkt_bytes = f->packet_bytes;
    if (g->pkt_bytes < need || g->pkt_bytes % 4)
        return invalid("depacketise: packet_bytes smaller than the largest packet or not a "
                       "multiple of 4");
    g->ne = ne;
    g->nch = nch;
    g->nspectra = nspectra;
    g->sample0 = sample0;
    g->nstation = (int)cdiv(ne, f->inputs_per_station);
    const long long end = sample0 + (long long)nspectra * nch;
    g->c0 = sample0 / f->sper_element;
    g->nslots = (long)((end + f->sper_element - 1) / f->sper_element - g->c0);
    return MDT_SUCCESS;
}

}  // namespace mdt

extern "C" {

MDT_API mdt_status mdt_depacketise_seen_words(const mdt_packet_format *fmt, int ne, int nch,
                                              long long sample0, int nspectra, size_t *words)
{
    mdt::DepackGeom g;
    mdt_status st = mdt::make_geom(fmt, ne, nch, sample0, nspectra, &g);
    if (st != MDT_SUCCESS) return st;
    if (!words) return mdt::invalid("depacketise_seen_words: null output");
    *words = (size_t)g.nstation * g.nsnap * g.nslots;
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_depacketise(const mdt_packet_format *fmt, const void *packets, int npackets,
                                   int ne, int nch, long long sample0, int nspectra, void *out,
                                   unsigned int *seen, mdt_depack_stats *stats,
                                   cudaStream_t stream)
{
    mdt::DepackGeom g;
    mdt_status st = mdt::make_geom(fmt, ne, nch, sample0, nspectra, &g);
    if (st != MDT_SUCCESS) return st;
    if (npackets < 0 || (npackets && !packets) || !out || !seen || !stats)
        return mdt::invalid("depacketise: bad buffers");
    if (npackets == 0) return MDT_SUCCESS;
    if (((uintptr_t)packets & 3) || ((uintptr_t)out & (fmt->sample_bits == 32 ? 7 : 1)))
        return mdt::invalid("depacketise: misaligned packets or output");
    mdt::depacketise_kernel<<<(unsigned)npackets, 128, 0, stream>>>(
        g, (const unsigned char *)packets, out, seen, stats);
    return mdt::launch_status("depacketise_kernel");
}

MDT_API mdt_status mdt_depacketise_finish(const mdt_packet_format *fmt, int ne, int nch,
                                          long long sample0, int nspectra, void *out,
                                          unsigned int *seen, mdt_depack_stats *stats,
                                          cudaStream_t stream)
{
    mdt::DepackGeom g;
    mdt_status st = mdt::make_geom(fmt, ne, nch, sample0, nspectra, &g);
    if (st != MDT_SUCCESS) return st;
    if (!out || !seen || !stats) return mdt::invalid("depacketise_finish: bad buffers");
    const long n = (long)g.nstation * g.nsnap * g.nslots;
    mdt::depack_finish_kernel<<<(unsigned)mdt::cdiv(n, 128), 128, 0, stream>>>(g, out, seen,
                                                                              stats);
    return mdt::launch_status("depack_finish_kernel");
}

}  // extern "C"
