// output.cu -- output formatter: visibilities -> the reference's output order,
// and streaming CSV / binary writers.
//
// The reference client writes, per integration, one CSV line per (baseline,
// channel) (MDT_OneStation_client.cu:1239-1266):
//   for j < Nelements, p < Npols, k = j..Nelements-1, q = p..Npols-1,
//     for z = 0..Nch-1 (channel i = (z + Nch/2) % Nch: fftshift, negative
//     frequencies first):
//       "%ld,%d,%ld,%d,%ld,%.6f,%.6f\n"  j, p, k, q, z, Re, Im
//   of V[i][(k*Npols + q)*NE + (j*Npols + p)]  (column-major, row = first
//   element, conjugate on the second).
// mdt_format_baselines does the gather on the GPU into a baseline-major
// buffer out[bl][z] (complex64), so the host only streams it out.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "mdt_common.cuh"

namespace mdt {

// Baseline index of (j, p, k, q), k >= j, q >= p, in the reference's loop order.
__host__ __device__ __forceinline__ long baseline_index(long nel, long np, long j, long p, long k,
                                                        long q)
{
    const long T = np * (np + 1) / 2;
    return T * (j * nel - j * (j - 1) / 2) + (nel - j) * (p * np - p * (p - 1) / 2) +
           (k - j) * (np - p) + (q - p);
}

// Block: one column c = k*Np + q, 32 rows r, 32 channels.  Reads run along r
// (contiguous in V), writes along z (contiguous in out).
__global__ void format_baselines_kernel(int nel, int np, int nch, int shift,
                                        const float2 *__restrict__ V, float2 *__restrict__ out)
{
    __shared__ float2 t[32][33];
    const int ne = nel * np;
    const int c = blockIdx.x;
    const int r0 = blockIdx.y * 32;
    const int z0 = blockIdx.z * 32;
    const int k = c / np, q = c - k * np;
    if (r0 > c) return;  // rows past the column hold no baseline (k >= j needs r <= c)
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int z = z0 + y, r = r0 + threadIdx.x;
        float2 v = make_float2(0.f, 0.f);
        if (z < nch && r < ne) {
            const int i = shift ? (z + nch / 2) % nch : z;
            v = V[((long)i * ne + c) * ne + r];
        }
        t[y][threadIdx.x] = v;
    }
    __syncthreads();
    const long nel_l = nel;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, z = z0 + threadIdx.x;
        if (r >= ne || z >= nch) continue;
        const int j = r / np, p = r - j * np;
        if (k < j || q < p) continue;
        const long bl = baseline_index(nel_l, np, j, p, k, q);
        out[bl * nch + z] = t[threadIdx.x][y];
    }
}

// ---------------------------------------------------------------- writers
// "%.6f" of a float, exactly as glibc printf rounds it (round half to even on
// the exact binary value): the value times 10^6 is formed exactly in integer
// arithmetic.  Values of magnitude >= 2^33 and non-finite values go through
// snprintf.  Returns the number of characters written at dst.
static int fmt6(char *dst, float f)
{
    if (!std::isfinite(f) || std::fabs(f) >= 8589934592.0f) return std::snprintf(dst, 64, "%.6f", f);
    uint32_t bits;
    std::memcpy(&bits, &f, 4);
    const bool neg = bits >> 31;
    const int ex = (bits >> 23) & 0xff;
    uint64_t m = bits & 0x7fffff;
    int e;
    if (ex == 0) {
        e = -149;  // subnormal
    } else {
        m |= 0x800000;
        e = ex - 150;
    }
    // value = m * 2^e;  N = round_half_even(m * 10^6 * 2^e)
    uint64_t N;
    const uint64_t num = m * 1000000ull;  // < 2^44
    if (e >= 0) {
        N = num << e;  // |f| < 2^33 keeps this below 2^63
    } else if (-e >= 64) {
        N = 0;
    } else {
        const int s = -e;
        const uint64_t qv = num >> s, rem = num & ((1ull << s) - 1), half = 1ull << (s - 1);
        N = qv + ((rem > half || (rem == half && (qv & 1))) ? 1 : 0);
    }
    char tmp[32];
    int n = 0;
    uint64_t ip = N / 1000000ull, fp = N % 1000000ull;
    for (int d = 0; d < 6; d++) {
        tmp[n++] = char('0' + fp % 10);
        fp /= 10;
    }
    tmp[n++] = '.';
    do {
        tmp[n++] = char('0' + ip % 10);
        ip /= 10;
    } while (ip);
    int w = 0;
    if (neg) dst[w++] = '-';
    while (n) dst[w++] = tmp[--n];
    return w;
}

static int fmt_long(char *dst, long v)
{
    char tmp[24];
    int n = 0;
    bool neg = v < 0;
    unsigned long u = neg ? 0ul - (unsigned long)v : (unsigned long)v;
    do {
        tmp[n++] = char('0' + u % 10);
        u /= 10;
    } while (u);
    int w = 0;
    if (neg) dst[w++] = '-';
    while (n) dst[w++] = tmp[--n];
    return w;
}

struct BlRC {
    long j, p, k, q;
};

static std::vector<BlRC> baseline_list(int nel, int np)
{
    std::vector<BlRC> v;
    for (long j = 0; j < nel; j++)
        for (long p = 0; p < np; p++)
            for (long k = j; k < nel; k++)
                for (long q = p; q < np; q++) v.push_back({j, p, k, q});
    return v;
}

}  // namespace mdt

extern "C" {

MDT_API mdt_status mdt_num_baselines(int nelements, int npols, long *nbl)
{
    if (nelements < 1 || npols < 1 || !nbl) return mdt::invalid("num_baselines: bad arguments");
    *nbl = (long)npols * (npols + 1) / 2 * ((long)nelements * (nelements + 1) / 2);
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_format_baselines(int nelements, int npols, int nch, const void *vis,
                                        void *out, int fftshift, cudaStream_t stream)
{
    if (nelements < 1 || npols < 1 || nch < 1 || !vis || !out || (long)nelements * npols > 65535)
        return mdt::invalid("format_baselines: bad arguments");
    if (fftshift && (nch & 1)) return mdt::invalid("format_baselines: fftshift needs even Nch");
    const int ne = nelements * npols;
    dim3 grid((unsigned)ne, (unsigned)mdt::cdiv(ne, 32), (unsigned)mdt::cdiv(nch, 32));
    if (grid.z > 65535) return mdt::invalid("format_baselines: Nch too large");
    mdt::format_baselines_kernel<<<grid, dim3(32, 8), 0, stream>>>(
        nelements, npols, nch, fftshift ? 1 : 0, (const float2 *)vis, (float2 *)out);
    return mdt::launch_status("format_baselines_kernel");
}

MDT_API mdt_status mdt_write_csv(const char *path, int nelements, int npols, int nch,
                                 const void *formatted, int append, int nthreads)
{
    if (!path || !formatted || nelements < 1 || npols < 1 || nch < 1)
        return mdt::invalid("write_csv: bad arguments");
    FILE *f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return mdt::invalid(std::string("write_csv: cannot open ") + path);
    const std::vector<mdt::BlRC> bls = mdt::baseline_list(nelements, npols);
    const float2 *V = (const float2 *)formatted;
    if (nthreads < 1) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    nthreads = std::min(nthreads, 64);
    // rounds of nthreads chunks, each chunk a run of baselines formatted by one
    // thread, written in order
    const long nbl = (long)bls.size();
    const long per = std::max(1L, (long)((1L << 22) / ((long)nch * 48)));  // ~4 MB of text
    std::vector<std::string> buf(nthreads);
    mdt_status st = MDT_SUCCESS;
    for (long b0 = 0; b0 < nbl && st == MDT_SUCCESS; b0 += per * nthreads) {
        auto work = [&](int t) {
            std::string &s = buf[t];
            s.clear();
            const long lo = b0 + t * per, hi = std::min(nbl, lo + per);
            if (lo >= hi) return;
            s.resize((size_t)(hi - lo) * nch * 200);  // a line is at most ~160 characters
            char *d = &s[0];
            for (long b = lo; b < hi; b++) {
                const mdt::BlRC &e = bls[b];
                char head[96];
                int h = 0;
                h += mdt::fmt_long(head + h, e.j);
                head[h++] = ',';
                h += mdt::fmt_long(head + h, e.p);
                head[h++] = ',';
                h += mdt::fmt_long(head + h, e.k);
                head[h++] = ',';
                h += mdt::fmt_long(head + h, e.q);
                head[h++] = ',';
                for (int z = 0; z < nch; z++) {
                    std::memcpy(d, head, h);
                    d += h;
                    d += mdt::fmt_long(d, z);
                    *d++ = ',';
                    const float2 v = V[b * nch + z];
                    d += mdt::fmt6(d, v.x);
                    *d++ = ',';
                    d += mdt::fmt6(d, v.y);
                    *d++ = '\n';
                }
            }
            s.resize(d - &s[0]);
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
        work(0);
        for (auto &x : th) x.join();
        for (int t = 0; t < nthreads && st == MDT_SUCCESS; t++)
            if (!buf[t].empty() && std::fwrite(buf[t].data(), 1, buf[t].size(), f) != buf[t].size())
                st = mdt::invalid(std::string("write_csv: write failed on ") + path);
    }
    if (std::fclose(f) != 0 && st == MDT_SUCCESS)
        st = mdt::invalid(std::string("write_csv: close failed on ") + path);
    return st;
}

// Binary form: a 32-byte header {"MDTVIS01", int32 nelements, npols, nch,
// nbl, int64 reserved}, int32 [nbl][4] (j, p, k, q), then complex64
// [nbl][Nch] (the formatted buffer).
MDT_API mdt_status mdt_write_binary(const char *path, int nelements, int npols, int nch,
                                    const void *formatted, int append)
{
    if (!path || !formatted || nelements < 1 || npols < 1 || nch < 1)
        return mdt::invalid("write_binary: bad arguments");
    FILE *f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return mdt::invalid(std::string("write_binary: cannot open ") + path);
    const std::vector<mdt::BlRC> bls = mdt::baseline_list(nelements, npols);
    int32_t hdr[8] = {0};
    std::memcpy(hdr, "MDTVIS01", 8);
    hdr[2] = nelements;
    hdr[3] = npols;
    hdr[4] = nch;
    hdr[5] = (int32_t)bls.size();
    std::vector<int32_t> tab(bls.size() * 4);
    for (size_t b = 0; b < bls.size(); b++) {
        tab[4 * b] = (int32_t)bls[b].j;
        tab[4 * b + 1] = (int32_t)bls[b].p;
        tab[4 * b + 2] = (int32_t)bls[b].k;
        tab[4 * b + 3] = (int32_t)bls[b].q;
    }
    const size_t nv = bls.size() * (size_t)nch;
    bool ok = std::fwrite(hdr, sizeof hdr, 1, f) == 1 &&
              std::fwrite(tab.data(), sizeof(int32_t), tab.size(), f) == tab.size() &&
              std::fwrite(formatted, 8, nv, f) == nv;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MDT_SUCCESS : mdt::invalid(std::string("write_binary: write failed on ") + path);
}

}  // extern "C"
