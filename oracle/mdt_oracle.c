/*
 * mdt_oracle.c -- the oracle: a plain-C CPU restatement of the reference's
 * GPU FX correlator hot path (aragorn2101/MDT_FPGA-GPU_pipeline), used ONLY to
 * check results in tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg. The product library never links, loads or calls it.
 *
 * Parity pins: the bit-exact functions (pps_f32_exact, reorder_c64) are checked
 * against the reference kernels themselves, compiled from the reference
 * sources for the CPU (oracle/build_ref.sh) and captured as golden fixtures in
 * tests/golden/. The FFT and X-engine restate the cuFFT / cuBLAS contracts
 * the reference calls (closed libraries, no golden vectors in the reference);
 * they are pinned against numpy's FFT and einsum and a naive DFT.
 *
 * Build: cc -O3 -fopenmp -ffp-contract=off -shared -fPIC (oracle/oracle.py).
 * -ffp-contract=off keeps every a*b+c as a rounded multiply and a rounded
 * add, except where fmaf() is written explicitly (PpS_Batch's own order).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define REAL double
#define SUFFIX _f64
#include "mdt_oracle_core.h"
#undef REAL
#undef SUFFIX

#define REAL float
#define SUFFIX _f32
#include "mdt_oracle_core.h"
#undef REAL
#undef SUFFIX

/* ---------------------------------------------------------------- windows */

/* Minimum 4-term Blackman-Harris windowed sinc, evaluated in double:
 *   W[n] = sinc((n - Ntaps*Nch/2)/Nch) * (0.35875 - 0.48829 cos(2 pi n/L)
 *          + 0.14128 cos(4 pi n/L) - 0.01168 cos(6 pi n/L)),  L = Ntaps*Nch
 * following PFB_Window_min4term_BH, MDT_device_functions.cu:52-88
 * (argument conventions kept: sinc centre at L/2, cos argument 2n/L in
 * units of pi). */
void mdt_oracle_window_bh4(int nch, int ntaps, double *w)
{
    long L = (long)ntaps * nch;
    for (long n = 0; n < L; n++) {
        double t1 = ((double)n - 0.5 * (double)L) / (double)nch;
        double f = (t1 == 0.0) ? 1.0 : sin(M_PI * t1) / (M_PI * t1);
        double t2 = 2.0 * (double)n / (double)L;
        double win = 0.35875 - 0.48829 * cos(M_PI * t2) + 0.14128 * cos(2.0 * M_PI * t2)
                     - 0.01168 * cos(3.0 * M_PI * t2);
        w[n] = f * win;
    }
}

/* Hamming windowed sinc used by the benchmark configurations, same argument
 * conventions as the Blackman-Harris generator above:
 *   W[n] = sinc((n - L/2)/Nch) * (0.54 - 0.46 cos(2 pi n / L)),  L = Ntaps*Nch
 * evaluated in double and rounded once to float. */
void mdt_oracle_window_hamming_sinc(int nch, int ntaps, float *w)
{
    long L = (long)ntaps * nch;
    for (long n = 0; n < L; n++) {
        double t1 = ((double)n - 0.5 * (double)L) / (double)nch;
        double f = (t1 == 0.0) ? 1.0 : sin(M_PI * t1) / (M_PI * t1);
        double win = 0.54 - 0.46 * cos(2.0 * M_PI * (double)n / (double)L);
        w[n] = (float)(f * win);
    }
}

/* ------------------------------------------------- bit-exact restatements */

/* PpS_Batch (MDT_device_functions.cu:113-161) in float with the kernel's own
 * operation order: per output, tmp = 0; for i in 0..Ntaps-1:
 *   tmp.x = fmaf(W[i*Nch+c], In[s+i][e][c].x, tmp.x)   (likewise .y)
 * Input spectra s+i, output spectrum s, element stride Nch, spectrum stride
 * NE*Nch (:177-183). Bit-identical to the reference kernel on any IEEE GPU. */
void mdt_oracle_pps_f32_exact(int nch, int ntaps, int ne, int nsp, const float *win,
                              const float *in, float *out)
{
    #pragma omp parallel for schedule(static)
    for (long row = 0; row < (long)nsp * ne; row++) {
        long s = row / ne, e = row % ne;
        for (int c = 0; c < nch; c++) {
            float re = 0.0f, im = 0.0f;
            for (int i = 0; i < ntaps; i++) {
                const float *p = in + 2 * (((s + i) * ne + e) * (long)nch + c);
                float w = win[(long)i * nch + c];
                re = fmaf(w, p[0], re);
                im = fmaf(w, p[1], im);
            }
            out[2 * (row * nch + c)] = re;
            out[2 * (row * nch + c) + 1] = im;
        }
    }
}

/* ReorderFOutput (MDT_device_functions.cu:183-208) index map, moving 8-byte
 * complex values:  X[(c*Nsp + s)*NE + e] = F[(s*NE + e)*Nch + c]. */
void mdt_oracle_reorder_c64(int ne, int nch, int nsp, const uint64_t *F, uint64_t *X)
{
    #pragma omp parallel for schedule(static)
    for (long s = 0; s < nsp; s++)
        for (long e = 0; e < ne; e++)
            for (long c = 0; c < nch; c++)
                X[(c * nsp + s) * ne + e] = F[(s * ne + e) * nch + c];
}

/* ------------------------------------------------ integer X-engine oracle */

/* Integer visibilities on an int8 I/Q X-engine input laid out channel-major,
 * time-major, element-fastest: X[((c*nsp + s)*ne + e)][2] (the
 * ReorderFOutput layout with int8 components).  Exact int64 sums of
 *   Re V[r,q] = sum_s xr_r xr_q + xi_r xi_q,   Im V[r,q] = sum_s xi_r xr_q - xr_r xi_q
 * stored column-major per channel: V[c][q*ne + r][2]. No 1/Nsp scale. */
void mdt_oracle_xengine_i8(int ne, int nch, int nsp, const int8_t *X, int64_t *V)
{
    #pragma omp parallel for schedule(dynamic, 1)
    for (int c = 0; c < nch; c++) {
        int64_t *vc = V + 2 * (size_t)c * ne * ne;
        memset(vc, 0, sizeof(int64_t) * 2 * (size_t)ne * ne);
        for (int s = 0; s < nsp; s++) {
            const int8_t *xs = X + 2 * ((size_t)c * nsp + s) * ne;
            for (int q = 0; q < ne; q++) {
                int64_t qr = xs[2 * q], qi = xs[2 * q + 1];
                int64_t *vq = vc + 2 * (size_t)q * ne;
                for (int r = 0; r < ne; r++) {
                    int64_t rr = xs[2 * r], ri = xs[2 * r + 1];
                    vq[2 * r] += rr * qr + ri * qi;
                    vq[2 * r + 1] += ri * qr - rr * qi;
                }
            }
        }
    }
}

/* ------------------------------------------------ synthetic int8 I/Q input */

/* splitmix64 output function (S. Vigna's published SplitMix64 finaliser). */
static inline uint64_t mdt_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Approximately N(0, 37836.9^2) integer: sum of four 16-bit uniforms minus
 * their mean (Irwin-Hall).  Key = (time, stream, component). */
static inline int64_t mdt_gauss_int(uint64_t seed, int64_t t, int stream, int comp)
{
    uint64_t key = ((uint64_t)t << 14) | ((uint64_t)stream << 1) | (uint64_t)comp;
    uint64_t h = mdt_mix64(mdt_mix64(key) ^ seed);
    int64_t z = (int64_t)(h & 0xFFFF) + (int64_t)((h >> 16) & 0xFFFF) +
                (int64_t)((h >> 32) & 0xFFFF) + (int64_t)(h >> 48);
    return z - 131070;
}

/* Deterministic integer-only int8 I/Q generator shared bit-for-bit with the
 * GPU generator and tests/golden/synth.py:
 *   sample(e, t) = clip(round(( z_e(t)*sigma_e + sum_k z_k(t - d_k,e)*sigma_k ) / (256*37836.9)
 *                             + tone_e(t mod Nch)), -127, 127)
 * in Q16 fixed point with M = 113512 ~ 2^40/(256*37836.9), an arithmetic
 * shift (floor), and round-half-up.  Layout out[(s*NE + e)*Nch + c][2] for
 * spectra s0 .. s0+nsp-1, time t = s*Nch + c (the depacketiser's sample
 * index, MDT_OneStation_client.cu:852-858).
 *   sigma_q8[ne]           noise sigma in 1/256 LSB
 *   tone_q16[ne*nch*2]     tone table in Q16 LSB (may be NULL)
 *   nsrc, src_sigma_q8[nsrc], src_delay[nsrc*ne]  common sources, delays in samples */
void mdt_oracle_synth_iq(uint64_t seed, int ne, int nch, long s0, long nsp,
                         const int32_t *sigma_q8, const int32_t *tone_q16,
                         int nsrc, const int32_t *src_sigma_q8, const int32_t *src_delay,
                         int8_t *out)
{
    const int64_t M = 113512;
    #pragma omp parallel for schedule(static)
    for (long row = 0; row < nsp * ne; row++) {
        long s = s0 + row / ne;
        int e = (int)(row % ne);
        for (int c = 0; c < nch; c++) {
            int64_t t = (int64_t)s * nch + c;
            for (int comp = 0; comp < 2; comp++) {
                int64_t num = mdt_gauss_int(seed, t, e, comp) * sigma_q8[e];
                for (int k = 0; k < nsrc; k++)
                    num += mdt_gauss_int(seed, t - src_delay[k * ne + e], 4096 + k, comp) *
                           src_sigma_q8[k];
                int64_t v = (num * M) >> 24;
                if (tone_q16) v += tone_q16[2 * ((size_t)e * nch + c) + comp];
                v = (v + 32768) >> 16;
                if (v > 127) v = 127;
                if (v < -127) v = -127;
                out[2 * ((size_t)row * nch + c) + comp] = (int8_t)v;
            }
        }
    }
}

/* ------------------------------------------------------------------------
 * Depacketiser, restating the reference client's rank-1 loop
 * (MDT_OneStation_client.cu:846-907) over a window of element-samples
 * [sample0, sample0 + nspectra*nch) instead of its two Nspectra stacks.
 * Packets are processed in order; samples outside the window are skipped.
 * sample_bits 32: two uint32 words per sample, the reference's conversion
 * (MDT_OneStation_client.cu:896-907): w >= 2^31 -> -(2^-19) * (int)(2^32 - w)
 * in double (2^32 - w wraps to INT_MIN through the int for w = 2^31, giving
 * +4096), else (2^-19) * (int)w; rounded to float.  sample_bits 8: int8 pairs
 * copied.  stats[0..2] += accepted, outside, bad.  Returns 0. */
static float mdt_fixed19(uint32_t w)
{
    const double lsb = 1.0 / 524288.0; /* 2^-19 */
    double d;
    if (w >= 0x80000000u) {
        int32_t m = (int32_t)(uint32_t)(0x100000000ULL - (uint64_t)w); /* wraps at w = 2^31 */
        d = -lsb * (double)m;
    } else {
        d = lsb * (double)(int32_t)w;
    }
    return (float)d;
}

int mdt_oracle_depacketise(int words_header, int sper, int ips, int nsnap,
                           const int *inputs_per_snap, int sample_bits, long packet_bytes,
                           const unsigned char *pkts, int npkt, int ne, int nch,
                           long long sample0, int nspectra, void *out, long long *stats)
{
    const int nstation = (ne + ips - 1) / ips;
    const long long wlen = (long long)nspectra * nch;
    for (int p = 0; p < npkt; p++) {
        const unsigned char *pk = pkts + (long)p * packet_bytes;
        uint32_t hdr[3];
        memcpy(hdr, pk, sizeof hdr);
        if (hdr[1] >= (uint32_t)nsnap || hdr[0] >= (uint32_t)nstation) {
            stats[2]++;
            continue;
        }
        long elem0 = (long)hdr[0] * ips;
        for (uint32_t k = 0; k < hdr[1]; k++) elem0 += inputs_per_snap[k];
        const int nin = inputs_per_snap[hdr[1]];
        if (elem0 + nin > ne) {
            stats[2]++;
            continue;
        }
        const long long first = (long long)hdr[2] * sper;
        if (first + sper <= sample0 || first >= sample0 + wlen) {
            stats[1]++;
            continue;
        }
        stats[0]++;
        for (int i = 0; i < sper; i++) {
            const long long s = first + i - sample0;
            if (s < 0 || s >= wlen) continue;
            const long long spec = s / nch, chan = s % nch;
            for (int j = 0; j < nin; j++) {
                const long o = ((long)spec * ne + elem0 + j) * nch + chan;
                const long b = 4L * words_header;
                if (sample_bits == 32) {
                    uint32_t w[2];
                    memcpy(w, pk + b + 8L * ((long)i * nin + j), sizeof w);
                    ((float *)out)[2 * o] = mdt_fixed19(w[0]);
                    ((float *)out)[2 * o + 1] = mdt_fixed19(w[1]);
                } else {
                    memcpy((int8_t *)out + 2 * o, pk + b + 2L * ((long)i * nin + j), 2);
                }
            }
        }
    }
    return 0;
}
