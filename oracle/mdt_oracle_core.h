/*
 * mdt_oracle_core.h -- CPU restatement of the MDT FX correlator hot path,
 * written once over a scalar type and instantiated twice by mdt_oracle.c:
 *   REAL=double  -> the FP64 oracle (suffix _f64), the correctness reference;
 *   REAL=float   -> the FP32 OpenMP CPU pipeline (suffix _f32), the timed CPU
 *                   baseline.
 *
 * TEST INFRASTRUCTURE ONLY: nothing in the product library links or calls this.
 *
 * The stages follow the reference sequence (MDT_OneStation_client.cu:1083-1128):
 *   PpS_Batch (MDT_device_functions.cu:113-161)   -> pps()
 *   cufftExecC2C forward, unnormalised (:1105)    -> fft_rows()
 *   ReorderFOutput (MDT_device_functions.cu:183)  -> folded into the X stage
 *   cublasCgemmBatched(N, C, alpha=1/Nspectra)    -> xengine()
 *     (MDT_OneStation_client.cu:1128, alpha at :683-686)
 *
 * Layouts (all complex values interleaved re,im):
 *   input  int8 I/Q  in[(s*NE + e)*Nch + c][2],  s in [0, Nsp+Ntaps-1)
 *   window float     W[i*Nch + c]  (tap-major, MDT_device_functions.cu:147)
 *   visibilities     V[k][q*NE + r] = alpha * sum_s X_c[s][r] * conj(X_c[s][q])
 *                    (column-major NE x NE per selected channel k, the cuBLAS
 *                    C-matrix layout with ldc=NE, MDT_OneStation_client.cu:1128)
 */

#define CAT2_(a, b) a##b
#define CAT2(a, b) CAT2_(a, b)
#define FN(name) CAT2(name, SUFFIX)

/* Forward, unnormalised, natural-order radix-2 FFT of one row of n complex
 * values (n a power of two), sign convention e^{-2 pi i k m / n} as cuFFT's
 * CUFFT_FORWARD.  tw[k] = exp(-2 pi i k / n) for k < n/2. */
static void FN(fft_row)(int n, int logn, REAL *x, const REAL *tw)
{
    /* bit reversal permutation */
    for (int i = 0; i < n; i++) {
        unsigned r = 0, v = (unsigned)i;
        for (int b = 0; b < logn; b++) { r = (r << 1) | (v & 1u); v >>= 1; }
        if ((int)r > i) {
            REAL t0 = x[2 * i], t1 = x[2 * i + 1];
            x[2 * i] = x[2 * r]; x[2 * i + 1] = x[2 * r + 1];
            x[2 * r] = t0; x[2 * r + 1] = t1;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int base = 0; base < n; base += len) {
            for (int j = 0; j < half; j++) {
                REAL wr = tw[2 * (j * step)], wi = tw[2 * (j * step) + 1];
                REAL *a = x + 2 * (base + j), *b = x + 2 * (base + j + half);
                REAL br = b[0] * wr - b[1] * wi;
                REAL bi = b[0] * wi + b[1] * wr;
                b[0] = a[0] - br; b[1] = a[1] - bi;
                a[0] = a[0] + br; a[1] = a[1] + bi;
            }
        }
    }
}

static int FN(ilog2)(int n)
{
    int l = 0;
    while ((1 << l) < n) l++;
    return ((1 << l) == n) ? l : -1;
}

/* Twiddle table exp(-2 pi i k / n), k < n/2, evaluated in double. */
static REAL *FN(make_twiddles)(int n)
{
    REAL *tw = (REAL *)malloc(sizeof(REAL) * (size_t)n);
    for (int k = 0; k < n / 2; k++) {
        double a = -2.0 * M_PI * (double)k / (double)n;
        tw[2 * k] = (REAL)cos(a);
        tw[2 * k + 1] = (REAL)sin(a);
    }
    return tw;
}

/* Batched forward FFT of `rows` contiguous rows of n complex values, in place
 * (the cufftPlan1d(n, C2C, rows) + cufftExecC2C(FORWARD) contract,
 * MDT_OneStation_client.cu:622,1105). Returns 0, or -1 if n is not 2^k. */
int FN(mdt_oracle_fft_rows)(long rows, int n, REAL *data)
{
    int logn = FN(ilog2)(n);
    if (logn < 0) return -1;
    REAL *tw = FN(make_twiddles)(n);
    #pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; r++) FN(fft_row)(n, logn, data + 2 * (size_t)n * r, tw);
    free(tw);
    return 0;
}

/* Full FX pipeline from int8 I/Q to visibilities for a subset of channels.
 *   ne, nch, ntaps, nsp : elements (Npol*Nelements), channels, taps, spectra
 *   in   : int8 I/Q, (nsp + ntaps - 1) spectra, layout above
 *   win  : float window, ntaps*nch, tap-major
 *   nsel, sel : channel list (sel == NULL -> all nch channels, nsel ignored)
 *   V    : out, nsel x ne x ne complex REAL, column-major per channel,
 *          scaled by 1/nsp (cublas alpha, MDT_OneStation_client.cu:683)
 * The reference's order, in chunks of spectra: the F-engine rows (PFB tap
 * sum, FFT) of every (spectrum, element) of the chunk, the selected channels
 * kept channel-major (the ReorderFOutput layout restricted to them); then the
 * per-channel products, each visibility summed over the spectra in increasing
 * order whatever the thread count (deterministic).  Only the lower triangle
 * r >= q is summed: the upper one is its conjugate, which is what the full
 * square gives bit for bit (the two products of a pair are the same
 * roundings with the imaginary part negated). */
int FN(mdt_oracle_fx)(int ne, int nch, int ntaps, int nsp, const int8_t *in,
                      const float *win, int nsel, const int *sel, REAL *V)
{
    int logn = FN(ilog2)(nch);
    if (logn < 0 || ne <= 0 || ntaps <= 0 || nsp <= 0) return -1;
    int *chan = NULL;
    if (sel == NULL) {
        nsel = nch;
        chan = (int *)malloc(sizeof(int) * (size_t)nch);
        for (int k = 0; k < nch; k++) chan[k] = k;
    } else {
        chan = (int *)malloc(sizeof(int) * (size_t)nsel);
        for (int k = 0; k < nsel; k++) {
            if (sel[k] < 0 || sel[k] >= nch) { free(chan); return -2; }
            chan[k] = sel[k];
        }
    }
    REAL *tw = FN(make_twiddles)(nch);
    const size_t vlen = (size_t)nsel * ne * ne * 2;
    memset(V, 0, sizeof(REAL) * vlen);
    const size_t row = (size_t)nch * 2;
    const size_t per_s = (size_t)nsel * ne * 2; /* REALs of selected F-output per spectrum */
    long chunk = (long)(((size_t)1 << 25) / per_s);
    if (chunk < 1) chunk = 1;
    if (chunk > nsp) chunk = nsp;
    REAL *xs = (REAL *)malloc(sizeof(REAL) * per_s * (size_t)chunk);
    const int qb = 16; /* columns per product task */
    const int nqb = (ne + qb - 1) / qb;

    for (long s0 = 0; s0 < nsp; s0 += chunk) {
        const long ns = (nsp - s0 < chunk) ? nsp - s0 : chunk;
        #pragma omp parallel
        {
            REAL *x = (REAL *)malloc(sizeof(REAL) * row);
            #pragma omp for schedule(static)
            for (long rr = 0; rr < ns * ne; rr++) {
                const long t = rr / ne, s = s0 + t;
                const int e = (int)(rr % ne);
                /* polyphase sum, tap i applied to spectrum s+i
                 * (MDT_device_functions.cu:143-152) */
                for (int c = 0; c < nch; c++) {
                    REAL re = 0, im = 0;
                    for (int i = 0; i < ntaps; i++) {
                        const int8_t *p = in + 2 * (((size_t)(s + i) * ne + e) * nch + c);
                        REAL w = (REAL)win[(size_t)i * nch + c];
                        re += w * (REAL)p[0];
                        im += w * (REAL)p[1];
                    }
                    x[2 * c] = re; x[2 * c + 1] = im;
                }
                FN(fft_row)(nch, logn, x, tw);
                for (int k = 0; k < nsel; k++) {
                    REAL *d = xs + 2 * (((size_t)k * ns + t) * ne + e);
                    d[0] = x[2 * chan[k]];
                    d[1] = x[2 * chan[k] + 1];
                }
            }
            free(x);
        }
        /* V_c[r + q*ne] += X[r] * conj(X[q]) (cublas OP_N x OP_C), r >= q */
        #pragma omp parallel for schedule(dynamic, 1)
        for (long task = 0; task < (long)nsel * nqb; task++) {
            const int k = (int)(task / nqb), q0 = (int)(task % nqb) * qb;
            const int q1 = (q0 + qb < ne) ? q0 + qb : ne;
            REAL *vk = V + 2 * (size_t)k * ne * ne;
            for (long t = 0; t < ns; t++) {
                const REAL *xk = xs + 2 * ((size_t)k * ns + t) * ne;
                for (int q = q0; q < q1; q++) {
                    const REAL qr = xk[2 * q], qi = xk[2 * q + 1];
                    REAL *vq = vk + 2 * (size_t)q * ne;
                    for (int r = q; r < ne; r++) {
                        const REAL rr = xk[2 * r], ri = xk[2 * r + 1];
                        vq[2 * r] += rr * qr + ri * qi;
                        vq[2 * r + 1] += ri * qr - rr * qi;
                    }
                }
            }
        }
    }
    const REAL scale = (REAL)1 / (REAL)nsp;
    #pragma omp parallel for schedule(static)
    for (long k = 0; k < nsel; k++) {
        REAL *vk = V + 2 * (size_t)k * ne * ne;
        for (int q = 0; q < ne; q++)
            for (int r = q; r < ne; r++) {
                REAL *lo = vk + 2 * ((size_t)q * ne + r), *up = vk + 2 * ((size_t)r * ne + q);
                lo[0] *= scale;
                lo[1] *= scale;
                up[0] = lo[0];
                up[1] = -lo[1];
            }
    }
    free(xs);
    free(tw);
    free(chan);
    return 0;
}

/* X-engine alone on a channel-major complex input X[c][s][e] (the
 * ReorderFOutput output layout, MDT_device_functions.cu:207):
 * V[c][q*ne + r] = alpha * sum_s X[c][s][r] conj(X[c][s][q]). */
void FN(mdt_oracle_xengine)(int ne, int nch, int nsp, const REAL *X, REAL alpha, REAL *V)
{
    #pragma omp parallel for schedule(dynamic, 1)
    for (int c = 0; c < nch; c++) {
        const REAL *xc = X + 2 * (size_t)c * nsp * ne;
        REAL *vc = V + 2 * (size_t)c * ne * ne;
        for (size_t j = 0; j < 2 * (size_t)ne * ne; j++) vc[j] = 0;
        for (int s = 0; s < nsp; s++) {
            const REAL *xs = xc + 2 * (size_t)s * ne;
            for (int q = 0; q < ne; q++) {
                REAL qr = xs[2 * q], qi = xs[2 * q + 1];
                REAL *vq = vc + 2 * (size_t)q * ne;
                for (int r = 0; r < ne; r++) {
                    REAL rr = xs[2 * r], ri = xs[2 * r + 1];
                    vq[2 * r] += rr * qr + ri * qi;
                    vq[2 * r + 1] += ri * qr - rr * qi;
                }
            }
        }
        for (size_t j = 0; j < 2 * (size_t)ne * ne; j++) vc[j] *= alpha;
    }
}

#undef FN
