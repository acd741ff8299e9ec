/*
 * mdt_fx.h -- C ABI of the GB300 (sm_103a) MDT FX correlator library
 * (libmdtfx.so).
 *
 * Three groups of entry points, all exported with C linkage, taking plain
 * device pointers, sizes and a cudaStream_t; no entry point aborts, all of
 * them report errors as an mdt_status (or, for the cuFFT / cuBLAS subset, as
 * those libraries' own status codes):
 *
 *  1. Drop-in reference API.  MDT_device_functions.h (this directory) keeps
 *     the reference's three __global__ kernels with their exact signatures
 *     (MDT_device_functions.h:44-46 of the reference); mdt_cufft_cublas_shim.h
 *     declares the cufftPlan1d/cufftSetStream/cufftExecC2C and
 *     cublasCreate/cublasSetStream/cublasCgemmBatched subset that the
 *     reference client calls (MDT_OneStation_client.cu:622,630,1105,690,699,
 *     1128), implemented on this library's own kernels.  The mdt_launch_*
 *     functions below launch the drop-in kernels with a caller-chosen grid,
 *     exactly as the reference client's <<<grid, block, 0, stream>>> does,
 *     for callers (ctypes, other languages) that cannot use <<<>>>.
 *
 *  2. Stage entry points (mdt_fft_*, mdt_xengine_*, mdt_fengine_*): one hot
 *     stage each, on caller-allocated device buffers.
 *
 *  3. The plan API (mdt_fx_*): the fused int8 F-engine + X-engine pipeline
 *     with PFB history carried across integrations.
 *
 * Conventions shared by every entry point
 *   NE      = Npols*Nelements (number of correlator inputs)
 *   Nch     = channels per spectrum (power of two, 32..16384)
 *   Ntaps   = PFB taps (4..128); Nsp = spectra per integration (2..16384)
 *   int8 I/Q input    iq[(s*NE + e)*Nch + c][2]  (I then Q), the reference's
 *                     Spectrum -> Element -> Channel order
 *                     (MDT_device_functions.cu:124-126)
 *   window            W[i*Nch + c], float, tap-major
 *   F-engine output   X[(c*Nsp + s)*NE + e], complex64 (ReorderFOutput layout)
 *   visibilities      V[c][q*NE + r] = (1/Nsp) sum_s X[c][s][r] conj(X[c][s][q]),
 *                     complex64, column-major NE x NE per channel, full square
 *                     (cublasCgemmBatched with OP_N, OP_C, alpha = 1/Nsp,
 *                     MDT_OneStation_client.cu:1128, :683)
 * Complex values are interleaved (re, im) float pairs (cuComplex layout).
 */
#ifndef MDT_FX_H
#define MDT_FX_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MDT_API __attribute__((visibility("default")))
#else
#define MDT_API
#endif

typedef enum {
    MDT_SUCCESS = 0,
    MDT_ERR_INVALID_VALUE = 1, /* a size, pointer or parameter is out of range */
    MDT_ERR_NOT_SUPPORTED = 2, /* valid request this library does not implement */
    MDT_ERR_CUDA = 3,          /* a CUDA runtime call failed; see mdt_last_error */
    MDT_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up */
    MDT_ERR_ALLOC = 5,         /* device or host allocation failed */
    MDT_ERR_STATE = 6          /* call out of order (e.g. no window set) */
} mdt_status;

/* Parameter domain of the reference client (MDT_host_functions.h:39-46). */
#define MDT_MIN_ELEMENTS 3
#define MDT_MAX_ELEMENTS 2048
#define MDT_MIN_CHANNELS 32
#define MDT_MAX_CHANNELS 16384
#define MDT_MIN_TAPS 4
#define MDT_MAX_TAPS 128
#define MDT_MIN_SPECTRA 2
#define MDT_MAX_SPECTRA 16384

/* Library version (major*1000 + minor*10 + patch). */
MDT_API int mdt_version(void);
/* Text of the most recent error on the calling thread ("" if none). */
MDT_API const char *mdt_last_error(void);

/* ------------------------------------------------------------------------
 * 1. Drop-in kernels launched with an explicit grid (as the reference client
 *    launches them).  Each returns MDT_ERR_CUDA if the launch fails.
 * ---------------------------------------------------------------------- */

/* PFB_Window_min4term_BH (reference MDT_device_functions.cu:52-88):
 * W[n] = sinc((n - Ntaps*Nch/2)/Nch) * minimum 4-term Blackman-Harris. */
MDT_API mdt_status mdt_launch_PFB_Window_min4term_BH(unsigned gx, unsigned gy, unsigned gz, unsigned bx,
    unsigned by, unsigned bz, cudaStream_t stream,
                                                     int nchannels, int ntaps, float *window);

/* PpS_Batch (reference MDT_device_functions.cu:113-161), bit-exact:
 * NE = gz, Nsp = gy; input (Nsp+Ntaps-1) spectra of complex64. */
MDT_API mdt_status mdt_launch_PpS_Batch(unsigned gx, unsigned gy, unsigned gz, unsigned bx,
    unsigned by, unsigned bz, cudaStream_t stream, int nchannels,
                                        int ntaps, float *window, void *insignal,
                                        void *polystruct);

/* ReorderFOutput (reference MDT_device_functions.cu:183-208), bit-exact:
 * Nsp = gz; any block shape (the reference needs block (32,32)). */
MDT_API mdt_status mdt_launch_ReorderFOutput(unsigned gx, unsigned gy, unsigned gz, unsigned bx,
    unsigned by, unsigned bz, cudaStream_t stream,
                                             int npolsxnelements, int nchannels, void *foutput,
                                             void *xinput);

/* Hamming windowed sinc of the benchmark configurations (no reference
 * counterpart; the reference's window is an input array to PpS_Batch,
 * MDT_device_functions.cu:113-117):
 *   W[n] = sinc((n - Ntaps*Nch/2)/Nch) * (0.54 - 0.46 cos(2 pi n/(Ntaps*Nch))). */
MDT_API mdt_status mdt_window_hamming_sinc(int nchannels, int ntaps, float *window,
                                           cudaStream_t stream);

/* ------------------------------------------------------------------------
 * 2. Stage entry points
 * ---------------------------------------------------------------------- */

/* Batched unnormalised C2C FFT over `rows` contiguous rows of n complex64
 * (n = 2^k, 2 <= n <= 16384); in place when in == out.  direction -1 is
 * forward (e^{-2 pi i k m/n}), +1 inverse.  Replaces cufftExecC2C
 * (reference MDT_OneStation_client.cu:1105). */
MDT_API mdt_status mdt_fft_c2c(const void *in, void *out, long rows, int n, int direction,
                               cudaStream_t stream);

/* Hermitian X-engine, FP32 SIMT:  for each channel c,
 *   V_c = alpha * X_c X_c^H   (X_c = NE x Nsp column-major with leading
 *   dimension ld >= NE, base X + c*xstride complex values), written full square
 *   column-major with leading dimension NE at V + c*NE*NE.  Only the lower
 *   triangle is computed; the upper is its conjugate mirror and the diagonal
 *   is real.  Replaces cublasCgemmBatched(OP_N, OP_C, A == B)
 *   (reference MDT_OneStation_client.cu:1128). */
MDT_API mdt_status mdt_xengine_f32(int ne, int nch, int nsp, const void *X, long ld,
                                   long xstride, float alpha, void *V, cudaStream_t stream);

/* Fused F-engine, FP32: int8 I/Q -> PFB (fmaf in the reference's tap order)
 * -> FFT -> channel-major complex64 X[(c*Nsp + s)*NE + e].
 * `iq` holds Nsp + Ntaps - 1 spectra.  Bit-identical to PpS_Batch ->
 * cufftExecC2C (this library) -> ReorderFOutput on the same samples.
 * `iq` and `window` must be 16-byte aligned (as are the sample buffers passed
 * to the plan entry points below). */
MDT_API mdt_status mdt_fengine_f32(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                   const float *window, void *X, cudaStream_t stream);

/* Fused F-engine, FP32, into the 8-spectrum blocked layout the plan's FP32
 * path uses:  XB[s/8][c][e][s%8] complex64 (ceil(Nsp/8) blocks, spectra past
 * Nsp zero) -- one 64-byte run per (8 spectra, channel, element).  Same
 * values as mdt_fengine_f32 (bit-identical), Nch <= 2048. */
MDT_API mdt_status mdt_fengine_c64b(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                    const float *window, void *XB, cudaStream_t stream);

/* Fused F-engine for the tensor-core path: int8 I/Q -> PFB -> FFT -> output
 * scaled by `scale` (a power of two keeps it exact) and rounded to f16
 * (ab_fmt 0) or bf16 (ab_fmt 1) in the X16 operand layout:
 *   X16[kc][c][e][128 bytes], kc = 32-spectrum chunk (ceil(Nsp/32) chunks),
 *   e < NEp = NE rounded up to 16, row = [re(32 spectra) | im(32 spectra)],
 *   16-byte chunk j of row e stored at chunk j ^ (e & 7) (the K-major
 *   128-byte-swizzled layout the tensor cores read), spectra past Nsp zero.
 * Rows NE..NEp-1 are not written (zero them once).  Nch <= 2048.  All
 * buffers 16-byte aligned. */
MDT_API mdt_status mdt_fengine_x16(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                   const float *window, void *X16, int ab_fmt, float scale,
                                   cudaStream_t stream);

/* Tensor-core F-engine (Nch = 1024, Ntaps 4 or 8): same inputs and X16
 * output layout as mdt_fengine_x16, with the 1024-point DFT done as two
 * 32-point DFT matrix products on tcgen05 (f16 operands, FP32 accumulation,
 * FP32 twiddles between them); the PFB output and the twiddled intermediate
 * are rounded to f16 once each.  `err` (device int, zeroed by the caller) is
 * set if a device wait timed out.  Replaces PpS_Batch -> cufftExecC2C ->
 * ReorderFOutput (reference MDT_OneStation_client.cu:1083-1114) for the
 * tensor-core X-engine. */
MDT_API mdt_status mdt_fengine_tc(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                  const float *window, void *X16, int ab_fmt, float scale,
                                  int *err, cudaStream_t stream);

/* The same tensor-core F-engine with the int8 requantisation of
 * mdt_fengine_q8 (per-channel qscales, rint, clamp to [-127, 127]) as its
 * output stage; the plan's INT8 precision uses it at Nch 1024. */
MDT_API mdt_status mdt_fengine_tc_q8(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                     const float *window, void *X16, const float *qscales,
                                     int *err, cudaStream_t stream);

/* Measured dense throughput of tcgen05.mma kind::f16 (M = 128, N = n of 128
 * or 256, K = 16, FP32 accumulate, random f16 operands resident in shared
 * memory): ctas_per_sm CTAs per SM (ctas_per_sm * n <= 512 TMEM columns),
 * each issuing iters x 4 MMAs into one accumulator; the best of `reps` timed
 * launches (after one warm-up) gives *best_ms and *tflops.  *err (device int)
 * is set if the completion wait timed out.  Measurement support: the
 * denominator for the X-engine's kind::f16 fraction. */
MDT_API mdt_status mdt_tc_peak_f16(int n, int ctas_per_sm, int iters, int reps, float *best_ms,
                                   double *tflops, int *err, cudaStream_t stream);

/* Measured FP32 FMA throughput: one 1024-thread CTA per SM, each thread
 * running independent FMA chains of `iters` steps (packed fma.rn.f32x2 when
 * `packed`, else scalar fma.rn.f32); the best of `reps` timed launches
 * (after one warm-up) gives *best_ms and *tflops (2 flops per FMA).
 * Measurement support: the denominator for the FP32 X-engine's fraction. */
MDT_API mdt_status mdt_fp32_peak(int packed, int iters, int reps, float *best_ms, double *tflops,
                                 cudaStream_t stream);

/* Exact-int8 F-engine: as mdt_fengine_x16 but the values are integers
 * clamp(rint(x * qscales[c]), -127, 127) (stored as f16, exactly). */
MDT_API mdt_status mdt_fengine_q8(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                  const float *window, void *X16, const float *qscales,
                                  cudaStream_t stream);

/* Exact int8 X-engine on tensor cores: X16 holding integers in [-127, 127];
 * f16 MMAs accumulate 512-spectrum windows in TMEM (exact: every partial sum
 * is an integer below 2^24) that are folded into int32 running sums.
 * `vis_i32` (int32 (re, im) [Nch][NE*NE], may be NULL) receives the exact
 * sums, `vis` (may be NULL) sums / (Nsp * qscales[c]^2), `vis_acc` (may be
 * NULL) adds them in FP64.  Nsp <= 16384 keeps every sum within int32. */
MDT_API mdt_status mdt_xengine_q8(int ne, int nch, int nsp, const void *X16, const float *qscales,
                                  void *vis, void *vis_acc, void *vis_i32, int *err,
                                  cudaStream_t stream);

/* Tensor-core Hermitian X-engine (tcgen05.mma kind::f16, FP32 accumulate)
 * on the X16 layout above: V_c = X_c X_c^H / (Nsp * scale^2), lower-triangle
 * tiles only, written full square column-major to `vis` (complex64
 * [Nch][NE*NE], may be NULL) and/or added to `vis_acc` (complex128, may be
 * NULL).  `err` (device int) is set to 1 if a bounded device-side wait gave
 * up.  Replaces cublasCgemmBatched (reference MDT_OneStation_client.cu:1128)
 * for the reduced-precision path. */
MDT_API mdt_status mdt_xengine_tc(int ne, int nch, int nsp, const void *X16, int ab_fmt,
                                  float scale, void *vis, void *vis_acc, int *err,
                                  cudaStream_t stream);

/* Deterministic synthetic int8 I/Q stream (integer-only arithmetic; same
 * samples as the CPU generator used by the tests): spectra s0 .. s0+nsp-1,
 * element noise sigma_q8[e]/256 LSB, optional tone table tone_q16[e][c][2]
 * (Q16 LSB), nsrc common sources with sigma src_sigma_q8[k]/256 and integer
 * delays src_delay[k][e] samples.  All table pointers are device pointers. */
MDT_API mdt_status mdt_synth_iq(uint64_t seed, int ne, int nch, long s0, long nsp,
                                const int32_t *sigma_q8, const int32_t *tone_q16, int nsrc,
                                const int32_t *src_sigma_q8, const int32_t *src_delay,
                                int8_t *out, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * 3. Plan API: fused F-engine + X-engine with streamed PFB history
 * ---------------------------------------------------------------------- */

typedef enum {
    MDT_PREC_FP32 = 0, /* complex64 F-output, FP32 SIMT X-engine (<=1e-5 vs FP64) */
    MDT_PREC_FP16 = 1, /* f16 F-output (power-of-two scaled), tcgen05 X-engine, FP32
                          accumulate (<=1e-3 vs FP64); Nch <= 2048 */
    MDT_PREC_BF16 = 2, /* as FP16 with bf16 operands */
    MDT_PREC_INT8 = 3  /* F-output requantised per channel to integers in [-127, 127];
                          exact int32 visibilities on the f16 tensor cores (windowed
                          FP32-exact accumulation folded into int32), scaled to float;
                          Nch <= 2048.  (sm_103a has no int8 tensor-core MMA.) */
} mdt_precision;

typedef struct {
    int nelements; /* NE = Npols*Nelements */
    int nchannels; /* Nch */
    int ntaps;     /* Ntaps */
    int nspectra;  /* Nsp per integration */
    int precision; /* mdt_precision */
} mdt_fx_desc;

typedef struct mdt_fx_plan_s *mdt_fx_plan;

/* Validates desc against the reference's parameter domain and allocates the
 * plan's device workspace (F-engine output for one integration, the PFB
 * history of Ntaps-1 spectra and the window). */
MDT_API mdt_status mdt_fx_create(const mdt_fx_desc *desc, mdt_fx_plan *plan);
MDT_API mdt_status mdt_fx_destroy(mdt_fx_plan plan);
MDT_API mdt_status mdt_fx_set_stream(mdt_fx_plan plan, cudaStream_t stream);
/* Copies Ntaps*Nch floats from a device pointer into the plan. */
MDT_API mdt_status mdt_fx_set_window(mdt_fx_plan plan, const float *window);
/* FP64 cross-integration accumulation: when `acc` (device, complex128
 * [Nch][NE*NE], 16-byte aligned, zeroed by the caller) is set, every
 * integration's visibilities are also added into it; NULL disables. */
MDT_API mdt_status mdt_fx_set_accumulator(mdt_fx_plan plan, void *acc);
/* INT8 plans: per-channel requantisation scales (device, Nch floats).  The
 * F-output x of channel c becomes clamp(rint(x * scales[c]), -127, 127);
 * visibilities are the exact integer sums / (Nsp * scales[c]^2).  Without a
 * call (or after a call with NULL) the plan calibrates them at the next
 * integration from its first min(Nsp, 64) spectra: scales[c] = 20 / rms_c. */
MDT_API mdt_status mdt_fx_set_channel_scales(mdt_fx_plan plan, const float *scales);
MDT_API mdt_status mdt_fx_get_channel_scales(mdt_fx_plan plan, float *scales);
/* The power-of-two scale applied to the F-engine output before rounding to
 * f16/bf16 (chosen from the window at mdt_fx_set_window; 1 for FP32); the
 * visibilities are divided by scale^2. */
MDT_API mdt_status mdt_fx_get_scale(mdt_fx_plan plan, float *scale);
/* Waits for the plan's stream and reports MDT_ERR_TIMEOUT if a bounded
 * device-side wait of the tensor-core X-engine gave up since the last check
 * (the flag is then cleared). */
MDT_API mdt_status mdt_fx_check(mdt_fx_plan plan);
/* Bytes of device memory the plan holds. */
MDT_API mdt_status mdt_fx_workspace_bytes(mdt_fx_plan plan, size_t *bytes);

/* One-shot: iq holds nint*Nsp + Ntaps - 1 contiguous spectra (a stream with
 * its own Ntaps-1 spectra of lead-in); writes nint integrations of
 * visibilities V[j][c][NE*NE] complex64.  The plan's history is not used. */
MDT_API mdt_status mdt_fx_execute(mdt_fx_plan plan, const int8_t *iq, int nint, void *vis);

/* Streaming: the first call after mdt_fx_stream_reset takes Nsp + Ntaps - 1
 * spectra (lead-in included); every later call takes Nsp new spectra and
 * reuses the last Ntaps-1 spectra of the previous call as PFB history (the
 * reference's device-to-device history shift, MDT_OneStation_client.cu:1170).
 * Writes one integration of visibilities. */
MDT_API mdt_status mdt_fx_stream_reset(mdt_fx_plan plan);
MDT_API mdt_status mdt_fx_stream_push(mdt_fx_plan plan, const int8_t *iq, void *vis);

/* Host-memory form of the streamed pipeline: h_iq (host) holds
 * nint*Nsp + Ntaps - 1 spectra, h_vis (host) receives nint integrations.
 * Integration j+1 is copied host->device on a second stream while j is
 * processed and j-1's visibilities are copied back (the reference's
 * rank 1 H2D -> rank 2 F/X -> rank 3 D2H chain, MDT_OneStation_client.cu
 * :1048,1083-1128,1199).  Pinned host memory gives full overlap.  Allocates
 * two input and two visibility staging buffers on first use; resets the
 * plan's stream history; returns when the last copy has completed. */
MDT_API mdt_status mdt_fx_execute_host(mdt_fx_plan plan, const int8_t *h_iq, int nint,
                                       void *h_vis);

/* Stage timing: when enabled, CUDA events are recorded on the plan's stream
 * around every F-engine and X-engine launch; mdt_fx_get_timing waits for
 * the last one, returns the summed kernel times in ms and the number of
 * integrations, and clears the record. */
MDT_API mdt_status mdt_fx_set_timing(mdt_fx_plan plan, int enable);
MDT_API mdt_status mdt_fx_get_timing(mdt_fx_plan plan, double *fengine_ms, double *xengine_ms,
                                     int *count);

/* ------------------------------------------------------------------------
 * 4. Batches: many independent jobs of uneven shape (benchmark configuration
 *    "24 ragged jobs"), f16 tensor-core path, Nch <= 2048, Ntaps 4 or 8.
 *    One F-engine launch per (Nch, Ntaps) group and one persistent X-engine
 *    launch over a work list spanning every job, captured in a CUDA graph on
 *    the batch's own stream and replayed; the X-engine's column-chunk width
 *    and work order come from an autotuner (timed on the batch, cached per
 *    shape; also in the file named by MDT_AUTOTUNE_CACHE when set).
 * ---------------------------------------------------------------------- */
typedef struct mdt_fx_batch_s *mdt_fx_batch;

/* descs[j]: each job's shape (precision must be MDT_PREC_FP16).  Allocates the
 * jobs' F-output buffers and a non-blocking stream; windows default to the
 * Hamming windowed sinc (mdt_window_hamming_sinc). */
MDT_API mdt_status mdt_fx_batch_create(const mdt_fx_desc *descs, int njobs, mdt_fx_batch *batch);
MDT_API mdt_status mdt_fx_batch_destroy(mdt_fx_batch batch);
/* Replaces job's window (device, Ntaps*Nch floats). */
MDT_API mdt_status mdt_fx_batch_set_window(mdt_fx_batch batch, int job, const float *window);
/* The stream every batch launch is issued on (synchronise on it or use
 * mdt_fx_batch_check). */
MDT_API mdt_status mdt_fx_batch_get_stream(mdt_fx_batch batch, cudaStream_t *stream);
/* Runs the autotuner now (otherwise the first execute does); reports the
 * chosen column-chunk width and whether the work list is cost-ordered. */
MDT_API mdt_status mdt_fx_batch_autotune(mdt_fx_batch batch, int *maxw, int *cost_order);
/* One integration of every job: iq[j] (device, Nsp_j + Ntaps_j - 1 spectra,
 * 16-byte aligned) -> vis[j] (device, complex64 [Nch_j][NE_j*NE_j]); iq and
 * vis are host arrays of njobs device pointers.  use_graph = 1 replays the
 * captured graph (captured on first use), 0 launches the kernels directly.
 * Asynchronous on the batch's stream. */
MDT_API mdt_status mdt_fx_batch_execute(mdt_fx_batch batch, const int8_t *const *iq,
                                        void *const *vis, int use_graph);
/* Waits for the batch's stream; MDT_ERR_TIMEOUT if a bounded device wait gave up. */
MDT_API mdt_status mdt_fx_batch_check(mdt_fx_batch batch);

/* ------------------------------------------------------------------------
 * GPU depacketiser.  Replaces the host loop of the reference client's rank 1
 * (MDT_OneStation_client.cu:846-907), which unpacks each SNAP UDP packet into
 * the [spectrum][element][channel] input stack.
 *
 * A packet: `words_header` uint32 header words ([0] station, [1] SNAP board,
 * [2] packet counter; the reference has 4), then for each of `sper_element`
 * samples i, for each input j < inputs_per_snap[snap]: the sample of input j
 * -- two uint32 (re, im; int32 fixed point with 19 fraction bits) when
 * sample_bits = 32 (the reference's format), or two int8 (re, im) when
 * sample_bits = 8.  Packets sit `packet_bytes` apart in the batch buffer.
 * Sample i of a packet is element-sample counter*sper_element + i, i.e.
 * spectrum (that / Nch), channel (that % Nch); its element is
 * station*inputs_per_station + sum_{k<snap} inputs_per_snap[k] + j.
 * The reference's SNAP layout: inputs_per_station 38, 4 SNAPs of
 * {10, 10, 10, 8} inputs (MDT_OneStation_client.h:64-68). */
#define MDT_MAX_SNAPS 8
typedef struct {
    int words_header;         /* >= 3 */
    int sper_element;         /* samples per element per packet */
    int inputs_per_station;
    int nsnap;                /* <= MDT_MAX_SNAPS */
    int inputs_per_snap[MDT_MAX_SNAPS];
    int sample_bits;          /* 32: int32 x 2^-19 -> complex64; 8: int8 I/Q -> int8 I/Q */
    int packet_bytes;         /* stride between packets, multiple of 4 */
} mdt_packet_format;

/* Device-side counters (zero them before the first call; they accumulate). */
typedef struct {
    unsigned long long accepted;   /* packets written into the window */
    unsigned long long outside;    /* packets whose counter lies outside the window */
    unsigned long long bad;        /* bad station / SNAP, or elements past NE */
    unsigned long long duplicate;  /* further arrivals of a slot already seen */
    unsigned long long missing;    /* slots zero-filled by mdt_depacketise_finish */
} mdt_depack_stats;

/* Number of uint32 arrival counters `seen` needs for a window:
 * ceil(NE / inputs_per_station) * nsnap * (packet slots touching the window). */
MDT_API mdt_status mdt_depacketise_seen_words(const mdt_packet_format *fmt, int ne, int nch,
                                              long long sample0, int nspectra, size_t *words);

/* Writes the samples of `npackets` packets (device buffer) that fall in the
 * window of element-samples [sample0, sample0 + nspectra*Nch) (sample0 a
 * multiple of Nch) into `out`: complex64 [nspectra][NE][Nch] for 32-bit
 * samples (bit-identical to the reference's conversion, which maps
 * 0x80000000 to +4096.0), int8 [nspectra][NE][Nch][2] for 8-bit samples.
 * `seen` (zeroed once) counts arrivals per (station, SNAP, slot).  Can be
 * called many times per window as packets arrive; duplicate packets write the
 * same place (the value of one of them remains). */
MDT_API mdt_status mdt_depacketise(const mdt_packet_format *fmt, const void *packets, int npackets,
                                   int ne, int nch, long long sample0, int nspectra, void *out,
                                   unsigned int *seen, mdt_depack_stats *stats,
                                   cudaStream_t stream);

/* Closes a window: zero-fills the samples of every packet slot that never
 * arrived (gap detection; stats->missing counts them) and clears `seen`. */
MDT_API mdt_status mdt_depacketise_finish(const mdt_packet_format *fmt, int ne, int nch,
                                          long long sample0, int nspectra, void *out,
                                          unsigned int *seen, mdt_depack_stats *stats,
                                          cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Streaming ingest pipeline: host packets -> pinned staging ring -> GPU
 * depacketiser -> fused F/X plan (PFB history carried) -> optional output
 * formatter -> pinned output ring.  Replaces the reference client's rank 1-3
 * chain and its MPI handshakes (MDT_OneStation_client.cu:846-1234) on one GPU.
 *
 * Integration n covers element-samples [S(n), S(n) + len(n)): window 0 is
 * Nsp + Ntaps - 1 spectra from sample 0, window n >= 1 the Nsp spectra after
 * (Ntaps - 1 + n*Nsp)*Nch.  Two windows are open at a time; a packet for a
 * later window closes the oldest (missing packets zero-filled and counted),
 * packets for closed windows are dropped as late.  Packets must be 8-bit
 * (int8 I/Q) in the given format, at most `max_packets` per push; they are
 * copied, so the caller's buffer is free when push returns.  Results come
 * back in order: complex64 [Nch][NE][NE] (formatted = 0) or the
 * baseline-major fftshifted form of mdt_format_baselines (formatted = 1,
 * Npols = 1).  At most 3 results wait for mdt_ingest_pop; a push that would
 * close more returns MDT_ERR_STATE and consumes nothing.  From the third
 * integration on, each integration's F/X work is one CUDA graph launch. */
typedef struct mdt_ingest_s *mdt_ingest;
MDT_API mdt_status mdt_ingest_create(const mdt_fx_desc *desc, const mdt_packet_format *fmt,
                                     int max_packets, int formatted, mdt_ingest *ingest);
MDT_API mdt_status mdt_ingest_destroy(mdt_ingest ingest);
MDT_API mdt_status mdt_ingest_set_window(mdt_ingest ingest, const float *window);
MDT_API mdt_status mdt_ingest_push(mdt_ingest ingest, const void *packets, int npackets);
/* Closes the open windows that hold any packet (end of stream). */
MDT_API mdt_status mdt_ingest_flush(mdt_ingest ingest);
/* Oldest finished integration: its index (-1 if none is ready -- or none is
 * pending -- when wait = 0, or none is pending when wait != 0), its result
 * copied to `out` (host, out_bytes; may be NULL) and its window's counters. */
MDT_API mdt_status mdt_ingest_pop(mdt_ingest ingest, void *out, long long *integration,
                                  mdt_depack_stats *stats, int wait);
MDT_API mdt_status mdt_ingest_counters(mdt_ingest ingest, long long *late, long long *bad,
                                       long long *next_window, size_t *out_bytes);

/* ------------------------------------------------------------------------
 * Output formatter and writers.  The reference writes each integration as
 * CSV lines "j,p,k,q,z,re,im" ("%ld,%d,%ld,%d,%ld,%.6f,%.6f") for
 * j < Nelements, p < Npols, k >= j, q >= p, channel z = 0..Nch-1 fftshifted
 * (z <- channel (z + Nch/2) % Nch), value V[i][(k*Npols+q)*NE + (j*Npols+p)]
 * (MDT_OneStation_client.cu:1239-1266).
 *
 * Number of baselines in that order: Npols(Npols+1)/2 * Nelements(Nelements+1)/2. */
MDT_API mdt_status mdt_num_baselines(int nelements, int npols, long *nbl);

/* GPU gather of the visibilities (complex64 [Nch][NE][NE] column-major, NE =
 * Nelements*Npols, device) into out[bl][z] (complex64, device), baselines in
 * the reference's order, channels fftshifted when `fftshift` (Nch even). */
MDT_API mdt_status mdt_format_baselines(int nelements, int npols, int nch, const void *vis,
                                        void *out, int fftshift, cudaStream_t stream);

/* Host writers of a formatted buffer (host memory, complex64 [nbl][Nch]).
 * CSV: byte-identical to the reference's fprintf lines, formatted by
 * `nthreads` threads (<= 0: all cores) and written in order; `append` adds
 * to an existing file.  Binary: header {"MDTVIS01", int32 Nelements, Npols,
 * Nch, nbl, 8 reserved bytes}, int32 [nbl][4] (j, p, k, q), complex64
 * [nbl][Nch].  Neither needs a GPU. */
MDT_API mdt_status mdt_write_csv(const char *path, int nelements, int npols, int nch,
                                 const void *formatted, int append, int nthreads);
MDT_API mdt_status mdt_write_binary(const char *path, int nelements, int npols, int nch,
                                    const void *formatted, int append);

/* ------------------------------------------------------------------------
 * Adjoints (differentiation through the FX path).  No counterpart in the
 * reference, which only runs forward; these are the backward halves of
 * mdt_fengine_f32 -> gains -> mdt_xengine_f32 for gain calibration and PFB
 * tap optimisation.  Gradients follow PyTorch's convention for complex
 * values: grad(z) = dL/dRe(z) + i dL/dIm(z) for a real loss L.  All complex
 * buffers are complex64; all are device pointers.
 *
 * Y[c][s][e] = gains[c][e] * X[c][s][e]   (X, Y: the layout of
 * mdt_fengine_f32; gains complex64 [Nch][NE]). */
MDT_API mdt_status mdt_apply_gains(int ne, int nch, int nsp, const void *X, const void *gains,
                                   void *Y, cudaStream_t stream);

/* X-engine adjoint: for V_c = scale * Y_c Y_c^H (mdt_xengine_f32, Y_c =
 * NE x Nsp, stored Y[c][s][e]) and G = grad(V) in the same column-major
 * visibility layout (G[c][q*NE + r] = G_rq),
 *   dY_c = scale * (G_c + G_c^H) Y_c          written dY[c][s][e]. */
MDT_API mdt_status mdt_xengine_adjoint_f32(int ne, int nch, int nsp, const void *G, const void *Y,
                                           void *dY, float scale, cudaStream_t stream);

/* Adjoint of the gains and of the channel-major reorder, given dY:
 *   dgains[c][e] = sum_s dY[c][s][e] conj(X[c][s][e])   (if dgains != NULL;
 *                  double accumulation, fixed order)
 *   dF[s][e][c]  = conj(gains[c][e]) dY[c][s][e]         (if dF != NULL;
 *                  gains NULL means unit gains).
 * dF is the gradient of the FFT output rows; mdt_fft_c2c with direction +1
 * (the unnormalised inverse) turns it into the gradient of the PFB output. */
MDT_API mdt_status mdt_gain_adjoint(int ne, int nch, int nsp, const void *dY, const void *X,
                                    const void *gains, void *dgains, void *dF,
                                    cudaStream_t stream);

/* PFB tap gradient: with P[s][e][k] = sum_i W[i*Nch + k] in[s+i][e][k]
 * (PpS_Batch, reference MDT_device_functions.cu) and gradP = grad(P)
 * (complex64 [Nsp][NE][Nch]),
 *   gradW[i*Nch + k] = sum_{s,e} Re(gradP[s][e][k] conj(in[s+i][e][k])).
 * `iq` holds Nsp + Ntaps - 1 spectra of int8 I/Q.  Partial sums are doubles
 * in `workspace` (at least Ntaps*Nch*8 bytes; up to 64 times that is used
 * for more parallelism), reduced in a fixed order (deterministic). */
MDT_API mdt_status mdt_pfb_tap_grad(int ne, int nch, int ntaps, int nsp, const void *gradP,
                                    const int8_t *iq, float *gradW, void *workspace,
                                    size_t workspace_bytes, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * One integration without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory
 * themselves -- a real-time ingest loop in which cudaMalloc's implicit device
 * synchronisation would stall other streams, a plugin host that fixes the
 * library's device-memory budget up front, or a foreign-language runtime that
 * owns every device allocation.
 *
 * Runs the plan's FP32 path (int8 I/Q -> spectrum-block F-engine ->
 * Hermitian X-engine) on `iq` (Nsp + Ntaps - 1 spectra, 16-byte aligned),
 * `window` (Ntaps*Nch floats, 16-byte aligned) into `vis` (complex64
 * [Nch][NE*NE], the layout of mdt_fx_execute, which it matches).  The
 * F-engine output lives in a file-scope device array of 96 MiB
 * (MDT_STATIC_SCRATCH_BYTES at build time) that every GPU loading the
 * library holds until exit: requests needing more than that --
 * Nch * ceil(Nsp/8)*8 * NE * 8 bytes -- or Nch > 2048 return
 * MDT_ERR_INVALID_VALUE, as do the shapes every entry point rejects (Nch
 * not a power of two in [32, 16384], NE, Ntaps or Nsp out of range).  The
 * first call on a device (with that device current) looks up the arrays'
 * device addresses and uploads the FFT twiddle tables, so make it before
 * any stream capture.  Under CUDA's default lazy module loading that first
 * call is also when the 96 MiB are committed on the device (at context
 * creation with CUDA_MODULE_LOADING=EAGER): a real-time caller makes one
 * warm-up call per device outside its loop.  All calls on a device share
 * the scratch, which keeps the last call's contents (every call overwrites
 * the part it reads, so nothing needs clearing); calls whose GPU work
 * overlaps race on it.
 * Calls no cudaMalloc/cudaFree. */
MDT_API mdt_status mdt_fx_integrate_static(int ne, int nch, int ntaps, int nsp, const int8_t *iq,
                                           const float *window, void *vis, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* MDT_FX_H */
