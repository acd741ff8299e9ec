// xengine_tc.cu -- Hermitian X-engine on the 5th-generation tensor cores
// (tcgen05.mma kind::f16, accumulators in tensor memory), replacing
// cublasCgemmBatched(OP_N, OP_C, A == B) (reference
// MDT_OneStation_client.cu:1128) for the reduced-precision path.
//
// Operand layout ("X16"), written by the f16/bf16 F-engine: for channel c and
// K-chunk kc of 32 spectra, a block of NEp rows (elements, NE rounded up to
// 16, zero rows beyond NE) of 128 bytes:
//     row e = [ re(s0..s0+31) | im(s0..s0+31) ]   (32 + 32 f16/bf16 values)
// with the 128-byte swizzle applied inside each 8-row atom (16-byte chunk j
// of row e stored at chunk j ^ (e & 7)), i.e. exactly the K-major SW128
// canonical layout, so any run of rows is one contiguous bulk copy that
// lands in shared memory ready for the tensor core.  Spectra beyond Nsp in
// the last chunk are zero.
//
// Per 128-byte row (32 spectra) the complex product V = X X^H is eight real
// K=16 MMAs on two accumulators (k-steps 0,1 = re, 2,3 = im):
//     Re V += A0 B0 + A1 B1 + A2 B2 + A3 B3
//     Im V += A2 B0 + A3 B1 - A0 B2 - A1 B3        (negate-A bit)
// On a diagonal tile (rows and columns are the same elements, A = B) the
// imaginary part is antisymmetric: Im V = G - G^T with G = X_im X_re^T, so
// only G += A2 B0 + A3 B1 is accumulated (six MMAs instead of eight) and the
// epilogue forms G[r][q] - G[q][r] through shared memory.
// A block owns one (channel, row tile of 128 elements, column chunk of up to
// 256 elements) of the lower triangle: only tiles on or below the diagonal
// are computed; the epilogue writes the lower triangle and its conjugate
// mirror (full square, column-major, the cuBLAS C layout) and can add the
// result into an FP64 cross-integration accumulator.
//
// Exact int8 mode (KIND 1): the F-engine requantises each channel to
// integers in [-127, 127] (stored as f16, which holds them exactly); the
// products are exact and an FP32 accumulator stays exact while every partial
// sum is an integer below 2^24, i.e. for 16 K-chunks (512 spectra:
// 512 * 2 * 127^2 < 2^24).  The MMAs therefore accumulate one 512-spectrum
// window at a time into one of two TMEM window buffers (2 x (Re, Im) x N =
// 512 columns for N = 128); 16 epilogue warps fold each finished window into
// int32 running sums held in their registers (a warp owns one TMEM lane
// quarter and 32 columns) while the MMAs fill the other buffer, and write the
// exact int32 visibilities (and their scaled float values) at the end.
//
// Warp roles: warp 0 lane 0 issues bulk copies into the shared-memory stage
// ring; warp 1 allocates tensor memory and its lane 0 issues the MMAs and
// commits; the epilogue warps (2-9, two per TMEM lane quarter, or 2-17 in the
// exact int8 mode) read the accumulators and write visibilities.  Every mbarrier wait is bounded; a
// timeout sets the error flag and the block finishes without further work.
#include <cstdlib>

#include "mdt_common.cuh"
#include "tc_ptx.cuh"
#include "xengine_tc.cuh"

namespace mdt {

constexpr int TC_STAGES = 4;
constexpr int TC_BROWS = 256;  // max column-chunk rows (N)
constexpr int TC_AROWS = 128;  // row tile (M)
constexpr int TC_THREADS = 192;  // the batched kernel: producer, MMA, 4 epilogue warps
// threads of a KIND 0 block (producer, MMA, 8 epilogue warps: two per TMEM lane
// quarter, each on half of the columns) or a KIND 1 block (producer, MMA, 16
// epilogue warps holding the int32 running sums)
constexpr int tc_threads(int kind) { return kind == 1 ? 576 : 320; }
constexpr int TC_MAX_TILES = 160;
constexpr uint32_t TC_A_BYTES = TC_AROWS * 128;
// Epilogue scratch of the f16/bf16 kernel with 128-wide chunks, reused from the
// stage ring once every MMA has completed: the conjugate mirror's transpose
// blocks (16 columns x 33 rows per epilogue warp, or 32 x 33 for each of the
// batched kernel's four), then a diagonal tile's G (128 rows of 129 floats,
// the odd stride keeping row and column accesses conflict-free).
constexpr int TC_GS = 129;
constexpr size_t TC_TB_BYTES = 4 * 32 * 33 * sizeof(float2);
constexpr size_t TC_GS_BYTES = (size_t)TC_AROWS * TC_GS * sizeof(float);
constexpr bool tc_sym(int kind, int brows) { return kind == 0 && brows == 128; }
// the batched kernel's stage (B chunks of <= TCB_MAXW rows, then A) and shared memory
constexpr uint32_t TCB_B_BYTES = TCB_MAXW * 128;
constexpr uint32_t TCB_STAGE_BYTES = TCB_B_BYTES + TC_A_BYTES;
constexpr size_t TCB_SMEM = 1024 + (size_t)TC_STAGES * TCB_STAGE_BYTES + TC_GS_BYTES + 256;
// offset of the mbarriers: after the stage ring and after the epilogue scratch
constexpr size_t tc_bar_off(int kind, int brows, int stages)
{
    return tc_sym(kind, brows) &&
                   TC_TB_BYTES + TC_GS_BYTES > (size_t)stages * ((size_t)brows * 128 + TC_A_BYTES)
               ? TC_TB_BYTES + TC_GS_BYTES
               : (size_t)stages * ((size_t)brows * 128 + TC_A_BYTES);
}
// shared memory of the single-launch kernel for a (KIND, BROWS, STAGES) shape
constexpr size_t tc_smem(int kind, int brows, int stages)
{
    return 1024 + tc_bar_off(kind, brows, stages) + 256;
}


struct TcArgs {
    const uint8_t *X;   // X16 operand base
    long chunk_bytes;   // stride between 32-spectrum chunks: Nch * NEp * 128
    long chan_bytes;    // stride between channels: NEp * 128
    int ne, nep, nkc;
    int ntiles;
    int ab_fmt;         // 0 = f16, 1 = bf16
    float alpha;        // applied to the accumulators (1/(Nsp * scale^2))
    float2 *V;          // [nch][ne*ne] complex64, column-major per channel (may be null)
    double2 *Vacc;      // [nch][ne*ne] complex128 accumulator (may be null)
    int *err;           // set to 1 on a wait timeout
    const float *qscales;  // exact int8 mode: per-channel requantisation scales
    int2 *raw;          // exact int8 mode: optional int32 (re, im) visibilities [nch][ne*ne]
    TcTile tiles[TC_MAX_TILES];
};

constexpr int TC_WIN = 16;  // K-chunks (of 32 spectra) per exact accumulation window

// STAGES-deep ring of (B: BROWS rows, A: 128 rows) stages; BROWS 256 with 4
// stages (one block per SM) or 128 with 3 stages (two blocks per SM, so one
// block's epilogue overlaps the other's products).
template <int KIND, int BROWS, int STAGES>  // KIND 0: f16 / bf16, float results; 1: exact int8
__global__ void __launch_bounds__(tc_threads(KIND), (KIND == 0 && BROWS == 128 ? 2 : 1))
    xengine_tc_kernel(const __grid_constant__ TcArgs a)
{
    constexpr uint32_t B_BYTES = BROWS * 128;
    constexpr uint32_t STAGE_BYTES = B_BYTES + TC_A_BYTES;
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte alignment for the swizzle atoms
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + tc_bar_off(KIND, BROWS, STAGES));
    // bars[0..S) full, bars[S..2S) empty, bars[2S] done, bars[2S+1..2S+2] window
    // full, bars[2S+3..2S+4] window empty; then the TMEM address slot
    uint64_t *win_full = bars + 2 * STAGES + 1;
    uint64_t *win_empty = bars + 2 * STAGES + 3;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * STAGES + 5);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ch = blockIdx.x / a.ntiles;
    const TcTile tile = a.tiles[blockIdx.x - ch * a.ntiles];
    const int N = tile.n;
    // diagonal tile: rows and columns are the same elements (A read from B's rows)
    const bool sym = tc_sym(KIND, BROWS) && tile.r0 == tile.q0 && !tile.a_sep;
    constexpr int NCOLMUL = (KIND == 0) ? 2 : 4;  // TMEM columns per output column
    const uint32_t ncols = (NCOLMUL * N <= 32) ? 32 : (NCOLMUL * N <= 64) ? 64
                         : (NCOLMUL * N <= 128) ? 128 : (NCOLMUL * N <= 256) ? 256 : 512;

    if (threadIdx.x == 0) {
        for (int s = 0; s < 2 * STAGES + 3; s++) tc::mbar_init(tc::smem_u32(&bars[s]), 1);
        tc::mbar_init(tc::smem_u32(&win_empty[0]), 16);  // one arrival per epilogue warp
        tc::mbar_init(tc::smem_u32(&win_empty[1]), 16);
        tc::fence_mbar_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(tc::smem_u32(tmem_slot), ncols);
        tc::tmem_relinquish();
        tc::fence_before_sync();
    }
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t d_re = tmem, d_im = tmem + (uint32_t)N;

    const uint8_t *xc = a.X + (long)ch * a.chan_bytes;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // ---------------- producer: bulk copies into the stage ring
        const uint32_t bbytes = (uint32_t)N * 128;
        const int arows = min(TC_AROWS, a.nep - tile.r0);
        const uint32_t abytes = tile.a_sep ? (uint32_t)arows * 128 : 0;
        for (int kc = 0; kc < a.nkc && ok; kc++) {
            const int s = kc % STAGES;
            if (kc >= STAGES) {
                ok = tc::mbar_wait(tc::smem_u32(&bars[STAGES + s]), ((kc / STAGES) - 1) & 1);
                if (!ok) break;
            }
            uint8_t *stage = smem + (size_t)s * STAGE_BYTES;
            const uint32_t full = tc::smem_u32(&bars[s]);
            tc::mbar_expect_tx(full, bbytes + abytes);
            const uint8_t *src = xc + (long)kc * a.chunk_bytes;
            tc::bulk_g2s(tc::smem_u32(stage), src + (long)tile.q0 * 128, bbytes, full);
            if (abytes)
                tc::bulk_g2s(tc::smem_u32(stage + B_BYTES), src + (long)tile.r0 * 128, abytes,
                             full);
        }
        // drain: wait until the MMAs consumed every issued stage, so no copy
        // is in flight when the block exits
        if (ok) {
            for (int kc = max(0, a.nkc - STAGES); kc < a.nkc && ok; kc++)
                ok = tc::mbar_wait(tc::smem_u32(&bars[STAGES + (kc % STAGES)]),
                                   (kc / STAGES) & 1);
        }
        if (!ok) atomicExch(a.err, 1);
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        const uint32_t id_pos = tc::idesc_f16(N, a.ab_fmt, 0);
        const uint32_t id_neg = tc::idesc_f16(N, a.ab_fmt, 1);
        for (int kc = 0; kc < a.nkc && ok; kc++) {
            const int s = kc % STAGES;
            uint32_t acc_re = d_re, acc_im = d_im;
            bool first = (kc == 0);
            if constexpr (KIND == 1) {
                const int w = kc / TC_WIN, h = w & 1;
                first = (kc % TC_WIN) == 0;
                if (first && w >= 2) {  // window buffer h must have been folded (window w-2)
                    ok = tc::mbar_wait(tc::smem_u32(&win_empty[h]), ((w >> 1) - 1) & 1);
                    if (!ok) break;
                    tc::fence_after_sync();
                }
                acc_re = tmem + (uint32_t)(h * 2 * N);
                acc_im = acc_re + (uint32_t)N;
            }
            ok = tc::mbar_wait(tc::smem_u32(&bars[s]), (kc / STAGES) & 1);
            if (!ok) break;
            tc::fence_after_sync();
            const uint32_t sb = tc::smem_u32(smem + (size_t)s * STAGE_BYTES);
            const uint32_t sa = tile.a_sep ? sb + B_BYTES : sb + (uint32_t)(tile.r0 - tile.q0) * 128;
            const uint64_t bd = tc::sw128_kmajor_desc(sb);
            const uint64_t ad = tc::sw128_kmajor_desc(sa);
            // k-step j advances the start address by 32 bytes (+2 in the >>4 field)
            tc::mma_f16(acc_re, ad + 0, bd + 0, id_pos, !first);
            tc::mma_f16(acc_re, ad + 2, bd + 2, id_pos, 1);
            tc::mma_f16(acc_re, ad + 4, bd + 4, id_pos, 1);
            tc::mma_f16(acc_re, ad + 6, bd + 6, id_pos, 1);
            tc::mma_f16(acc_im, ad + 4, bd + 0, id_pos, !first);
            tc::mma_f16(acc_im, ad + 6, bd + 2, id_pos, 1);
            if (!sym) {  // a diagonal tile's Im is G - G^T, formed in the epilogue
                tc::mma_f16(acc_im, ad + 0, bd + 4, id_neg, 1);
                tc::mma_f16(acc_im, ad + 2, bd + 6, id_neg, 1);
            }
            tc::mma_commit(tc::smem_u32(&bars[STAGES + s]));
            if constexpr (KIND == 1) {
                if ((kc % TC_WIN) == TC_WIN - 1 || kc == a.nkc - 1)
                    tc::mma_commit(tc::smem_u32(&win_full[(kc / TC_WIN) & 1]));
            }
        }
        tc::mma_commit(tc::smem_u32(&bars[2 * STAGES]));
        if (!ok) atomicExch(a.err, 1);
    } else if (warp >= 2 && KIND == 1) {
        // ---------------- epilogue, exact int8 mode: 16 warps; warp w reads TMEM
        // lane quarter w % 4, columns [32 cg, 32 cg + 32) with cg = (w - 2) / 4, and
        // keeps the int32 running sums of its row and 32 columns in registers
        const int quarter = warp & 3, cg = (warp - 2) >> 2;
        const int r = tile.r0 + quarter * 32 + lane;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        const int nwin = (a.nkc + TC_WIN - 1) / TC_WIN;
        float2 *Vc = a.V ? a.V + (long)ch * a.ne * a.ne : nullptr;
        double2 *Ac = a.Vacc ? a.Vacc + (long)ch * a.ne * a.ne : nullptr;
        int2 *Rc = a.raw ? a.raw + (long)ch * a.ne * a.ne : nullptr;
        const float qs = __ldg(a.qscales + ch);
        const float alpha = a.alpha / (qs * qs);
        int rr[32], ri[32];
#pragma unroll
        for (int j = 0; j < 32; j++) rr[j] = ri[j] = 0;
        for (int w = 0; w < nwin; w++) {
            const int h = w & 1;
            ok = ok && tc::mbar_wait_sleep(tc::smem_u32(&win_full[h]), (w >> 1) & 1);
            tc::fence_after_sync();
            const uint32_t wre = tmem + (uint32_t)(h * 2 * N), wim = wre + (uint32_t)N;
#pragma unroll
            for (int hf = 0; hf < 2; hf++) {
                const int n0 = 32 * cg + 16 * hf;
                if (n0 >= N) continue;  // warp-uniform
                uint32_t vr[16], vi[16];
                tc::tmem_ld16(wre + lane_off + n0, vr);
                tc::tmem_ld16(wim + lane_off + n0, vi);
                tc::tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    // the window sums are integers below 2^24: exact in FP32
                    rr[16 * hf + j] += __float2int_rn(__uint_as_float(vr[j]));
                    ri[16 * hf + j] += __float2int_rn(__uint_as_float(vi[j]));
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(&win_empty[h]));
        }
        if (ok && r < a.ne) {
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int q = tile.q0 + 32 * cg + j;
                if (32 * cg + j >= N || q >= a.ne || q > r) continue;
                const int ire = rr[j];
                const int iim = (q == r) ? 0 : ri[j];
                const long lo = (long)q * a.ne + r, up = (long)r * a.ne + q;
                if (Rc) {
                    Rc[lo] = make_int2(ire, iim);
                    if (q != r) Rc[up] = make_int2(ire, -iim);
                }
                const float re = (float)ire * alpha, im = (float)iim * alpha;
                if (Vc) {
                    Vc[lo] = make_float2(re, im);
                    if (q != r) Vc[up] = make_float2(re, -im);
                }
                if (Ac) {
                    double2 x = Ac[lo];
                    Ac[lo] = make_double2(x.x + (double)re, x.y + (double)im);
                    if (q != r) {
                        double2 y = Ac[up];
                        Ac[up] = make_double2(y.x + (double)re, y.y - (double)im);
                    }
                }
            }
        }
        if (!ok && lane == 0) atomicExch(a.err, 1);
    } else if (warp >= 2 && KIND == 0) {
        // ---------------- epilogue: TMEM -> visibilities, 8 warps: warp w reads
        // TMEM lane quarter w % 4 and the columns of half (w - 2) / 4
        ok = tc::mbar_wait_sleep(tc::smem_u32(&bars[2 * STAGES]), 0);
        tc::fence_after_sync();
        const int quarter = warp & 3, half = (warp - 2) >> 2;
        const int r = tile.r0 + quarter * 32 + lane;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        float2 *Vc = a.V ? a.V + (long)ch * a.ne * a.ne : nullptr;
        double2 *Ac = a.Vacc ? a.Vacc + (long)ch * a.ne * a.ne : nullptr;
        // this warp's columns [c0, c1): N is a multiple of 16, halves are too
        const int nh = ((N + 31) / 32) * 16;
        const int c0 = half * nh, c1 = min(N, c0 + nh);
        // The lower triangle V[q*NE + r] is written along r (the lanes).  The
        // conjugate mirror V[r*NE + q] is transposed through shared memory (the
        // stage ring is idle once every MMA has completed) in 16-column blocks
        // so that it is written along q as well, two rows per store.
        float2 *tb = reinterpret_cast<float2 *>(smem) + (size_t)(warp - 2) * 16 * 33;  // [q][r]
        const int rbase = tile.r0 + quarter * 32;
        // diagonal tile: G (the Im accumulator) row by row into shared memory, so
        // that each thread can read the transposed entry G[q][r] (tile-local)
        float *gs = reinterpret_cast<float *>(smem + TC_TB_BYTES);
        const int rl = quarter * 32 + lane;
        if (sym) {
            for (int n0 = c0; n0 < c1; n0 += 16) {
                uint32_t vg[16];
                tc::tmem_ld16(d_im + lane_off + n0, vg);
                tc::tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 16; j++) gs[rl * TC_GS + n0 + j] = __uint_as_float(vg[j]);
            }
        }
        if (tc_sym(KIND, BROWS)) tc::named_barrier(1, 256);  // the eight epilogue warps
        for (int n0 = c0; n0 < c1; n0 += 16) {
            uint32_t vr[16], vi[16];
            tc::tmem_ld16(d_re + lane_off + n0, vr);
            tc::tmem_ld16(d_im + lane_off + n0, vi);
            tc::tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int q = tile.q0 + n0 + j;
                const bool live = ok && r < a.ne && q < a.ne && q <= r;
                const float re = live ? __uint_as_float(vr[j]) * a.alpha : 0.0f;
                const float g = sym && live ? gs[(n0 + j) * TC_GS + rl] : 0.0f;
                const float im = (live && q != r) ? (__uint_as_float(vi[j]) - g) * a.alpha : 0.0f;
                tb[j * 33 + lane] = make_float2(re, -im);
                if (!live) continue;
                const long lo = (long)q * a.ne + r;
                if (Vc) Vc[lo] = make_float2(re, im);
                if (Ac) {
                    double2 x = Ac[lo];
                    Ac[lo] = make_double2(x.x + (double)re, x.y + (double)im);
                }
            }
            __syncwarp();
            // mirror: rows rbase + rr (two per step), columns q = tile.q0 + n0 + (lane & 15)
            const int qc = lane & 15, q = tile.q0 + n0 + qc;
#pragma unroll 4
            for (int i = 0; i < 16; i++) {
                const int rr = 2 * i + (lane >> 4), rm = rbase + rr;
                if (!ok || rm >= a.ne || q >= a.ne || q >= rm) continue;
                const float2 v = tb[qc * 33 + rr];
                const long up = (long)rm * a.ne + q;
                if (Vc) Vc[up] = v;
                if (Ac) {
                    double2 y = Ac[up];
                    Ac[up] = make_double2(y.x + (double)v.x, y.y + (double)v.y);
                }
            }
            __syncwarp();
        }
        if (!ok && lane == 0) atomicExch(a.err, 1);
        tc::fence_before_sync();
    }
    __syncthreads();
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, ncols);
    }
}

// ------------------------------------------------------------------------
// Persistent batched X-engine (kind::f16): one launch for every job of a
// batch.  The work list holds (job, channel, tile) entries, sorted by the
// host; block b processes entries b, b + grid, b + 2 grid, ...  The shared
// memory stage ring runs on across entries, and the two TMEM accumulator
// sets (Re | Im, N <= 128 columns each, at columns 0 and 256) alternate
// between consecutive entries, so the epilogue of one entry overlaps the
// MMAs of the next.
__global__ void __launch_bounds__(TC_THREADS, 1)
    xengine_tc_batched_kernel(const XJob *__restrict__ jobs, const XWork *__restrict__ work,
                              int nwork, int *err)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // stage ring, then a diagonal entry's G (128 x TC_GS floats), then the barriers
    float *gs = reinterpret_cast<float *>(smem + (size_t)TC_STAGES * TCB_STAGE_BYTES);
    uint64_t *bars = (uint64_t *)(smem + (size_t)TC_STAGES * TCB_STAGE_BYTES + TC_GS_BYTES);
    uint64_t *acc_full = bars + 2 * TC_STAGES, *acc_empty = bars + 2 * TC_STAGES + 2;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * TC_STAGES + 4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < 2 * TC_STAGES + 2; s++) tc::mbar_init(tc::smem_u32(&bars[s]), 1);
        tc::mbar_init(tc::smem_u32(&acc_empty[0]), 4);
        tc::mbar_init(tc::smem_u32(&acc_empty[1]), 4);
        tc::fence_mbar_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(tc::smem_u32(tmem_slot), 512);
        tc::tmem_relinquish();
        tc::fence_before_sync();
    }
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        long it = 0;  // stage-ring position across entries
        for (int w = blockIdx.x; w < nwork && ok; w += gridDim.x) {
            const XWork wk = work[w];
            const XJob jb = jobs[wk.job];
            const uint8_t *xc = jb.X + (long)wk.ch * jb.chan_bytes;
            const uint32_t bbytes = (uint32_t)wk.tile.n * 128;
            const int arows = min(TC_AROWS, jb.nep - wk.tile.r0);
            const uint32_t abytes = wk.tile.a_sep ? (uint32_t)arows * 128 : 0;
            for (int kc = 0; kc < jb.nkc && ok; kc++, it++) {
                const int s = (int)(it % TC_STAGES);
                if (it >= TC_STAGES) {
                    ok = tc::mbar_wait(tc::smem_u32(&bars[TC_STAGES + s]),
                                       (uint32_t)((it / TC_STAGES) - 1) & 1);
                    if (!ok) break;
                }
                uint8_t *stage = smem + (size_t)s * TCB_STAGE_BYTES;
                const uint32_t full = tc::smem_u32(&bars[s]);
                tc::mbar_expect_tx(full, bbytes + abytes);
                const uint8_t *src = xc + (long)kc * jb.chunk_bytes;
                tc::bulk_g2s(tc::smem_u32(stage), src + (long)wk.tile.q0 * 128, bbytes, full);
                if (abytes)
                    tc::bulk_g2s(tc::smem_u32(stage + TCB_B_BYTES), src + (long)wk.tile.r0 * 128,
                                 abytes, full);
            }
        }
        // drain: every issued stage consumed before the block exits
        for (long k = (it > TC_STAGES ? it - TC_STAGES : 0); k < it && ok; k++)
            ok = tc::mbar_wait(tc::smem_u32(&bars[TC_STAGES + (int)(k % TC_STAGES)]),
                               (uint32_t)(k / TC_STAGES) & 1);
        if (!ok) atomicExch(err, 1);
    } else if (warp == 1 && lane == 0) {
        long it = 0;
        int t = 0;
        for (int w = blockIdx.x; w < nwork && ok; w += gridDim.x, t++) {
            const XWork wk = work[w];
            const XJob jb = jobs[wk.job];
            const int N = wk.tile.n, h = t & 1;
            // diagonal entry (A read from B's rows): Im = G - G^T in the epilogue
            const bool sym = wk.tile.r0 == wk.tile.q0 && !wk.tile.a_sep;
            if (t >= 2) {
                ok = tc::mbar_wait(tc::smem_u32(&acc_empty[h]), ((t >> 1) - 1) & 1);
                if (!ok) break;
                tc::fence_after_sync();
            }
            const uint32_t d_re = tmem + (uint32_t)(h * 256), d_im = d_re + (uint32_t)N;
            const uint32_t id_pos = tc::idesc_f16(N, 0, 0), id_neg = tc::idesc_f16(N, 0, 1);
            for (int kc = 0; kc < jb.nkc && ok; kc++, it++) {
                const int s = (int)(it % TC_STAGES);
                ok = tc::mbar_wait(tc::smem_u32(&bars[s]), (uint32_t)(it / TC_STAGES) & 1);
                if (!ok) break;
                tc::fence_after_sync();
                const uint32_t sb = tc::smem_u32(smem + (size_t)s * TCB_STAGE_BYTES);
                const uint32_t sa = wk.tile.a_sep ? sb + TCB_B_BYTES
                                                  : sb + (uint32_t)(wk.tile.r0 - wk.tile.q0) * 128;
                const uint64_t bd = tc::sw128_kmajor_desc(sb), ad = tc::sw128_kmajor_desc(sa);
                const uint32_t acc = kc > 0;
                tc::mma_f16(d_re, ad + 0, bd + 0, id_pos, acc);
                tc::mma_f16(d_re, ad + 2, bd + 2, id_pos, 1);
                tc::mma_f16(d_re, ad + 4, bd + 4, id_pos, 1);
                tc::mma_f16(d_re, ad + 6, bd + 6, id_pos, 1);
                tc::mma_f16(d_im, ad + 4, bd + 0, id_pos, acc);
                tc::mma_f16(d_im, ad + 6, bd + 2, id_pos, 1);
                if (!sym) {
                    tc::mma_f16(d_im, ad + 0, bd + 4, id_neg, 1);
                    tc::mma_f16(d_im, ad + 2, bd + 6, id_neg, 1);
                }
                tc::mma_commit(tc::smem_u32(&bars[TC_STAGES + s]));
            }
            tc::mma_commit(tc::smem_u32(&acc_full[h]));
        }
        if (!ok) atomicExch(err, 1);
    } else if (warp >= 2) {
        const int quarter = warp & 3;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        int t = 0;
        for (int w = blockIdx.x; w < nwork; w += gridDim.x, t++) {
            const XWork wk = work[w];
            const XJob jb = jobs[wk.job];
            const int N = wk.tile.n, h = t & 1;
            const bool sym = wk.tile.r0 == wk.tile.q0 && !wk.tile.a_sep;
            ok = ok && tc::mbar_wait_sleep(tc::smem_u32(&acc_full[h]), (t >> 1) & 1);
            // the four epilogue warps agree on ok (so that they leave together and
            // meet at every barrier below) and have finished the previous entry's
            // reads of gs
            ok = !tc::named_barrier_or(1, 128, !ok);
            tc::fence_after_sync();
            const uint32_t d_re = tmem + (uint32_t)(h * 256), d_im = d_re + (uint32_t)N;
            const int rl = quarter * 32 + lane;
            const int r = wk.tile.r0 + rl;
            if (sym) {  // G row by row into shared memory, for the transposed entries
                for (int n0 = 0; n0 < N; n0 += 16) {
                    uint32_t vg[16];
                    tc::tmem_ld16(d_im + lane_off + n0, vg);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 16; j++)
                        if (n0 + j < N) gs[rl * TC_GS + n0 + j] = __uint_as_float(vg[j]);
                }
                tc::named_barrier(1, 128);
            }
            // no visibility buffer (autotuning before the first execute): no writes
            float2 *Vc = jb.V ? jb.V + (long)wk.ch * jb.ne * jb.ne : nullptr;
            for (int n0 = 0; n0 < N; n0 += 16) {
                uint32_t vr[16], vi[16];
                tc::tmem_ld16(d_re + lane_off + n0, vr);
                tc::tmem_ld16(d_im + lane_off + n0, vi);
                tc::tmem_ld_wait();
                if (!ok || r >= jb.ne || !Vc) continue;
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int q = wk.tile.q0 + n0 + j;
                    if (q >= jb.ne || q > r) continue;
                    const float re = __uint_as_float(vr[j]) * jb.alpha;
                    const float g = sym ? gs[(n0 + j) * TC_GS + rl] : 0.0f;
                    const float im = (q == r) ? 0.0f : (__uint_as_float(vi[j]) - g) * jb.alpha;
                    Vc[(long)q * jb.ne + r] = make_float2(re, im);
                    if (q != r) Vc[(long)r * jb.ne + q] = make_float2(re, -im);
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(tc::smem_u32(&acc_empty[h]));
            if (!ok) break;
        }
        if (!ok && lane == 0) atomicExch(err, 1);
    }
    __syncthreads();
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 512);
    }
}

mdt_status xengine_tc_batched(const XJob *jobs, const XWork *work, int nwork, int *err,
                              cudaStream_t stream)
{
    if (nwork <= 0) return MDT_SUCCESS;
    cudaError_t e = cudaFuncSetAttribute(xengine_tc_batched_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TCB_SMEM);
    if (e != cudaSuccess) return cuda_status(e, "batched X-engine smem attribute");
    const int blocks = std::min(nwork, sm_count());
    xengine_tc_batched_kernel<<<blocks, TC_THREADS, TCB_SMEM, stream>>>(jobs, work, nwork, err);
    return launch_status("xengine_tc_batched_kernel");
}

// Lower-triangle work list for NE elements: row tiles of 128, column chunks
// of up to maxw from 0 to the end of the row tile's diagonal block.
int make_tiles(int ne, int nep, int maxw, TcTile *tiles)
{
    int n = 0;
    for (int r0 = 0; r0 < nep; r0 += TC_AROWS) {
        const int cend = std::min(nep, r0 + TC_AROWS);
        for (int q0 = 0; q0 < cend;) {
            if (n >= TC_MAX_TILES) return -1;
            // Chunks narrower than the row tile leave the diagonal block whole:
            // its chunk holds every row of the tile, so that A is read from B's
            // rows and the imaginary part is formed as G - G^T.
            const int w = (maxw < TC_AROWS && q0 == r0) ? cend - q0 : std::min(maxw, cend - q0);
            TcTile t;
            t.r0 = (int16_t)r0;
            t.q0 = (int16_t)q0;
            t.n = (int16_t)w;
            // A is read from the B rows only when the chunk holds every valid
            // row of the tile (rows past NEp feed accumulator rows that are
            // never stored) and the 128 A rows stay inside the B region of
            // the stage; otherwise A is loaded on its own.
            const bool inside = q0 <= r0 && std::min(r0 + TC_AROWS, nep) <= q0 + w &&
                                r0 - q0 + TC_AROWS <= TC_BROWS;
            t.a_sep = (int16_t)(inside ? 0 : 1);
            tiles[n++] = t;
            q0 += w;
        }
    }
    return n;
}

int x16_padded_rows(int ne) { return (ne + 15) / 16 * 16; }
int x16_chunks(int nsp) { return (nsp + 31) / 32; }

mdt_status xengine_tc(int ne, int nch, int nsp, const void *X16, int ab_fmt, float scale,
                      float2 *V, double2 *Vacc, int *err, cudaStream_t stream)
{
    if (!X16 || (!V && !Vacc) || !err) return invalid("xengine_tc: null pointer");
    if (((uintptr_t)X16 & 15) != 0) return invalid("xengine_tc: X16 must be 16-byte aligned");
    TcArgs a;
    a.ne = ne;
    a.nep = x16_padded_rows(ne);
    a.nkc = x16_chunks(nsp);
    a.chan_bytes = (long)a.nep * 128;
    a.chunk_bytes = (long)nch * a.chan_bytes;
    a.X = (const uint8_t *)X16;
    a.ab_fmt = ab_fmt;
    a.alpha = 1.0f / ((float)nsp * scale * scale);
    a.V = V;
    a.Vacc = Vacc;
    a.err = err;
    a.qscales = nullptr;
    a.raw = nullptr;
    // column chunks of <= 128 with a 3-stage ring: two blocks per SM;
    // MDT_XTILE=256 selects <= 256-wide chunks, 4 stages, one block per SM
    static const bool wide = [] {
        const char *v = getenv("MDT_XTILE");
        return v && atoi(v) == 256;
    }();
    const int maxw = wide ? 256 : 128;
    a.ntiles = make_tiles(ne, a.nep, maxw, a.tiles);
    if (a.ntiles <= 0) return invalid("xengine_tc: too many tiles");
    long blocks = (long)nch * a.ntiles;
    if (blocks > 0x7fffffffL) return invalid("xengine_tc: grid too large");
    auto launch = [&](auto kern, size_t smem) -> mdt_status {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return cuda_status(e, "xengine_tc smem attribute");
        kern<<<(unsigned)blocks, tc_threads(0), smem, stream>>>(a);
        return launch_status("xengine_tc_kernel");
    };
    return wide ? launch(xengine_tc_kernel<0, 256, 4>, tc_smem(0, 256, 4))
                : launch(xengine_tc_kernel<0, 128, 3>, tc_smem(0, 128, 3));
}

// Exact int8 mode: X16 holds integers in [-127, 127] (f16) requantised with
// qscales[c]; vis = int32 sums / (Nsp * qscales[c]^2); raw = the int32 sums.
mdt_status xengine_q8(int ne, int nch, int nsp, const void *X16, const float *qscales, float2 *V,
                      double2 *Vacc, int2 *raw, int *err, cudaStream_t stream)
{
    if (!X16 || !qscales || (!V && !Vacc && !raw) || !err)
        return invalid("xengine_q8: null pointer");
    if (((uintptr_t)X16 & 15) != 0) return invalid("xengine_q8: X16 must be 16-byte aligned");
    TcArgs a;
    a.ne = ne;
    a.nep = x16_padded_rows(ne);
    a.nkc = x16_chunks(nsp);
    a.chan_bytes = (long)a.nep * 128;
    a.chunk_bytes = (long)nch * a.chan_bytes;
    a.X = (const uint8_t *)X16;
    a.ab_fmt = 0;
    a.alpha = 1.0f / (float)nsp;
    a.V = V;
    a.Vacc = Vacc;
    a.err = err;
    a.qscales = qscales;
    a.raw = raw;
    a.ntiles = make_tiles(ne, a.nep, 128, a.tiles);
    if (a.ntiles <= 0) return invalid("xengine_q8: too many tiles");
    cudaError_t e = cudaFuncSetAttribute(xengine_tc_kernel<1, 128, 4>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tc_smem(1, 128, 4));
    if (e != cudaSuccess) return cuda_status(e, "xengine_q8 smem attribute");
    long blocks = (long)nch * a.ntiles;
    if (blocks > 0x7fffffffL) return invalid("xengine_q8: grid too large");
    xengine_tc_kernel<1, 128, 4><<<(unsigned)blocks, tc_threads(1), tc_smem(1, 128, 4), stream>>>(a);
    return launch_status("xengine_tc_kernel<exact int8>");
}

}  // namespace mdt

extern "C" MDT_API mdt_status mdt_xengine_q8(int ne, int nch, int nsp, const void *X16,
                                             const float *qscales, void *vis, void *vis_acc,
                                             void *vis_i32, int *err, cudaStream_t stream)
{
    if (ne < 1 || ne > MDT_MAX_ELEMENTS || nch < 1 || nsp < 1 || nsp > MDT_MAX_SPECTRA)
        return mdt::invalid("xengine_q8: bad arguments");
    return mdt::xengine_q8(ne, nch, nsp, X16, qscales, (float2 *)vis, (double2 *)vis_acc,
                           (int2 *)vis_i32, err, stream);
}

extern "C" MDT_API mdt_status mdt_xengine_tc(int ne, int nch, int nsp, const void *X16, int ab_fmt,
                                             float scale, void *vis, void *vis_acc, int *err,
                                             cudaStream_t stream)
{
    if (ne < 1 || ne > MDT_MAX_ELEMENTS || nch < 1 || nsp < 1 || (ab_fmt != 0 && ab_fmt != 1) ||
        !(scale > 0.0f))
        return mdt::invalid("xengine_tc: bad arguments");
    return mdt::xengine_tc(ne, nch, nsp, X16, ab_fmt, scale, (float2 *)vis, (double2 *)vis_acc,
                           err, stream);
}
