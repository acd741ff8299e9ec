// xengine_simt.cu -- FP32 (SIMT) X-engine: per channel c the Hermitian
// product V_c = alpha * X_c X_c^H (+ beta V_c), computed on the lower
// triangle only and mirrored, which is the reference's cublasCgemmBatched
// call (OP_N, OP_C, A == B, alpha = 1/Nspectra, beta = 0;
// MDT_OneStation_client.cu:1128, :656-660, :683-686).  Also the cuBLAS
// subset the reference calls (cublasCreate/cublasSetStream/cublasDestroy/
// cublasCgemmBatched, :690,:699,:1128), with a general batched CGEMM for
// argument patterns other than the Hermitian one.
//
// Tiling: a block owns one pair (I >= J) of 64-wide super-tiles of one
// channel; each thread accumulates a 4x4 complex micro-tile.  Only micro-tiles
// on or below the diagonal are computed in diagonal pairs.  When a pair has
// fewer than 256 micro-tiles the spare threads split the K (time) loop and
// the partial sums are added in a fixed order.  Operand chunks of 32 time
// samples are staged with cp.async into a double buffer (one barrier pair
// per chunk, no staging registers).
#include <cublas_v2.h>
#include "mdt_cufft_cublas_shim.h"  // checks the exported signatures

#include <algorithm>
#include <new>

#include "mdt_common.cuh"

namespace mdt {

constexpr int XS_ST = 64;       // super-tile width
constexpr int XS_MT = 4;        // micro-tile width
constexpr int XS_KC = 32;       // time samples staged per chunk
constexpr int XS_THREADS = 256;
// Complex multiply-adds of the micro-tile as packed f32x2 fmas.
#ifndef MDT_XS_F32X2
#define MDT_XS_F32X2 1
#endif
// Staged operand rows are element-major: row e holds the chunk's XS_KC time
// samples as XS_KC/2 16-byte pairs; pair j of row e sits at position
// j ^ ((e / XS_MT) & 7), so the 16-byte loads of lanes with different
// micro-tile rows fall in different bank groups.
constexpr int XS_ROWB = XS_KC * 8;  // bytes per staged row

struct XengArgs {
    int ne, nsp, nsuper, npairs;
    const float2 *X;             // base (when Xptrs == nullptr)
    const float2 *const *Xptrs;  // per-channel operand pointers (cuBLAS shim)
    long ld, xstride;
    float2 *V;
    float2 *const *Vptrs;
    long ldv, vstride;
    float2 alpha, beta;
    int beta_zero;
    int blocked;  // operand layout: 0 = X[k*ld + e]; 1 = blocks of 8 samples, X[(k/8)*ld + e*8 + k%8]
    int dual;     // NE <= 64: a block takes two channels (A and B buffers hold one each)
    long nbatch;
};

__device__ __forceinline__ void pair_index(int p, int &I, int &J)
{
    // p enumerates (I, J), I >= J, row by row: p = I(I+1)/2 + J
    int i = (int)((sqrtf(8.0f * p + 1.0f) - 1.0f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= p) i++;
    while (i * (i + 1) / 2 > p) i--;
    I = i;
    J = p - i * (i + 1) / 2;
}

// 8-byte asynchronous global->shared copy; src_bytes 0 fills zeros.
__device__ __forceinline__ void cp_async8(void *dst, const void *src, int src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}
// 16-byte asynchronous global->shared copy; src_bytes 0 fills zeros.
__device__ __forceinline__ void cp_async16(void *dst, const void *src, int src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

constexpr size_t XS_SMEM = (size_t)2 /*stages*/ * 2 /*A,B*/ * XS_ST * XS_ROWB;

// byte offset of time sample kk of element e in a staged operand
__device__ __forceinline__ int xs_off(int e, int kk)
{
    return e * XS_ROWB + ((((kk >> 1) ^ ((e >> 2) & 7))) << 4) + ((kk & 1) << 3);
}

__global__ void __launch_bounds__(XS_THREADS, 3) xengine_herm_f32_kernel(XengArgs a)
{
    // [stage][operand][k][element]; the K-slice reduction reuses the space
    extern __shared__ float4 xs_smem4[];
    float2 *sbuf = reinterpret_cast<float2 *>(xs_smem4);
    auto tileA = [&](int st) { return reinterpret_cast<uint8_t *>(sbuf) + (size_t)(st * 2 + 0) * XS_ST * XS_ROWB; };
    auto tileB = [&](int st) { return reinterpret_cast<uint8_t *>(sbuf) + (size_t)(st * 2 + 1) * XS_ST * XS_ROWB; };

    // dual mode (single diagonal super-tile per channel): channels 2b and
    // 2b+1, staged into the A and B buffers; otherwise one (channel, pair)
    const int ch = a.dual ? 2 * (int)blockIdx.x : (int)blockIdx.x / a.npairs;
    const int pr = a.dual ? 0 : (int)blockIdx.x - ch * a.npairs;
    const bool has2 = a.dual && ch + 1 < a.nbatch;
    int I, J;
    pair_index(pr, I, J);
    const bool diag = (I == J);
    const int r0 = I * XS_ST, q0 = J * XS_ST;
    const int nr = min(XS_ST, a.ne - r0), nq = min(XS_ST, a.ne - q0);
    const int nmr = (nr + XS_MT - 1) / XS_MT, nmq = (nq + XS_MT - 1) / XS_MT;
    const int nmt = diag ? nmr * (nmr + 1) / 2 : nmr * nmq;
    const int nmt2 = a.dual ? 2 * nmt : nmt;  // micro-tiles of the block
    const int ksl = min(XS_KC / 2, max(1, XS_THREADS / nmt2));  // K slices (of sample pairs)
    const int tid = threadIdx.x;
    const int mt2 = tid % nmt2, ks = tid / nmt2;
    const int cs = mt2 / nmt, mt = mt2 - cs * nmt;  // channel slot (dual), micro-tile
    const bool active = tid < nmt2 * ksl && (cs == 0 || has2);
    int mi, mj;
    if (diag) {
        pair_index(mt, mi, mj);
    } else {
        mi = mt / nmq;
        mj = mt - mi * nmq;
    }

    const float2 *Xc = a.Xptrs ? a.Xptrs[ch] : a.X + (long)ch * a.xstride;
    const float2 *Xc2 = !has2 ? Xc : (a.Xptrs ? a.Xptrs[ch + 1] : a.X + (long)(ch + 1) * a.xstride);

    // stage chunk k0 into buffer st: 64 element rows of XS_KC samples per operand
    auto stage = [&](int k0, int st) {
        uint8_t *A = tileA(st), *B = tileB(st);
        // rows the micro-tiles read: rows past the operand's last element up to
        // the micro-tile edge are zero-filled, rows beyond it are not staged
        if (a.blocked) {
            // blocks of 8 samples ld apart: every (8-sample block, element) is 64
            // contiguous bytes, copied as four 16-byte pairs; blocks past the input
            // are zero-filled
            for (int idx = tid; idx < (XS_KC / 8) * XS_ST * 4; idx += XS_THREADS) {
                const int q = idx & 3, e = (idx >> 2) & (XS_ST - 1), sbl = idx >> 8;
                const int kk = 8 * sbl + 2 * q;
                const bool kin = k0 + 8 * sbl < a.nsp;
                const long off = (long)((k0 >> 3) + sbl) * a.ld + 2 * q;
                const int dst = xs_off(e, kk);
                const bool ina = kin && e < nr;
                if (e < ((nr + XS_MT - 1) & ~(XS_MT - 1))) {
                    cp_async16(A + dst, ina ? Xc + off + (long)(r0 + e) * 8 : Xc, ina ? 16 : 0);
                    if (has2)  // the second channel's rows go to the B buffer
                        cp_async16(B + dst, ina ? Xc2 + off + (long)(r0 + e) * 8 : Xc2, ina ? 16 : 0);
                }
                if (!has2 && !diag && e < ((nq + XS_MT - 1) & ~(XS_MT - 1))) {
                    const bool inb = kin && e < nq;
                    cp_async16(B + dst, inb ? Xc + off + (long)(q0 + e) * 8 : Xc, inb ? 16 : 0);
                }
            }
        } else {
            // X[k*ld + e]: consecutive threads take consecutive elements of one sample
            for (int idx = tid; idx < XS_KC * XS_ST; idx += XS_THREADS) {
                const int kk = idx / XS_ST, e = idx - kk * XS_ST;
                const long off = (long)(k0 + kk) * a.ld;
                const bool kin = k0 + kk < a.nsp;
                const int dst = xs_off(e, kk);
                const bool ina = kin && e < nr;
                if (e < ((nr + XS_MT - 1) & ~(XS_MT - 1))) {
                    cp_async8(A + dst, ina ? Xc + off + r0 + e : Xc, ina ? 8 : 0);
                    if (has2) cp_async8(B + dst, ina ? Xc2 + off + r0 + e : Xc2, ina ? 8 : 0);
                }
                if (!has2 && !diag && e < ((nq + XS_MT - 1) & ~(XS_MT - 1))) {
                    const bool inb = kin && e < nq;
                    cp_async8(B + dst, inb ? Xc + off + q0 + e : Xc, inb ? 8 : 0);
                }
            }
        }
        cp_async_commit();
    };

    float2 acc[XS_MT][XS_MT];
#pragma unroll
    for (int i = 0; i < XS_MT; i++)
#pragma unroll
        for (int j = 0; j < XS_MT; j++) acc[i][j] = make_float2(0.f, 0.f);

    const int nchunk = (a.nsp + XS_KC - 1) / XS_KC;
    stage(0, 0);
    for (int c = 0; c < nchunk; c++) {
        const int st = c & 1;
        if (c + 1 < nchunk) {
            stage((c + 1) * XS_KC, st ^ 1);
            cp_async_wait1();
        } else {
            cp_async_wait0();
        }
        __syncthreads();
        if (active) {
            const uint8_t *A = cs ? tileB(st) : tileA(st);
            const uint8_t *B = diag ? A : tileB(st);
            for (int kp = ks; kp < XS_KC / 2; kp += ksl) {
                // samples 2 kp and 2 kp + 1 of the micro-tile's 4 rows and 4 columns
                float4 av[XS_MT], bv[XS_MT];
#pragma unroll
                for (int i = 0; i < XS_MT; i++) {
                    av[i] = *reinterpret_cast<const float4 *>(A + xs_off(XS_MT * mi + i, 2 * kp));
                    bv[i] = *reinterpret_cast<const float4 *>(B + xs_off(XS_MT * mj + i, 2 * kp));
                }
#if MDT_XS_F32X2
                // acc += a * conj(b) on (re, im) pairs, one f32x2 fma per term:
                //   acc += (a.re, a.im) * (b.re, b.re);  acc += (a.im, -a.re) * (b.im, b.im)
                // each lane the same fmaf sequence as the scalar form below
#pragma unroll
                for (int h = 0; h < 2; h++) {  // sample 2 kp, then 2 kp + 1
                    float2 a1[XS_MT], a2[XS_MT];
#pragma unroll
                    for (int i = 0; i < XS_MT; i++) {
                        const float ar = h ? av[i].z : av[i].x, ai = h ? av[i].w : av[i].y;
                        a1[i] = make_float2(ar, ai);
                        a2[i] = make_float2(ai, -ar);
                    }
#pragma unroll
                    for (int j = 0; j < XS_MT; j++) {
                        const float br = h ? bv[j].z : bv[j].x, bi = h ? bv[j].w : bv[j].y;
#pragma unroll
                        for (int i = 0; i < XS_MT; i++) {
                            acc[i][j] = __ffma2_rn(a1[i], make_float2(br, br), acc[i][j]);
                            acc[i][j] = __ffma2_rn(a2[i], make_float2(bi, bi), acc[i][j]);
                        }
                    }
                }
#else
#pragma unroll
                for (int i = 0; i < XS_MT; i++)
#pragma unroll
                    for (int j = 0; j < XS_MT; j++) {
                        // acc += a * conj(b), sample 2 kp then 2 kp + 1
                        acc[i][j].x = fmaf(av[i].x, bv[j].x, acc[i][j].x);
                        acc[i][j].x = fmaf(av[i].y, bv[j].y, acc[i][j].x);
                        acc[i][j].y = fmaf(av[i].y, bv[j].x, acc[i][j].y);
                        acc[i][j].y = fmaf(-av[i].x, bv[j].y, acc[i][j].y);
                    }
#pragma unroll
                for (int i = 0; i < XS_MT; i++)
#pragma unroll
                    for (int j = 0; j < XS_MT; j++) {
                        acc[i][j].x = fmaf(av[i].z, bv[j].z, acc[i][j].x);
                        acc[i][j].x = fmaf(av[i].w, bv[j].w, acc[i][j].x);
                        acc[i][j].y = fmaf(av[i].w, bv[j].z, acc[i][j].y);
                        acc[i][j].y = fmaf(-av[i].z, bv[j].w, acc[i][j].y);
                    }
#endif
            }
        }
        __syncthreads();  // buffer st is overwritten by the next stage() call
    }

    // reduce the K slices in a fixed order (slice 0 + 1 + 2 ...)
    if (ksl > 1) {
        float2 *red = sbuf;  // (ksl-1)*nmt*16 < 256*16 complex
        if (active && ks > 0) {
#pragma unroll
            for (int i = 0; i < XS_MT; i++)
#pragma unroll
                for (int j = 0; j < XS_MT; j++) red[((ks - 1) * nmt2 + mt2) * 16 + i * 4 + j] = acc[i][j];
        }
        __syncthreads();
        if (active && ks == 0) {
            for (int s2 = 1; s2 < ksl; s2++) {
#pragma unroll
                for (int i = 0; i < XS_MT; i++)
#pragma unroll
                    for (int j = 0; j < XS_MT; j++) {
                        float2 v = red[((s2 - 1) * nmt2 + mt2) * 16 + i * 4 + j];
                        acc[i][j].x += v.x;
                        acc[i][j].y += v.y;
                    }
            }
        }
    }
    if (!active || ks != 0) return;

    const int cho = ch + cs;  // output channel
    float2 *Vc = a.Vptrs ? a.Vptrs[cho] : a.V + (long)cho * a.vstride;
#pragma unroll
    for (int i = 0; i < XS_MT; i++) {
#pragma unroll
        for (int j = 0; j < XS_MT; j++) {
            const int r = r0 + mi * XS_MT + i, q = q0 + mj * XS_MT + j;
            if (r >= a.ne || q >= a.ne || r < q) continue;
            float2 v = acc[i][j];
            if (r == q) v.y = 0.f;  // autocorrelations are real
            // lower:  V[r,q] = alpha v + beta V[r,q]
            float2 lo = make_float2(a.alpha.x * v.x - a.alpha.y * v.y,
                                    a.alpha.x * v.y + a.alpha.y * v.x);
            long il = (long)q * a.ldv + r;
            if (!a.beta_zero) {
                float2 o = Vc[il];
                lo.x += a.beta.x * o.x - a.beta.y * o.y;
                lo.y += a.beta.x * o.y + a.beta.y * o.x;
            }
            Vc[il] = lo;
            if (r != q) {
                // upper mirror: V[q,r] = alpha conj(v) + beta V[q,r]
                float2 up = make_float2(a.alpha.x * v.x + a.alpha.y * v.y,
                                        -a.alpha.x * v.y + a.alpha.y * v.x);
                long iu = (long)r * a.ldv + q;
                if (!a.beta_zero) {
                    float2 o = Vc[iu];
                    up.x += a.beta.x * o.x - a.beta.y * o.y;
                    up.y += a.beta.x * o.y + a.beta.y * o.x;
                }
                Vc[iu] = up;
            }
        }
    }
}

mdt_status xengine_herm_f32(int ne, long nbatch, int nsp, const float2 *X,
                            const float2 *const *Xptrs, long ld, long xstride, float2 *V,
                            float2 *const *Vptrs, long ldv, long vstride, float2 alpha,
                            float2 beta, bool beta_zero, cudaStream_t stream, int blocked)
{
    if (ne <= 0 || nbatch <= 0) return MDT_SUCCESS;
    XengArgs a;
    a.ne = ne;
    a.nsp = nsp;
    a.nsuper = (int)cdiv(ne, XS_ST);
    a.npairs = a.nsuper * (a.nsuper + 1) / 2;
    a.X = X;
    a.Xptrs = Xptrs;
    a.ld = (blocked && ld == 0) ? (long)ne * 8 : ld;  // blocked: complex64 between 8-sample blocks
    a.xstride = xstride;
    a.V = V;
    a.Vptrs = Vptrs;
    a.ldv = ldv;
    a.vstride = vstride;
    a.alpha = alpha;
    a.beta = beta;
    a.beta_zero = beta_zero ? 1 : 0;
    a.blocked = blocked;
    a.nbatch = nbatch;
    {
        // two channels per block only while both channels' micro-tiles fit the block
        const int nmr = (int)cdiv(ne, XS_MT);
        a.dual = (a.nsuper == 1 && nmr * (nmr + 1) <= XS_THREADS) ? 1 : 0;
    }
    long blocks = a.dual ? (nbatch + 1) / 2 : nbatch * a.npairs;
    if (blocks > 0x7fffffffL) return invalid("xengine: grid too large");
    cudaError_t e = cudaFuncSetAttribute(xengine_herm_f32_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)XS_SMEM);
    if (e != cudaSuccess) return cuda_status(e, "xengine smem attribute");
    xengine_herm_f32_kernel<<<(unsigned)blocks, XS_THREADS, XS_SMEM, stream>>>(a);
    return launch_status("xengine_herm_f32_kernel");
}

// ---------------------------------------------------- general batched CGEMM
// C = alpha op(A) op(B) + beta C, column-major, 16x16 tiles; for the cuBLAS
// argument patterns that are not the Hermitian X-engine.
struct GemmArgs {
    int m, n, k, ta, tb;  // 0 = N, 1 = T, 2 = C
    const float2 *const *A;
    const float2 *const *B;
    float2 *const *C;
    int lda, ldb, ldc;
    float2 alpha, beta;
    int beta_zero;
    int blocked;  // operand layout: 0 = X[k*ld + e]; 1 = XB[k/8][e][k%8] (NE rows per block)
};

__device__ __forceinline__ float2 opval(const float2 *M, int ld, int t, int row, int col)
{
    // element (row, col) of op(M)
    float2 v = (t == 0) ? M[(long)col * ld + row] : M[(long)row * ld + col];
    if (t == 2) v.y = -v.y;
    return v;
}

__global__ void cgemm_batched_kernel(GemmArgs g)
{
    __shared__ float2 sa[16][17], sb[16][17];
    const int b = blockIdx.z;
    const float2 *A = g.A[b], *B = g.B[b];
    float2 *C = g.C[b];
    const int i = blockIdx.x * 16 + threadIdx.x, j = blockIdx.y * 16 + threadIdx.y;
    float2 acc = make_float2(0.f, 0.f);
    for (int l0 = 0; l0 < g.k; l0 += 16) {
        int ar = blockIdx.x * 16 + threadIdx.x, ac = l0 + threadIdx.y;
        sa[threadIdx.y][threadIdx.x] =
            (ar < g.m && ac < g.k) ? opval(A, g.lda, g.ta, ar, ac) : make_float2(0.f, 0.f);
        int br = l0 + threadIdx.x, bc = blockIdx.y * 16 + threadIdx.y;
        sb[threadIdx.y][threadIdx.x] =
            (br < g.k && bc < g.n) ? opval(B, g.ldb, g.tb, br, bc) : make_float2(0.f, 0.f);
        __syncthreads();
#pragma unroll
        for (int l = 0; l < 16; l++) {
            float2 x = sa[l][threadIdx.x], y = sb[threadIdx.y][l];
            acc.x = fmaf(x.x, y.x, acc.x);
            acc.x = fmaf(-x.y, y.y, acc.x);
            acc.y = fmaf(x.x, y.y, acc.y);
            acc.y = fmaf(x.y, y.x, acc.y);
        }
        __syncthreads();
    }
    if (i < g.m && j < g.n) {
        float2 r = make_float2(g.alpha.x * acc.x - g.alpha.y * acc.y,
                               g.alpha.x * acc.y + g.alpha.y * acc.x);
        long ic = (long)j * g.ldc + i;
        if (!g.beta_zero) {
            float2 o = C[ic];
            r.x += g.beta.x * o.x - g.beta.y * o.y;
            r.y += g.beta.x * o.y + g.beta.y * o.x;
        }
        C[ic] = r;
    }
}

}  // namespace mdt

// ---------------------------------------------------------------- C ABI
extern "C" {

MDT_API mdt_status mdt_xengine_f32(int ne, int nch, int nsp, const void *X, long ld,
                                   long xstride, float alpha, void *V, cudaStream_t stream)
{
    if (!X || !V || ne <= 0 || nch < 0 || nsp < 0 || ld < ne)
        return mdt::invalid("xengine_f32: bad arguments");
    return mdt::xengine_herm_f32(ne, nch, nsp, (const float2 *)X, nullptr, ld, xstride,
                                 (float2 *)V, nullptr, ne, (long)ne * ne,
                                 make_float2(alpha, 0.f), make_float2(0.f, 0.f), true, stream, 0);
}

}  // extern "C"

// cuBLAS handle of the shim: only the stream is kept.
struct cublasContext {
    unsigned magic;
    cudaStream_t stream;
};
static const unsigned kShimMagic = 0x4d445446u;  // "MDTF"

extern "C" {

// cublasCreate (reference MDT_OneStation_client.cu:690)
cublasStatus_t CUBLASWINAPI cublasCreate_v2(cublasHandle_t *handle)
{
    if (!handle) return CUBLAS_STATUS_INVALID_VALUE;
    cublasContext *c = new (std::nothrow) cublasContext;
    if (!c) return CUBLAS_STATUS_ALLOC_FAILED;
    c->magic = kShimMagic;
    c->stream = 0;
    *handle = c;
    return CUBLAS_STATUS_SUCCESS;
}

cublasStatus_t CUBLASWINAPI cublasDestroy_v2(cublasHandle_t handle)
{
    if (!handle || handle->magic != kShimMagic) return CUBLAS_STATUS_NOT_INITIALIZED;
    handle->magic = 0;
    delete handle;
    return CUBLAS_STATUS_SUCCESS;
}

// cublasSetStream (reference :699)
cublasStatus_t CUBLASWINAPI cublasSetStream_v2(cublasHandle_t handle, cudaStream_t streamId)
{
    if (!handle || handle->magic != kShimMagic) return CUBLAS_STATUS_NOT_INITIALIZED;
    handle->stream = streamId;
    return CUBLAS_STATUS_SUCCESS;
}

cublasStatus_t CUBLASWINAPI cublasGetStream_v2(cublasHandle_t handle, cudaStream_t *streamId)
{
    if (!handle || handle->magic != kShimMagic) return CUBLAS_STATUS_NOT_INITIALIZED;
    if (!streamId) return CUBLAS_STATUS_INVALID_VALUE;
    *streamId = handle->stream;
    return CUBLAS_STATUS_SUCCESS;
}

// cublasCgemmBatched (reference :1128).  alpha/beta are host pointers (the
// default pointer mode).  transa = N, transb = C, m == n, Aarray == Barray,
// lda == ldb selects the Hermitian X-engine; any other pattern runs the
// general batched CGEMM.
cublasStatus_t CUBLASWINAPI cublasCgemmBatched(cublasHandle_t handle, cublasOperation_t transa,
                                               cublasOperation_t transb, int m, int n, int k,
                                               const cuComplex *alpha,
                                               const cuComplex *const Aarray[], int lda,
                                               const cuComplex *const Barray[], int ldb,
                                               const cuComplex *beta,
                                               cuComplex *const Carray[], int ldc,
                                               int batchCount)
{
    if (!handle || handle->magic != kShimMagic) return CUBLAS_STATUS_NOT_INITIALIZED;
    auto opcode = [](cublasOperation_t t) {
        return t == CUBLAS_OP_N ? 0 : t == CUBLAS_OP_T ? 1 : t == CUBLAS_OP_C ? 2 : -1;
    };
    int ta = opcode(transa), tb = opcode(transb);
    if (ta < 0 || tb < 0) return CUBLAS_STATUS_INVALID_VALUE;
    if (m < 0 || n < 0 || k < 0 || batchCount < 0 || !alpha || !beta)
        return CUBLAS_STATUS_INVALID_VALUE;
    if (lda < std::max(1, ta == 0 ? m : k) || ldb < std::max(1, tb == 0 ? k : n) ||
        ldc < std::max(1, m))
        return CUBLAS_STATUS_INVALID_VALUE;
    if (m == 0 || n == 0 || batchCount == 0) return CUBLAS_STATUS_SUCCESS;
    if (!Aarray || !Barray || !Carray) return CUBLAS_STATUS_INVALID_VALUE;
    float2 al = make_float2(alpha->x, alpha->y), be = make_float2(beta->x, beta->y);
    bool beta_zero = (be.x == 0.f && be.y == 0.f);
    mdt_status st;
    if (ta == 0 && tb == 2 && m == n && (const void *)Aarray == (const void *)Barray &&
        lda == ldb) {
        st = mdt::xengine_herm_f32(m, batchCount, k, nullptr,
                                   reinterpret_cast<const float2 *const *>(Aarray), lda, 0,
                                   nullptr, reinterpret_cast<float2 *const *>(Carray), ldc, 0,
                                   al, be, beta_zero, handle->stream, 0);
    } else {
        if (batchCount > 65535) return CUBLAS_STATUS_NOT_SUPPORTED;
        mdt::GemmArgs g;
        g.m = m; g.n = n; g.k = k; g.ta = ta; g.tb = tb;
        g.A = reinterpret_cast<const float2 *const *>(Aarray);
        g.B = reinterpret_cast<const float2 *const *>(Barray);
        g.C = reinterpret_cast<float2 *const *>(Carray);
        g.lda = lda; g.ldb = ldb; g.ldc = ldc;
        g.alpha = al; g.beta = be; g.beta_zero = beta_zero;
        dim3 grid((unsigned)mdt::cdiv(m, 16), (unsigned)mdt::cdiv(n, 16), (unsigned)batchCount);
        mdt::cgemm_batched_kernel<<<grid, dim3(16, 16), 0, handle->stream>>>(g);
        st = mdt::launch_status("cgemm_batched_kernel");
    }
    return st == MDT_SUCCESS ? CUBLAS_STATUS_SUCCESS : CUBLAS_STATUS_EXECUTION_FAILED;
}

}  // extern "C"
