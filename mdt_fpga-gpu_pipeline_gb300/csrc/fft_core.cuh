// fft_core.cuh -- shared-memory Stockham FFT core (forward, unnormalised,
// natural order in and out), used by the standalone batched FFT (the
// cufftExecC2C replacement) and by the fused F-engine.
//
// One row of N = 2^L complex values is transformed by TPR threads through
// L/4 radix-16 passes and, when L is not a multiple of 4, one final radix-2,
// radix-4 or radix-8 pass.  Pass p (radix R, NS = 16^p) on butterfly b:
//   v[m]  = x[b + m*N/R]                              m = 0..R-1
//   v[m] *= exp(-2 pi i m (b mod NS) / (NS*R))        (table lookup)
//   v     = DFT_R(v)
//   y[(b/NS)*NS*R + (b mod NS) + m*NS] = v[m]
// which is the self-sorting (Stockham) formulation: the first pass reads the
// row in natural order and the last pass writes it in natural order, so the
// first pass can take its inputs from any producer (global memory, the PFB
// tap sum) and the last pass can hand its outputs to any consumer.
// Intermediate passes exchange through shared memory as interleaved float2
// (one 8-byte access per complex value) at padded index i + i/16, which
// keeps every pass's warp accesses at the minimum two wavefronts for the
// strides the passes use.
// All arithmetic uses explicitly rounded intrinsics so every instantiation
// of the core produces bit-identical results.
#pragma once
#include "mdt_common.cuh"

// Radix-8 / radix-16 twiddles: 0 = one table load per power; 1 = loads of
// w, w^2, w^4 (and w^8) and the other powers as complex products (fewer load
// instructions, a few ulp more rounding).
#ifndef MDT_FFT_TW_PRODUCTS
#define MDT_FFT_TW_PRODUCTS 1
#endif

namespace mdt {
namespace fft {

constexpr int clog2(int n) { return n <= 1 ? 0 : 1 + clog2(n / 2); }
constexpr int ipow16(int p) { return p == 0 ? 1 : 16 * ipow16(p - 1); }

__host__ __device__ constexpr int pad(int i) { return i + (i >> 4); }

template <int N>
struct Shape {
    static constexpr int L = clog2(N);
    static constexpr int P16 = L / 4;    // radix-16 passes
    static constexpr int REM = L % 4;    // final radix-2^REM pass if REM > 0
    static constexpr int NPASS = P16 + (REM ? 1 : 0);
    static constexpr int TPR = (N / 8 < 1) ? 1 : ((N / 8 > 1024) ? 1024 : N / 8);  // threads per row
    static constexpr int PADN = pad(N);  // float2 slots of one padded row
};

constexpr float kRsqrt2 = 0.70710678118654752440f;

// Complex add, subtract and multiply on packed FP32 pairs (the f32x2
// add / multiply / fma instructions of sm_100 and later, one instruction
// for both lanes).  Each lane is rounded exactly as the scalar helpers of
// mdt_common.cuh round it (x - y = x + (-y) and round(-x) = -round(x) under
// round-to-nearest-even), so either form gives bit-identical transforms.
#ifndef MDT_FFT_F32X2
#define MDT_FFT_F32X2 1
#endif
__device__ __forceinline__ float2 padd(float2 a, float2 b)
{
#if MDT_FFT_F32X2
    return __fadd2_rn(a, b);
#else
    return cadd(a, b);
#endif
}
__device__ __forceinline__ float2 psub(float2 a, float2 b)
{
#if MDT_FFT_F32X2
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
#else
    return csub(a, b);
#endif
}
// a * b: (-a.y b.y, a.y b.x) + a.x (b.x, b.y), the roundings of cmul
__device__ __forceinline__ float2 pcmul(float2 a, float2 b)
{
#if MDT_FFT_F32X2
    const float2 p = __fmul2_rn(make_float2(a.y, a.y), make_float2(-b.y, b.x));
    return __ffma2_rn(make_float2(a.x, a.x), b, p);
#else
    return cmul(a, b);
#endif
}

// Compact twiddle table: the entries of exp(-2 pi i k / N) that pass p >= 1
// reads, stored per pass as [slot][jm] (jm = butterfly mod NS), so a warp's
// loads of one slot fall on consecutive entries.  The slots are the powers
// the pass loads: w, w^2, w^4 (and w^8) for radix 8 (16) with
// MDT_FFT_TW_PRODUCTS, else w^1 .. w^(R-1).  Entry values are copies of the
// device table, so both sources give bit-identical transforms.
template <int N>
__host__ __device__ constexpr int pass_radix(int p)
{
    return p < Shape<N>::P16 ? 16 : 1 << Shape<N>::REM;
}
__host__ __device__ constexpr int tw_slots(int r)
{
    return (MDT_FFT_TW_PRODUCTS && r == 16) ? 4 : ((MDT_FFT_TW_PRODUCTS && r == 8) ? 3 : r - 1);
}
// power of slot `slot` for radix r
__host__ __device__ constexpr int tw_slot_power(int r, int slot)
{
    return (MDT_FFT_TW_PRODUCTS && (r == 16 || r == 8)) ? 1 << slot : slot + 1;
}
template <int N>
__host__ __device__ constexpr int tw_off(int p)
{
    return p <= 1 ? 0 : tw_off<N>(p - 1) + ipow16(p - 1) * tw_slots(pass_radix<N>(p - 1));
}
// float2 entries of the compact table (at least 1)
template <int N>
__host__ __device__ constexpr int tw_compact_len()
{
    return tw_off<N>(Shape<N>::NPASS) > 0 ? tw_off<N>(Shape<N>::NPASS) : 1;
}

// Copies the compact table from the device table `tw` into `dst` (shared
// memory); thread `tid` of `nthreads`.  The caller synchronises before the
// first pass that reads it.
template <int N>
__device__ __forceinline__ void fill_tw_compact(float2 *dst, const float2 *__restrict__ tw, int tid,
                                                int nthreads)
{
#pragma unroll
    for (int p = 1; p < Shape<N>::NPASS; p++) {
        const int r = pass_radix<N>(p), ns = ipow16(p), ts = N / (ns * r);
        const int n = ns * tw_slots(r);
        for (int i = tid; i < n; i += nthreads) {
            const int slot = i / ns, jm = i - slot * ns;
            dst[tw_off<N>(p) + i] = __ldg(&tw[tw_slot_power(r, slot) * jm * ts]);
        }
    }
}

template <int R>
__device__ __forceinline__ void dft(float2 *v);

template <>
__device__ __forceinline__ void dft<1>(float2 *)
{
}

template <>
__device__ __forceinline__ void dft<2>(float2 *v)
{
    float2 a = padd(v[0], v[1]), b = psub(v[0], v[1]);
    v[0] = a;
    v[1] = b;
}

// y_k = sum_n x_n (-i)^{nk}
__device__ __forceinline__ void dft4v(float2 &x0, float2 &x1, float2 &x2, float2 &x3)
{
    float2 c0 = padd(x0, x2), c1 = psub(x0, x2);
    float2 c2 = padd(x1, x3), c3 = cmul_mi(psub(x1, x3));
    x0 = padd(c0, c2);
    x1 = padd(c1, c3);
    x2 = psub(c0, c2);
    x3 = psub(c1, c3);
}

template <>
__device__ __forceinline__ void dft<4>(float2 *v)
{
    dft4v(v[0], v[1], v[2], v[3]);
}

// v * (1 - i)/sqrt2 and v * (-1 - i)/sqrt2 (W16^2 and W16^6):
//   ((x + y) r, (y - x) r)  and  ((y - x) r, -((x + y) r)),  r = 1/sqrt2
__device__ __forceinline__ float2 mul_w8(float2 b)
{
#if MDT_FFT_F32X2
    return __fmul2_rn(__fadd2_rn(b, make_float2(b.y, -b.x)), make_float2(kRsqrt2, kRsqrt2));
#else
    return make_float2(__fmul_rn(__fadd_rn(b.x, b.y), kRsqrt2), __fmul_rn(__fsub_rn(b.y, b.x), kRsqrt2));
#endif
}
__device__ __forceinline__ float2 mul_w8_3(float2 b)
{
#if MDT_FFT_F32X2
    return __fmul2_rn(__fadd2_rn(make_float2(b.y, b.x), make_float2(-b.x, b.y)),
                      make_float2(kRsqrt2, -kRsqrt2));
#else
    return make_float2(__fmul_rn(__fsub_rn(b.y, b.x), kRsqrt2), -__fmul_rn(__fadd_rn(b.x, b.y), kRsqrt2));
#endif
}

// Radix-8 by one decimation-in-frequency split into two radix-4 DFTs:
//   y_{2k}   = DFT4(v_n + v_{n+4})_k
//   y_{2k+1} = DFT4((v_n - v_{n+4}) W8^n)_k,   W8 = exp(-2 pi i/8)
template <>
__device__ __forceinline__ void dft<8>(float2 *v)
{
    float2 a0 = padd(v[0], v[4]), a1 = padd(v[1], v[5]), a2 = padd(v[2], v[6]),
           a3 = padd(v[3], v[7]);
    float2 b0 = psub(v[0], v[4]), b1 = psub(v[1], v[5]), b2 = psub(v[2], v[6]),
           b3 = psub(v[3], v[7]);
    // b1 *= (1 - i)/sqrt2 ; b2 *= -i ; b3 *= (-1 - i)/sqrt2
    b1 = mul_w8(b1);
    b2 = cmul_mi(b2);
    b3 = mul_w8_3(b3);
    dft4v(a0, a1, a2, a3);
    dft4v(b0, b1, b2, b3);
    v[0] = a0; v[2] = a1; v[4] = a2; v[6] = a3;
    v[1] = b0; v[3] = b1; v[5] = b2; v[7] = b3;
}

// cos(pi/8), sin(pi/8)
constexpr float kC16 = 0.92387953251128675613f, kS16 = 0.38268343236508977173f;

// Radix-16 as 4 x 4: DFT4 over m1 of v[m2 + 4 m1] for each m2, twiddles
// W16^(m2 q), DFT4 over m2 for each q; output k = q + 4 r is left in
// position 4 q + r and moved to natural order at the end.
template <>
__device__ __forceinline__ void dft<16>(float2 *v)
{
#pragma unroll
    for (int m2 = 0; m2 < 4; m2++) dft4v(v[m2], v[m2 + 4], v[m2 + 8], v[m2 + 12]);
    // v[m2 + 4 q] *= W16^(m2 q),  W16^k = cos(k pi/8) - i sin(k pi/8)
    const float2 w1 = make_float2(kC16, -kS16), w3 = make_float2(kS16, -kC16),
                 w9 = make_float2(-kC16, kS16);
    v[1 + 4] = pcmul(v[1 + 4], w1);     // m2 1, q 1: W^1
    v[1 + 8] = mul_w8(v[1 + 8]);        // m2 1, q 2: W^2
    v[1 + 12] = pcmul(v[1 + 12], w3);   // m2 1, q 3: W^3
    v[2 + 4] = mul_w8(v[2 + 4]);        // m2 2, q 1: W^2
    v[2 + 8] = cmul_mi(v[2 + 8]);       // m2 2, q 2: W^4 = -i
    v[2 + 12] = mul_w8_3(v[2 + 12]);    // m2 2, q 3: W^6
    v[3 + 4] = pcmul(v[3 + 4], w3);     // m2 3, q 1: W^3
    v[3 + 8] = mul_w8_3(v[3 + 8]);      // m2 3, q 2: W^6
    v[3 + 12] = pcmul(v[3 + 12], w9);   // m2 3, q 3: W^9
#pragma unroll
    for (int q = 0; q < 4; q++) dft4v(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    float2 y[16];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
        for (int r = 0; r < 4; r++) y[q + 4 * r] = v[4 * q + r];
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = y[k];
}

// One Stockham pass over one row.  `t` is the thread's index within the row
// (0..TPR-1); every thread of the block must call every pass (barriers).
// LOADFN (pass 0 only): inputs come from load(i) instead of shared memory,
//   so no barrier is needed before the pass writes shared memory.
// STOREFN (last pass only): outputs go to store(i, v) instead of shared memory.
// Padded indices are formed from the pass's compile-time strides where the
// strides are multiples of 16 (pad(x + 16k) = pad(x) + 17k).
// TWS: twiddles from the compact table `tws` (shared memory) instead of the
//   device table `tw`.
template <int N, int TPR, int P, bool LOADFN, bool STOREFN, bool TWS, class Load, class Store>
__device__ __forceinline__ void stockham_pass(float2 *sx, int t,
                                              const float2 *__restrict__ tw, const float2 *tws,
                                              Load &load, Store &store)
{
    constexpr int R = (P < Shape<N>::P16) ? 16 : (1 << Shape<N>::REM);
    constexpr int NS = ipow16(P);
    constexpr int NB = N / R;
    constexpr int NBT = (NB + TPR - 1) / TPR;
    float2 v[NBT][R];
#pragma unroll
    for (int k = 0; k < NBT; k++) {
        const int b = t + k * TPR;
        if (NBT * TPR == NB || b < NB) {
#pragma unroll
            for (int m = 0; m < R; m++) {
                const int idx = b + m * NB;
                if constexpr (LOADFN) {
                    v[k][m] = load(idx);
                } else {
                    const int pi = (NB % 16 == 0) ? pad(b) + m * pad(NB) : pad(idx);
                    v[k][m] = sx[pi];
                }
            }
            if constexpr (NS > 1) {
                const int jm = b & (NS - 1);
                constexpr int TS = N / (NS * R);
                // power tw_slot_power(R, slot) of this butterfly's twiddle
                auto twl = [&](int slot) {
                    if constexpr (TWS)
                        return tws[tw_off<N>(P) + slot * NS + jm];
                    else
                        return __ldg(&tw[tw_slot_power(R, slot) * jm * TS]);
                };
#if MDT_FFT_TW_PRODUCTS
                // radix 8: w, w^2, w^4 from the table, the other powers as products
                if constexpr (R == 8) {
                    const float2 w1 = twl(0), w2 = twl(1), w4 = twl(2);
                    const float2 w3 = pcmul(w1, w2);
                    v[k][1] = pcmul(v[k][1], w1);
                    v[k][2] = pcmul(v[k][2], w2);
                    v[k][3] = pcmul(v[k][3], w3);
                    v[k][4] = pcmul(v[k][4], w4);
                    v[k][5] = pcmul(v[k][5], pcmul(w1, w4));
                    v[k][6] = pcmul(v[k][6], pcmul(w2, w4));
                    v[k][7] = pcmul(v[k][7], pcmul(w3, w4));
                } else if constexpr (R == 16) {
                    // radix 16: w, w^2, w^4, w^8 from the table, the others as products
                    const float2 w1 = twl(0), w2 = twl(1), w4 = twl(2), w8 = twl(3);
                    const float2 w3 = pcmul(w1, w2), w5 = pcmul(w1, w4), w6 = pcmul(w2, w4),
                                 w7 = pcmul(w3, w4);
                    v[k][1] = pcmul(v[k][1], w1);
                    v[k][2] = pcmul(v[k][2], w2);
                    v[k][3] = pcmul(v[k][3], w3);
                    v[k][4] = pcmul(v[k][4], w4);
                    v[k][5] = pcmul(v[k][5], w5);
                    v[k][6] = pcmul(v[k][6], w6);
                    v[k][7] = pcmul(v[k][7], w7);
                    v[k][8] = pcmul(v[k][8], w8);
                    v[k][9] = pcmul(v[k][9], pcmul(w1, w8));
                    v[k][10] = pcmul(v[k][10], pcmul(w2, w8));
                    v[k][11] = pcmul(v[k][11], pcmul(w3, w8));
                    v[k][12] = pcmul(v[k][12], pcmul(w4, w8));
                    v[k][13] = pcmul(v[k][13], pcmul(w5, w8));
                    v[k][14] = pcmul(v[k][14], pcmul(w6, w8));
                    v[k][15] = pcmul(v[k][15], pcmul(w7, w8));
                } else
#endif
                {
#pragma unroll
                    for (int m = 1; m < R; m++) v[k][m] = pcmul(v[k][m], twl(m - 1));
                }
            }
            dft<R>(v[k]);
        }
    }
    if constexpr (!LOADFN) __syncthreads();  // every read of this pass precedes any write
#pragma unroll
    for (int k = 0; k < NBT; k++) {
        const int b = t + k * TPR;
        if (NBT * TPR == NB || b < NB) {
            const int base = (b / NS) * NS * R + (b & (NS - 1));
#pragma unroll
            for (int m = 0; m < R; m++) {
                const int o = base + m * NS;
                if constexpr (STOREFN) {
                    store(o, v[k][m]);
                } else {
                    const int po = (NS % 16 == 0) ? pad(base) + m * pad(NS) : pad(o);
                    sx[po] = v[k][m];
                }
            }
        }
    }
    if constexpr (!STOREFN) __syncthreads();  // writes visible to the next pass
}

template <int N, int TPR, int P, bool LOADFN, bool STOREFN, bool TWS, class Load, class Store>
__device__ __forceinline__ void run_passes(float2 *sx, int t, const float2 *__restrict__ tw,
                                           const float2 *tws, Load &load, Store &store)
{
    constexpr int NP = Shape<N>::NPASS;
    stockham_pass<N, TPR, P, LOADFN && P == 0, STOREFN && P == NP - 1, TWS>(sx, t, tw, tws, load,
                                                                             store);
    if constexpr (P + 1 < NP)
        run_passes<N, TPR, P + 1, LOADFN, STOREFN, TWS>(sx, t, tw, tws, load, store);
}

// Transforms one row: first-pass inputs from load(i) (LOADFN) or from the
// row's shared slots in natural order (then the caller must have written
// them and synchronised), natural-order outputs to store(i, v) (STOREFN) or
// left in shared memory.  sx: the row's Shape<N>::PADN float2 slots,
// element i at pad(i).  TPR threads per row; when TPR < N/8 each thread
// handles several butterflies per pass.
template <int N, int TPR, bool LOADFN, bool STOREFN, class Load, class Store>
__device__ __forceinline__ void transform_row(float2 *sx, int t, const float2 *__restrict__ tw,
                                              Load &load, Store &store)
{
    run_passes<N, TPR, 0, LOADFN, STOREFN, false>(sx, t, tw, nullptr, load, store);
}

// As transform_row, with the twiddles read from the compact table `tws`
// (filled by fill_tw_compact<N> and synchronised before the call).
template <int N, int TPR, bool LOADFN, bool STOREFN, class Load, class Store>
__device__ __forceinline__ void transform_row_tws(float2 *sx, int t, const float2 *tws, Load &load,
                                                  Store &store)
{
    run_passes<N, TPR, 0, LOADFN, STOREFN, true>(sx, t, nullptr, tws, load, store);
}

}  // namespace fft

// Device twiddle table exp(-2 pi i k / n), k < n, built in double on the host
// on first use per (device, n) and kept until process exit.  Must be called
// outside stream capture the first time for a given n.
const float2 *fft_twiddles(int n, mdt_status *st);

}  // namespace mdt
