// adjoint.cu -- hand-written adjoint kernels of the FX path, for gradients
// through the correlator (gain calibration, PFB tap optimisation).
//
// Gradients follow the convention of PyTorch for complex tensors: for a real
// loss L and complex z, grad(z) = dL/dRe(z) + i dL/dIm(z) = 2 dL/dconj(z).
//
// * X-engine: V_c = Y_c Y_c^H / Nsp (Y_c = NE x Nsp, stored Y[c][s][e]).
//   grad(Y_c) = (G_c + G_c^H) Y_c / Nsp with G = grad(V) in the visibility
//   layout (column-major per channel: G[c][q*NE + r] = G_rq).
// * F-engine: X = DFT(P), P[s][e][k] = sum_i W[i][k] in[s+i][e][k] with real
//   taps W.  grad(P) = DFT^H grad(X) (the unnormalised inverse FFT, done with
//   mdt_fft_c2c direction +1) and
//   grad(W)[i][k] = sum_{s,e} Re(grad(P)[s][e][k] * conj(in[s+i][e][k])).
#include <algorithm>

#include "mdt_common.cuh"

namespace mdt {

// Y[c][s][e] = g[c][e] * X[c][s][e] (complex gains on the F-engine output).
__global__ void apply_gains_kernel(long n, int ne, int nsp, const float2 *__restrict__ X,
                                   const float2 *__restrict__ g, float2 *__restrict__ Y)
{
    const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const long e = j % ne, c = j / ((long)nsp * ne);
    Y[j] = cmul(g[c * ne + e], X[j]);
}

// dg[c][e] = sum_s dY[c][s][e] * conj(X[c][s][e]).  32 (c, e) pairs per block,
// 8 spectrum phases per pair summed in double and combined in a fixed order.
__global__ void gain_grad_kernel(int ne, int nch, int nsp, const float2 *__restrict__ dY,
                                 const float2 *__restrict__ X, float2 *__restrict__ dg)
{
    __shared__ double sre[8][33], sim[8][33];
    const long j = (long)blockIdx.x * 32 + threadIdx.x;
    const int ph = threadIdx.y;
    double re = 0.0, im = 0.0;
    if (j < (long)nch * ne) {
        const long c = j / ne, e = j - c * ne;
        const long base = c * nsp * (long)ne + e;
        for (int s = ph; s < nsp; s += 8) {
            const float2 a = dY[base + (long)s * ne], b = X[base + (long)s * ne];
            re += (double)a.x * b.x + (double)a.y * b.y;
            im += (double)a.y * b.x - (double)a.x * b.y;
        }
    }
    sre[ph][threadIdx.x] = re;
    sim[ph][threadIdx.x] = im;
    __syncthreads();
    if (ph == 0 && j < (long)nch * ne) {
        for (int p = 1; p < 8; p++) {
            re += sre[p][threadIdx.x];
            im += sim[p][threadIdx.x];
        }
        dg[j] = make_float2((float)re, (float)im);
    }
}

// Adjoint of the gains and of the channel-major reorder:
// dF[s][e][c] = conj(g[c][e]) * dY[c][s][e] -- a 32 x 32 tiled transpose of
// (channel) x (spectrum, element) rows.
__global__ void fout_adjoint_kernel(int ne, int nch, long rows, const float2 *__restrict__ dY,
                                    const float2 *__restrict__ g, float2 *__restrict__ dF)
{
    __shared__ float2 t[32][33];
    const long r0 = (long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int c = c0 + y;
        const long r = r0 + threadIdx.x;
        float2 v = make_float2(0.f, 0.f);
        if (c < nch && r < rows) {
            const float2 gv = g ? g[(long)c * ne + r % ne] : make_float2(1.f, 0.f);
            v = cmul(cconj(gv), dY[(long)c * rows + r]);
        }
        t[y][threadIdx.x] = v;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += 8) {
        const long r = r0 + y;
        const int c = c0 + threadIdx.x;
        if (c < nch && r < rows) dF[r * nch + c] = t[threadIdx.x][y];
    }
}

// dY[c][s][r] = scale * sum_q (G_rq + conj(G_qr)) Y[c][s][q]; 16x16 tiles of
// (s, r), K loop over q through shared memory.
__global__ void xengine_adjoint_kernel(int ne, int nsp, const float2 *__restrict__ G,
                                       const float2 *__restrict__ Y, float2 *__restrict__ dY,
                                       float scale)
{
    __shared__ float2 sy[16][17], sh[16][17];
    const int c = blockIdx.z;
    const float2 *Gc = G + (long)c * ne * ne;
    const float2 *Yc = Y + (long)c * nsp * ne;
    const int s = blockIdx.y * 16 + threadIdx.y;
    const int r = blockIdx.x * 16 + threadIdx.x;
    float2 acc = make_float2(0.f, 0.f);
    for (int q0 = 0; q0 < ne; q0 += 16) {
        // sy[ty][tx] = Y[s = s0 + ty][q = q0 + tx]
        const int qy = q0 + threadIdx.x;
        sy[threadIdx.y][threadIdx.x] =
            (s < nsp && qy < ne) ? Yc[(long)s * ne + qy] : make_float2(0.f, 0.f);
        // sh[ty][tx] = H[r = r0 + tx][q = q0 + ty] = G_rq + conj(G_qr)
        const int rh = blockIdx.x * 16 + threadIdx.x, qh = q0 + threadIdx.y;
        float2 h = make_float2(0.f, 0.f);
        if (rh < ne && qh < ne) {
            const float2 a = Gc[(long)qh * ne + rh];  // G_rq (column-major)
            const float2 b = Gc[(long)rh * ne + qh];  // G_qr
            h = make_float2(a.x + b.x, a.y - b.y);
        }
        sh[threadIdx.y][threadIdx.x] = h;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const float2 y = sy[threadIdx.y][k], hv = sh[k][threadIdx.x];
            acc.x = fmaf(hv.x, y.x, acc.x);
            acc.x = fmaf(-hv.y, y.y, acc.x);
            acc.y = fmaf(hv.x, y.y, acc.y);
            acc.y = fmaf(hv.y, y.x, acc.y);
        }
        __syncthreads();
    }
    if (s < nsp && r < ne) dY[((long)c * nsp + s) * ne + r] = make_float2(acc.x * scale, acc.y * scale);
}

// Partial tap gradients: split p of the (spectrum, element) rows.
// part[p][i][k] = sum over the split's rows (s, e) of
//                 Re(gP[s][e][k] * conj(in[s+i][e][k])), accumulated in double.
__global__ void pfb_tap_grad_partial_kernel(int nch, int ntaps, int ne, int nsp, int nsplit,
                                            const float2 *__restrict__ gP,
                                            const char2 *__restrict__ iq,
                                            double *__restrict__ part)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    const int p = blockIdx.z;
    if (k >= nch) return;
    const long rows = (long)nsp * ne;
    const long r0 = rows * p / nsplit, r1 = rows * (p + 1) / nsplit;
    double acc = 0.0;
    for (long row = r0; row < r1; row++) {
        const long s = row / ne, e = row - s * ne;
        const float2 g = gP[row * nch + k];
        const char2 x = iq[((s + i) * ne + e) * nch + k];
        acc += (double)g.x * (double)x.x + (double)g.y * (double)x.y;
    }
    part[((long)p * ntaps + i) * nch + k] = acc;
}

// All taps at once (Ntaps <= 16): gP is read once, the int8 input of the
// NT taps from L2.  part[p][i][k] as above.
template <int NT>
__global__ void pfb_tap_grad_all_kernel(int nch, int ne, int nsp, int nsplit,
                                        const float2 *__restrict__ gP,
                                        const char2 *__restrict__ iq, double *__restrict__ part)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int p = blockIdx.y;
    if (k >= nch) return;
    const long rows = (long)nsp * ne;
    const long r0 = rows * p / nsplit, r1 = rows * (p + 1) / nsplit;
    double acc[NT];
#pragma unroll
    for (int i = 0; i < NT; i++) acc[i] = 0.0;
    for (long row = r0; row < r1; row++) {
        const long s = row / ne, e = row - s * ne;
        const float2 g = gP[row * nch + k];
#pragma unroll
        for (int i = 0; i < NT; i++) {
            const char2 x = iq[((s + i) * ne + e) * nch + k];
            acc[i] += (double)g.x * (double)x.x + (double)g.y * (double)x.y;
        }
    }
#pragma unroll
    for (int i = 0; i < NT; i++) part[((long)p * NT + i) * nch + k] = acc[i];
}

// gW[i][k] = sum_p part[p][i][k] in increasing p (deterministic).
__global__ void pfb_tap_grad_reduce_kernel(int n, int nsplit, const double *__restrict__ part,
                                           float *__restrict__ gW)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double acc = 0.0;
    for (int p = 0; p < nsplit; p++) acc += part[(long)p * n + j];
    gW[j] = (float)acc;
}

}  // namespace mdt

extern "C" {

MDT_API mdt_status mdt_xengine_adjoint_f32(int ne, int nch, int nsp, const void *G, const void *Y,
                                           void *dY, float scale, cudaStream_t stream)
{
    if (!G || !Y || !dY || ne < 1 || nch < 1 || nsp < 1 || nch > 65535)
        return mdt::invalid("xengine_adjoint_f32: bad arguments");
    dim3 grid((unsigned)mdt::cdiv(ne, 16), (unsigned)mdt::cdiv(nsp, 16), (unsigned)nch);
    if (grid.y > 65535) return mdt::invalid("xengine_adjoint_f32: Nsp too large");
    mdt::xengine_adjoint_kernel<<<grid, dim3(16, 16), 0, stream>>>(
        ne, nsp, (const float2 *)G, (const float2 *)Y, (float2 *)dY, scale);
    return mdt::launch_status("xengine_adjoint_kernel");
}

MDT_API mdt_status mdt_apply_gains(int ne, int nch, int nsp, const void *X, const void *gains,
                                   void *Y, cudaStream_t stream)
{
    if (!X || !gains || !Y || ne < 1 || nch < 1 || nsp < 1)
        return mdt::invalid("apply_gains: bad arguments");
    const long n = (long)nch * nsp * ne;
    mdt::apply_gains_kernel<<<(unsigned)mdt::cdiv(n, 256), 256, 0, stream>>>(
        n, ne, nsp, (const float2 *)X, (const float2 *)gains, (float2 *)Y);
    return mdt::launch_status("apply_gains_kernel");
}

MDT_API mdt_status mdt_gain_adjoint(int ne, int nch, int nsp, const void *dY, const void *X,
                                    const void *gains, void *dgains, void *dF,
                                    cudaStream_t stream)
{
    if (!dY || ne < 1 || nch < 1 || nsp < 1 || nch > 65535 * 32)
        return mdt::invalid("gain_adjoint: bad arguments");
    if (dgains) {
        if (!X) return mdt::invalid("gain_adjoint: X is needed for the gain gradient");
        mdt::gain_grad_kernel<<<(unsigned)mdt::cdiv((long)nch * ne, 32), dim3(32, 8), 0, stream>>>(
            ne, nch, nsp, (const float2 *)dY, (const float2 *)X, (float2 *)dgains);
        mdt_status st = mdt::launch_status("gain_grad_kernel");
        if (st != MDT_SUCCESS) return st;
    }
    if (dF) {
        const long rows = (long)nsp * ne;
        dim3 grid((unsigned)mdt::cdiv(rows, 32), (unsigned)mdt::cdiv(nch, 32));
        mdt::fout_adjoint_kernel<<<grid, dim3(32, 8), 0, stream>>>(
            ne, nch, rows, (const float2 *)dY, (const float2 *)gains, (float2 *)dF);
        return mdt::launch_status("fout_adjoint_kernel");
    }
    return MDT_SUCCESS;
}

MDT_API mdt_status mdt_pfb_tap_grad(int ne, int nch, int ntaps, int nsp, const void *gradP,
                                    const int8_t *iq, float *gradW, void *workspace,
                                    size_t workspace_bytes, cudaStream_t stream)
{
    if (!gradP || !iq || !gradW || !workspace || ne < 1 || nch < 1 || ntaps < 1 || nsp < 1 ||
        ntaps > 65535)
        return mdt::invalid("pfb_tap_grad: bad arguments");
    const long n = (long)ntaps * nch;
    int nsplit = (int)std::min<long>(64, std::max<long>(1, workspace_bytes / (sizeof(double) * n)));
    if (nsplit < 1 || workspace_bytes < sizeof(double) * n)
        return mdt::invalid("pfb_tap_grad: workspace must hold Ntaps*Nch doubles");
    mdt_status st;
    if (ntaps == 4 || ntaps == 8) {
        dim3 grid((unsigned)mdt::cdiv(nch, 128), (unsigned)nsplit);
        if (ntaps == 4)
            mdt::pfb_tap_grad_all_kernel<4><<<grid, 128, 0, stream>>>(
                nch, ne, nsp, nsplit, (const float2 *)gradP, (const char2 *)iq, (double *)workspace);
        else
            mdt::pfb_tap_grad_all_kernel<8><<<grid, 128, 0, stream>>>(
                nch, ne, nsp, nsplit, (const float2 *)gradP, (const char2 *)iq, (double *)workspace);
        st = mdt::launch_status("pfb_tap_grad_all_kernel");
    } else {
        dim3 grid((unsigned)mdt::cdiv(nch, 128), (unsigned)ntaps, (unsigned)nsplit);
        mdt::pfb_tap_grad_partial_kernel<<<grid, 128, 0, stream>>>(
            nch, ntaps, ne, nsp, nsplit, (const float2 *)gradP, (const char2 *)iq,
            (double *)workspace);
        st = mdt::launch_status("pfb_tap_grad_partial_kernel");
    }
    if (st != MDT_SUCCESS) return st;
    mdt::pfb_tap_grad_reduce_kernel<<<(unsigned)mdt::cdiv(n, 256), 256, 0, stream>>>(
        (int)n, nsplit, (const double *)workspace, gradW);
    return mdt::launch_status("pfb_tap_grad_reduce_kernel");
}

}  // extern "C"
