"""FP64 references for the adjoint tests (test infrastructure).

fx64: the FX forward (PFB tap sum -> FFT e^{-2 pi i} -> channel-major
reorder -> gains -> V = Y Y^H / Nsp) in PyTorch float64 on the CPU, whose
autograd gradient is the FP64 reference gradient.  fd_*: FP64 central
finite differences of L = Re sum conj(C) V on the FP64 oracle's pipeline
(oracle.fx), exact up to FP64 rounding because V is quadratic in each tap and
bilinear in (g, conj g)."""
import numpy as np
import torch


def crandn(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def fx64(iq, W, g, ne, nch, ntaps, nsp):
    """V[c, q, r] = (1/Nsp) sum_s Y[c,s,r] conj(Y[c,s,q]) in float64."""
    x = torch.from_numpy(iq.astype(np.float64).reshape(nsp + ntaps - 1, ne, nch, 2))
    x = torch.complex(x[..., 0], x[..., 1])
    W = W.reshape(ntaps, nch)
    P = sum(W[i][None, None, :] * x[i:i + nsp] for i in range(ntaps))
    F = torch.fft.fft(P, dim=-1)              # [s][e][c]
    X = F.permute(2, 0, 1)                    # [c][s][e]
    Y = g[:, None, :] * X
    return torch.einsum("csr,csq->cqr", Y, Y.conj()) / nsp


def make_case(oracle, ne=6, nch=64, ntaps=4, nsp=40, seed=11):
    """int8 I/Q, perturbed float32 window, gains, and loss weights C."""
    rng = np.random.default_rng(seed)
    iq = oracle.synth_iq(seed, ne, nch, 0, nsp + ntaps - 1, np.full(ne, 16 * 256, np.int32))
    W = (oracle.window_hamming_sinc(nch, ntaps) *
         rng.uniform(0.5, 1.5, nch * ntaps)).astype(np.float32)
    g = (rng.uniform(0.8, 1.2, (nch, ne)) *
         np.exp(1j * rng.uniform(-np.pi, np.pi, (nch, ne)))).astype(np.complex64)
    C = crandn(rng, nch, ne, ne)  # L = Re sum conj(C) V, so grad(V) = C
    return iq, W, g, C


def reference_gradient(iq, W, g, C, ne, nch, ntaps, nsp):
    """(V, grad W, grad g) from float64 autograd of fx64."""
    Wt = torch.from_numpy(W.astype(np.float64)).requires_grad_(True)
    gt = torch.from_numpy(g.astype(np.complex128)).requires_grad_(True)
    V = fx64(iq, Wt, gt, ne, nch, ntaps, nsp)
    V.backward(torch.from_numpy(C))
    return V.detach().numpy(), Wt.grad.numpy(), gt.grad.numpy()


def _loss(oracle, iq, W, g, C, ne, nch, ntaps, nsp):
    V0 = oracle.fx(iq, W, ne, nch, ntaps, nsp)           # [c][q][r], FP64
    V = g[:, None, :] * np.conj(g)[:, :, None] * V0      # g_r conj(g_q) V0_rq
    return float(np.sum(np.real(np.conj(C) * V)))


def fd_taps(oracle, iq, W, g, C, ne, nch, ntaps, nsp, idx):
    """FP64 central differences dL/dW_j for j in idx (float32 steps)."""
    g = g.astype(np.complex128)
    out = []
    for j in idx:
        h = np.float32(1e-2 * max(abs(W[j]), 1e-3))
        Wp, Wm = W.copy(), W.copy()
        Wp[j] += h
        Wm[j] -= h
        d = float(Wp[j]) - float(Wm[j])  # the float32 step actually taken
        out.append((_loss(oracle, iq, Wp, g, C, ne, nch, ntaps, nsp) -
                    _loss(oracle, iq, Wm, g, C, ne, nch, ntaps, nsp)) / d)
    return np.array(out)


def fd_gains(oracle, iq, W, g, C, ne, nch, ntaps, nsp, idx, h=1e-4):
    """FP64 central differences dL/dRe g + i dL/dIm g at (c, e) in idx."""
    V0 = oracle.fx(iq, W, ne, nch, ntaps, nsp)
    g = g.astype(np.complex128)
    out = []
    for (c, e) in idx:
        def lc(gx):
            V = gx[c][None, :] * np.conj(gx[c])[:, None] * V0[c]
            return float(np.sum(np.real(np.conj(C[c]) * V)))
        z = 0j
        for unit in (1.0, 1j):
            gp, gm = g.copy(), g.copy()
            gp[c, e] += h * unit
            gm[c, e] -= h * unit
            z += unit * (lc(gp) - lc(gm)) / (2 * h)
        out.append(z)
    return np.array(out)
