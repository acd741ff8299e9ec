"""Differentiation through the FX path: torch.autograd.Function over the
library's forward and adjoint kernels, and per-antenna complex-gain
calibration by gradient descent.

Forward (FP32, the plan's arithmetic):
    X = F-engine(iq; taps)      mdt_fengine_f32: PpS_Batch -> FFT -> reorder
                                (reference MDT_device_functions.cu PpS_Batch,
                                MDT_OneStation_client.cu:1083-1114)
    Y = diag(gains) X           mdt_apply_gains, gains [Nch][NE] complex
    V = Y Y^H / Nsp             mdt_xengine_f32 (replaces cublasCgemmBatched,
                                MDT_OneStation_client.cu:1128)
Backward (hand-written adjoints, no PyTorch math on the path):
    dY     = (G + G^H) Y / Nsp          mdt_xengine_adjoint_f32
    dgains = sum_s dY conj(X)           mdt_gain_adjoint
    dF     = reorder^T(conj(g) dY)      mdt_gain_adjoint
    dP     = DFT^H dF                   mdt_fft_c2c(direction=+1)
    dtaps  = sum Re(dP conj(in))        mdt_pfb_tap_grad
The F-engine output is recomputed in the backward pass instead of being kept
from the forward pass (it is Nch*Nsp*NE*8 bytes, the largest tensor here).
Gradients follow PyTorch's complex convention, grad = dL/dRe + i dL/dIm.
"""
import torch

from . import binding as B


def _cplx(n, device):
    return torch.empty(n, dtype=torch.complex64, device=device)


def _fengine(iq, taps, ne, nch, ntaps, nsp):
    X = _cplx(nch * nsp * ne, iq.device)
    B.fengine_f32(ne, nch, ntaps, nsp, iq, taps, X)
    return X


class FxCorrelate(torch.autograd.Function):
    """V[c, q, r] = (1/Nsp) sum_s Y[c,s,r] conj(Y[c,s,q]),  Y = gains * F(iq; taps).

    iq: int8 CUDA tensor of (Nsp + Ntaps - 1) * NE * Nch * 2 values (no gradient);
    taps: float32 [Ntaps * Nch] (window, tap-major); gains: complex64 [Nch, NE].
    Returns complex64 [Nch, NE, NE] (the column-major visibility layout)."""

    @staticmethod
    def forward(ctx, iq, taps, gains, ne, nch, ntaps, nsp):
        if not (iq.is_cuda and taps.is_cuda and gains.is_cuda):
            raise B.MdtError("FxCorrelate: inputs must be CUDA tensors")
        taps = taps.detach().contiguous().to(torch.float32)
        gains = gains.detach().contiguous().to(torch.complex64)
        if taps.numel() != ntaps * nch or gains.numel() != nch * ne:
            raise B.MdtError("FxCorrelate: taps must hold Ntaps*Nch and gains Nch*NE values")
        X = _fengine(iq, taps, ne, nch, ntaps, nsp)
        Y = torch.empty_like(X)
        B.apply_gains(ne, nch, nsp, X, gains, Y)
        del X
        V = torch.empty(nch, ne, ne, dtype=torch.complex64, device=iq.device)
        B.xengine_f32(ne, nch, nsp, Y, ne, nsp * ne, 1.0 / nsp, V)
        ctx.save_for_backward(iq, taps, gains)
        ctx.dims = (ne, nch, ntaps, nsp)
        return V

    @staticmethod
    def backward(ctx, gV):
        iq, taps, gains = ctx.saved_tensors
        ne, nch, ntaps, nsp = ctx.dims
        need_taps, need_gains = ctx.needs_input_grad[1], ctx.needs_input_grad[2]
        if not (need_taps or need_gains):
            return (None,) * 7
        G = gV.detach().to(torch.complex64).contiguous()
        X = _fengine(iq, taps, ne, nch, ntaps, nsp)  # recomputed, not stored
        Y = torch.empty_like(X)
        B.apply_gains(ne, nch, nsp, X, gains, Y)
        dY = torch.empty_like(X)
        B.xengine_adjoint_f32(ne, nch, nsp, G, Y, dY, 1.0 / nsp)
        dgains = torch.empty(nch, ne, dtype=torch.complex64, device=iq.device) \
            if need_gains else None
        dF = Y if need_taps else None  # Y is dead from here on: reuse it
        B.gain_adjoint(ne, nch, nsp, dY, X=X if need_gains else None, gains=gains,
                       dgains=dgains, dF=dF)
        dtaps = None
        if need_taps:
            del X
            dP = dY  # dY is consumed: the inverse FFT writes over it
            B.fft_c2c(dF, dP, nsp * ne, nch, B.CUFFT_INVERSE)
            dtaps = torch.empty(ntaps * nch, dtype=torch.float32, device=iq.device)
            ws = torch.empty(ntaps * nch * 64, dtype=torch.float64, device=iq.device)
            B.pfb_tap_grad(ne, nch, ntaps, nsp, dP, iq, dtaps, ws)
        return None, dtaps, dgains, None, None, None, None


def _sqnorm(z):
    # |z|^2 through real and imaginary parts: abs() has no gradient at 0
    return (z.real ** 2 + z.imag ** 2).sum()


def fx_correlate(iq, taps, gains, ne, nch, ntaps, nsp):
    """Differentiable FX correlation (see FxCorrelate)."""
    return FxCorrelate.apply(iq, taps, gains, ne, nch, ntaps, nsp)


def baseline_mask(ne, device):
    """True on the pairs a < b of the [q, r] visibility layout (r < q)."""
    idx = torch.arange(ne, device=device)
    return idx[None, :] < idx[:, None]


def gain_error(est, true):
    """Relative error of estimated gains after removing each channel's global
    phase (which the baseline loss cannot see):  ||est e^{i phi} - true|| /
    ||true||, phi per channel from the best alignment; float."""
    # plain real arithmetic (float64), so no complex128 reduction kernels are needed
    e = torch.view_as_real(est.to(torch.complex64).contiguous()).double()
    t = torch.view_as_real(true.to(torch.complex64).contiguous()).double()
    er, ei, tr, ti = e[..., 0], e[..., 1], t[..., 0], t[..., 1]
    pr = (er * tr + ei * ti).sum(dim=1, keepdim=True)   # sum conj(est) * true
    pi = (er * ti - ei * tr).sum(dim=1, keepdim=True)
    mag = torch.sqrt(pr * pr + pi * pi).clamp_min(1e-300)
    cr, ci = pr / mag, pi / mag
    dr = er * cr - ei * ci - tr
    di = er * ci + ei * cr - ti
    return float(torch.sqrt((dr * dr + di * di).sum() / (tr * tr + ti * ti).sum()))


def solve_gains(iq, taps, data, model, ne, nch, ntaps, nsp, iters=200, tol=1e-9, step=0.5,
                true_gains=None, callback=None, g0=None, gtol=1e-7):
    """Per-antenna, per-channel complex gains by gradient descent.

    Loss  L(g) = sum_c sum_{a<b} |data_ab - V(g)_ab|^2,  V(g) = the FX
    correlation of the model's samples `iq` under gains g (FxCorrelate).  With
    `iq` the noise-free streams of the sky model's sources (known flux and
    delays) and model = V(1) their correlation, V(g)_ab = g_a conj(g_b) model_ab,
    so this is the loss |data - g_a g_b^* model|^2 of a calibration against
    the source model, with `data` the measured (gained, noisy) visibilities.
    Gradients come from the adjoint kernels; each step is preconditioned per
    (channel, antenna) by the diagonal of the Gauss-Newton normal equations,
        h_ca = sum_{b != a} |g_cb|^2 |model_c,ab|^2,
    computed with the iterate in FP64 on the GPU:  g <- g - step * grad / (2h).
    Starts from `g0` (default unit gains); stops when the relative loss drops
    below `tol` (data the model explains exactly), when a step changes the
    gains by less than `gtol` relative (the minimiser of a noisy loss), or
    after `iters` steps.  Returns (gains complex64 [Nch, NE], history
    list of (relative loss, error against true_gains or None))."""
    dev = iq.device
    mask = baseline_mask(ne, dev)
    mr = torch.view_as_real(model.detach().to(torch.complex64).contiguous()).double()
    m2 = mr[..., 0] ** 2 + mr[..., 1] ** 2  # |model|^2, [c, q, r]
    m2 = m2 * (1 - torch.eye(ne, dtype=torch.float64, device=dev))
    g = (torch.ones(nch, ne, dtype=torch.complex128, device=dev) if g0 is None
         else g0.detach().to(torch.complex128).clone())
    data = data.detach()
    dnorm = float(_sqnorm(data[:, mask]))
    hist = []
    for _ in range(iters):
        gv = g.to(torch.complex64).requires_grad_(True)
        V = fx_correlate(iq, taps, gv, ne, nch, ntaps, nsp)
        loss = _sqnorm((V - data)[:, mask])
        loss.backward()
        err = gain_error(g, true_gains) if true_gains is not None else None
        hist.append((float(loss.detach()) / dnorm, err))
        if callback is not None:
            callback(len(hist), hist[-1])
        if hist[-1][0] < tol:
            break
        gg = g.real ** 2 + g.imag ** 2
        h = (m2 * gg[:, None, :]).sum(dim=2)  # model is Hermitian: |M_ab| = |M_ba|
        dg = step * gv.grad.to(torch.complex128) / (2 * h)
        g = g - dg
        if float(_sqnorm(dg)) <= gtol ** 2 * float(_sqnorm(g)):
            break
    return g.to(torch.complex64), hist


def c5_calibration_inputs(mdt, cfg, taps, model_scale=4, seed_salt=9):
    """The inputs of a configuration-5 gain calibration on the current device.

    data : visibilities of the configured sky (the sources plus unit receiver
           noise at the configured SNR, int8 I/Q from the integer generator)
           through the F-engine with true gains applied to its output,
           Y = diag(g) X  (FxCorrelate), multiplied by model_scale^2;
    iq_model : the same sources alone (known flux, delays from the element
           positions; no receiver noise), generated at model_scale times
           their amplitude so that int8 rounding stays ~2e-4 of their power,
           and the model's visibilities model = V(1) of those streams;
    g_true : gains with amplitude U[0.8, 1.2] and phase U[-pi, pi] per
           (channel, element), seeded.
    data and model share the source streams (the generator is keyed by
    source and time), never the noise.  Returns (data, iq_model, model,
    g_true)."""
    dev = taps.device
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    total = nsp + ntaps - 1
    ssig, sdel = cfg.sources()

    def t(a):
        return torch.from_numpy(a).to(dev)

    iq = torch.empty(total * ne * nch * 2, dtype=torch.int8, device=dev)
    B.synth_iq(cfg.seed, ne, nch, 0, total, t(cfg.sigma_q8()), iq,
               src_sigma_q8=t(ssig), src_delay=t(sdel))
    iq_model = torch.empty_like(iq)
    B.synth_iq(cfg.seed, ne, nch, 0, total, t(0 * cfg.sigma_q8()), iq_model,
               src_sigma_q8=t(ssig * model_scale), src_delay=t(sdel))
    import numpy as np
    rng = np.random.default_rng([cfg.seed, seed_salt])
    g_true = t((rng.uniform(0.8, 1.2, (nch, ne)) *
                np.exp(1j * rng.uniform(-np.pi, np.pi, (nch, ne)))).astype(np.complex64))
    ones = torch.ones(nch, ne, dtype=torch.complex64, device=dev)
    with torch.no_grad():
        data = fx_correlate(iq, taps, g_true, ne, nch, ntaps, nsp) * float(model_scale ** 2)
        model = fx_correlate(iq_model, taps, ones, ne, nch, ntaps, nsp)
    del iq
    return data, iq_model, model, g_true
