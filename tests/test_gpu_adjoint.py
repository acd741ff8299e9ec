"""Adjoint kernels and the torch.autograd.Function over them.

* each adjoint kernel against an FP64 restatement on the same inputs
  (ragged sizes: NE not a multiple of 16, Nsp not a multiple of 16);
* the full gradient (taps and gains) against an FP64 reference gradient
  (PyTorch float64 autograd of the same forward) and against FP64 central
  finite differences of the FP64 oracle's FX pipeline;
* determinism of the reductions;
* gain calibration on the c5_gaincal64 configuration (NE=64, Nch=512,
  Ntaps=4, Nsp=2048, 3-source sky) to <= 1e-4 relative gain error.
FP32 gradients are compared with tolerances written at each assertion."""
import importlib

import numpy as np
import pytest
import torch

from adjref import crandn, fd_gains, fd_taps, make_case, reference_gradient
from conftest import PKG_NAME

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adj(mdt):
    return importlib.import_module(PKG_NAME + ".adjoint")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("ne,nch,nsp", [(130, 3, 37), (8, 5, 200), (1, 2, 16)])
def test_xengine_adjoint_kernel(mdt, cuda, ne, nch, nsp):
    rng = np.random.default_rng(ne + nsp)
    G = crandn(rng, nch, ne, ne)          # G[c][q][r] = grad(V_rq)
    Y = crandn(rng, nch, nsp, ne)
    dY = torch.empty(nch * nsp * ne, dtype=torch.complex64, device="cuda")
    mdt.xengine_adjoint_f32(ne, nch, nsp, dev(G.astype(np.complex64)),
                            dev(Y.astype(np.complex64)), dY, 0.25)
    torch.cuda.synchronize()
    Gm = np.transpose(G, (0, 2, 1))       # Gm[c][r][q] = G_rq
    H = Gm + np.conj(np.transpose(Gm, (0, 2, 1)))
    want = 0.25 * np.einsum("crq,csq->csr", H, Y)
    got = dY.cpu().numpy().reshape(nch, nsp, ne)
    assert rel(got, want) < 2e-6  # FP32 dot products of length NE


@pytest.mark.parametrize("ne,nch,nsp", [(40, 64, 33), (3, 96, 8)])
def test_gain_adjoint_kernel(mdt, cuda, ne, nch, nsp):
    rng = np.random.default_rng(nch + nsp)
    dY = crandn(rng, nch, nsp, ne).astype(np.complex64)
    X = crandn(rng, nch, nsp, ne).astype(np.complex64)
    g = crandn(rng, nch, ne).astype(np.complex64)
    dg = torch.empty(nch, ne, dtype=torch.complex64, device="cuda")
    dF = torch.empty(nsp, ne, nch, dtype=torch.complex64, device="cuda")
    mdt.gain_adjoint(ne, nch, nsp, dev(dY), X=dev(X), gains=dev(g), dgains=dg, dF=dF)
    torch.cuda.synchronize()
    want_dg = np.einsum("cse,cse->ce", dY.astype(np.complex128), np.conj(X))
    assert rel(dg.cpu().numpy(), want_dg) < 1e-6  # double sums, FP32 result
    c128 = np.complex128
    want_dF = np.transpose(np.conj(g.astype(c128))[:, None, :] * dY, (1, 2, 0))
    assert rel(dF.cpu().numpy(), want_dF) < 1e-7  # one complex product in FP32
    # apply_gains is the forward of the same map
    Y = torch.empty(nch * nsp * ne, dtype=torch.complex64, device="cuda")
    mdt.apply_gains(ne, nch, nsp, dev(X), dev(g), Y)
    torch.cuda.synchronize()
    assert rel(Y.cpu().numpy().reshape(nch, nsp, ne), g.astype(c128)[:, None, :] * X) < 1e-7


def test_pfb_tap_grad_kernel_and_determinism(mdt, cuda):
    ne, nch, ntaps, nsp = 5, 256, 4, 50
    rng = np.random.default_rng(7)
    iq = rng.integers(-128, 128, size=(nsp + ntaps - 1, ne, nch, 2)).astype(np.int8)
    gP = crandn(rng, nsp, ne, nch).astype(np.complex64)
    x = iq[..., 0].astype(np.float64) + 1j * iq[..., 1]
    want = np.stack([np.real(np.sum(gP * np.conj(x[i:i + nsp]), axis=(0, 1)))
                     for i in range(ntaps)]).ravel()
    outs = []
    for nsplit in (1, 64, 64):
        gW = torch.empty(ntaps * nch, dtype=torch.float32, device="cuda")
        ws = torch.empty(ntaps * nch * nsplit, dtype=torch.float64, device="cuda")
        mdt.pfb_tap_grad(ne, nch, ntaps, nsp, dev(gP), dev(iq.reshape(-1)), gW, ws)
        torch.cuda.synchronize()
        outs.append(gW.cpu().numpy())
        assert rel(outs[-1], want) < 2e-7  # double sums, one FP32 rounding
    assert np.array_equal(outs[1], outs[2])
    with pytest.raises(mdt.MdtError):
        small = torch.empty(ntaps * nch - 1, dtype=torch.float64, device="cuda")
        mdt.pfb_tap_grad(ne, nch, ntaps, nsp, dev(gP), dev(iq.reshape(-1)), gW, small)


def _ours(adj, iq, W, g, C, ne, nch, ntaps, nsp):
    taps = dev(W).requires_grad_(True)
    gains = dev(g).requires_grad_(True)
    V = adj.fx_correlate(dev(iq.reshape(-1)), taps, gains, ne, nch, ntaps, nsp)
    V.backward(dev(C.astype(np.complex64)))
    torch.cuda.synchronize()
    return V.detach().cpu().numpy(), taps.grad.cpu().numpy(), gains.grad.cpu().numpy()


def test_gradient_vs_fp64_reference_gradient(adj, oracle, cuda):
    ne, nch, ntaps, nsp = 6, 64, 4, 40
    iq, W, g, C = make_case(oracle, ne, nch, ntaps, nsp)
    V, gW, gg = _ours(adj, iq, W, g, C, ne, nch, ntaps, nsp)
    V64, gW64, gg64 = reference_gradient(iq, W, g, C, ne, nch, ntaps, nsp)
    assert rel(V, V64) < 1e-5      # FP32 forward
    assert rel(gW, gW64) < 1e-5    # FP32 adjoint chain (X-adjoint, inverse FFT, tap sums)
    assert rel(gg, gg64) < 1e-5


@pytest.mark.parametrize("shape", [(6, 64, 4, 40), (17, 128, 8, 21)])
def test_gradient_vs_fp64_finite_differences(adj, oracle, cuda, shape):
    ne, nch, ntaps, nsp = shape
    iq, W, g, C = make_case(oracle, ne, nch, ntaps, nsp, seed=ne)
    _, gW, gg = _ours(adj, iq, W, g, C, ne, nch, ntaps, nsp)
    rng = np.random.default_rng(3)
    idx = rng.choice(ntaps * nch, 8, replace=False)
    fd = fd_taps(oracle, iq, W, g, C, ne, nch, ntaps, nsp, idx)
    assert np.abs(fd - gW[idx]).max() <= 1e-5 * np.abs(gW).max()  # FP32 vs FP64
    gidx = [(0, 0), (nch // 2, ne // 2), (nch - 1, ne - 1)]
    fdg = fd_gains(oracle, iq, W, g, C, ne, nch, ntaps, nsp, gidx)
    got = np.array([gg[c, e] for c, e in gidx])
    assert np.abs(fdg - got).max() <= 1e-5 * np.abs(gg).max()


def test_backward_is_repeatable(adj, oracle, cuda):
    ne, nch, ntaps, nsp = 6, 64, 4, 40
    iq, W, g, C = make_case(oracle, ne, nch, ntaps, nsp)
    a = _ours(adj, iq, W, g, C, ne, nch, ntaps, nsp)
    b = _ours(adj, iq, W, g, C, ne, nch, ntaps, nsp)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_gain_calibration_c5_against_source_model(mdt, adj, cuda):
    """Configuration 5: the data are the visibilities of the noisy sky (three
    sources in unit receiver noise at SNR 0.1) with true gains applied to the
    F-engine output; the model is the correlation of the noise-free source
    streams (known flux and delays), generated separately.  The solver must
    reach the loss minimiser (within 1e-4, relative gain error), and that
    minimiser must sit at the receiver-noise floor around the true gains."""
    cfg = mdt.configs.C5
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    win = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, win)
    data, iq_model, model, g_true = adj.c5_calibration_inputs(mdt, cfg, win)
    g, hist = adj.solve_gains(iq_model, win, data, model, ne, nch, ntaps, nsp, iters=400,
                              tol=1e-13, gtol=1e-7, true_gains=g_true)
    g_min, hist_min = adj.solve_gains(iq_model, win, data, model, ne, nch, ntaps, nsp,
                                      iters=400, tol=1e-13, gtol=1e-7, g0=g_true)
    err, to_min = adj.gain_error(g, g_true), adj.gain_error(g, g_min)
    floor = adj.gain_error(g_min, g_true)
    # expected floor: per-baseline noise sqrt(P_a P_b / Nsp) (P = per-antenna
    # power) against the model's cross-power, whose rms over baselines is
    # S / sqrt(nsrc) for nsrc equal sources at random phases (S = their total
    # power), combined over the NE-1 baselines of an antenna
    P, S = 1.0 + cfg.snr, cfg.snr
    predicted = P / np.sqrt(nsp) / (S / np.sqrt(cfg.nsrc)) / np.sqrt(ne - 1)
    print("c5 calibration against the source model: %d steps (%d from the truth), "
          "gain error %.3e vs true, %.3e vs the loss minimiser; noise floor %.3e "
          "(predicted ~%.1e)" % (len(hist), len(hist_min), err, to_min, floor, predicted))
    assert hist[0][1] > 0.1  # the start (unit gains) is far off
    assert to_min <= 1e-4
    assert floor < 2.5 * predicted
    assert err <= floor + 1e-4
