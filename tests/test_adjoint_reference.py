"""The FP64 references of the adjoint tests agree with each other (CPU only):
the PyTorch float64 forward equals the FP64 oracle's FX pipeline, and its
autograd gradient equals FP64 central finite differences of the oracle."""
import numpy as np
import pytest

from adjref import fd_gains, fd_taps, fx64, make_case, reference_gradient

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("shape", [(6, 64, 4, 40), (3, 32, 8, 9)])
def test_fp64_reference_gradient_matches_oracle_fd(oracle, shape):
    ne, nch, ntaps, nsp = shape
    iq, W, g, C = make_case(oracle, ne, nch, ntaps, nsp, seed=ne + nch)
    V, gW, gg = reference_gradient(iq, W, g, C, ne, nch, ntaps, nsp)
    V0 = oracle.fx(iq, W, ne, nch, ntaps, nsp)
    g64 = g.astype(np.complex128)
    want = g64[:, None, :] * np.conj(g64)[:, :, None] * V0
    assert np.abs(V - want).max() <= 1e-11 * np.abs(want).max()
    idx = np.random.default_rng(1).choice(ntaps * nch, 10, replace=False)
    fd = fd_taps(oracle, iq, W, g, C, ne, nch, ntaps, nsp, idx)
    assert np.abs(fd - gW[idx]).max() <= 1e-8 * np.abs(gW).max()
    gidx = [(0, 0), (nch - 1, ne - 1), (nch // 3, 1)]
    fdg = fd_gains(oracle, iq, W, g, C, ne, nch, ntaps, nsp, gidx)
    got = np.array([gg[c, e] for c, e in gidx])
    assert np.abs(fdg - got).max() <= 1e-8 * np.abs(gg).max()


def test_fx64_matches_oracle_unit_gains(oracle):
    ne, nch, ntaps, nsp = 4, 16, 4, 12
    iq, W, _, _ = make_case(oracle, ne, nch, ntaps, nsp)
    V = fx64(iq, torch.from_numpy(W.astype(np.float64)),
             torch.ones(nch, ne, dtype=torch.complex128), ne, nch, ntaps, nsp).numpy()
    V0 = oracle.fx(iq, W, ne, nch, ntaps, nsp)
    assert np.abs(V - V0).max() <= 1e-11 * np.abs(V0).max()
