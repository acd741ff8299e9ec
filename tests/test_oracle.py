"""Pins the oracle (oracle/mdt_oracle.c) before anything is checked against it:
against the reference kernels' own outputs (tests/golden/ref_kernels.npz,
made by tests/golden/make_golden.py from the reference source), and against
independent numpy restatements of the cuFFT / cuBLAS contracts."""
import numpy as np
import pytest

from conftest import rel_fro


def test_pps_matches_reference_kernel_bit_exact(oracle, golden):
    for k in range(4):
        nch, ntaps, ne, nsp, _ = golden["pps%d_shape" % k]
        out = oracle.pps_f32_exact(golden["pps%d_win" % k], golden["pps%d_in" % k],
                                   nch, ntaps, ne, nsp)
        ref = golden["pps%d_out" % k]
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), k


def test_reorder_matches_reference_kernel_bit_exact(oracle, golden):
    for k in range(4):
        ne, nch, nsp = golden["reorder%d_shape" % k]
        out = oracle.reorder_c64(golden["reorder%d_in" % k], ne, nch, nsp)
        assert np.array_equal(out.view(np.uint32), golden["reorder%d_out" % k].view(np.uint32))


def test_window_bh4_matches_reference_kernel(oracle, golden):
    # the reference evaluates in float with CUDA sinpif/cospif (here: the
    # double-evaluated stand-ins); the oracle evaluates in double
    for k in range(3):
        nch, ntaps = golden["window%d_shape" % k]
        w = oracle.window_bh4(nch, ntaps)
        np.testing.assert_allclose(w, golden["window%d_out" % k], rtol=0, atol=5e-7)


def test_window_hamming_sinc_definition(oracle):
    nch, ntaps = 64, 4
    L = nch * ntaps
    n = np.arange(L)
    t = (n - L / 2) / nch
    ref = np.sinc(t) * (0.54 - 0.46 * np.cos(2 * np.pi * n / L))
    np.testing.assert_array_equal(oracle.window_hamming_sinc(nch, ntaps), ref.astype(np.float32))


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 16384])
def test_fft_matches_numpy(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    y = oracle.fft_rows(x, n).reshape(3, n)
    ref = np.fft.fft(x, axis=1)
    assert np.max(np.abs(y - ref)) / np.max(np.abs(ref)) < 1e-13


def test_fft_matches_naive_dft(oracle):
    n = 32
    rng = np.random.default_rng(7)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    k = np.arange(n)
    dft = np.exp(-2j * np.pi * np.outer(k, k) / n) @ x  # cuFFT forward sign
    np.testing.assert_allclose(oracle.fft_rows(x, n), dft, rtol=0, atol=1e-12)


def test_fft_rejects_non_power_of_two(oracle):
    with pytest.raises(ValueError):
        oracle.fft_rows(np.zeros(24, complex), 24)


def numpy_fx(iq, win, ne, nch, ntaps, nsp):
    """Independent numpy restatement: PFB (tap i on spectrum s+i) -> FFT ->
    V[c, q, r] = 1/nsp sum_s X[s, r, c] conj(X[s, q, c])."""
    x = iq.astype(np.float64).reshape(nsp + ntaps - 1, ne, nch, 2)
    x = x[..., 0] + 1j * x[..., 1]
    w = win.astype(np.float64).reshape(ntaps, nch)
    p = sum(w[i][None, None, :] * x[i:i + nsp] for i in range(ntaps))
    f = np.fft.fft(p, axis=2)  # [s, e, c]
    return np.einsum("sec,sqc->cqe", f, np.conj(f)) / nsp


def test_fx_matches_numpy_restatement(oracle):
    ne, nch, ntaps, nsp = 5, 64, 4, 12
    rng = np.random.default_rng(11)
    iq = rng.integers(-127, 128, size=(nsp + ntaps - 1) * ne * nch * 2).astype(np.int8)
    win = oracle.window_hamming_sinc(nch, ntaps)
    V = oracle.fx(iq, win, ne, nch, ntaps, nsp)
    ref = numpy_fx(iq, win, ne, nch, ntaps, nsp)
    assert rel_fro(V, ref) < 1e-13
    # Hermitian, real autocorrelations
    np.testing.assert_allclose(V, np.conj(np.transpose(V, (0, 2, 1))), atol=1e-9)
    # channel subset agrees with the full computation
    sel = [0, 7, 63, 31]
    Vs = oracle.fx(iq, win, ne, nch, ntaps, nsp, channels=sel)
    np.testing.assert_allclose(Vs, V[sel], rtol=1e-13, atol=1e-10)


def test_fx_f32_cpu_pipeline_close_to_f64(oracle):
    ne, nch, ntaps, nsp = 4, 128, 8, 40
    rng = np.random.default_rng(12)
    iq = rng.integers(-127, 128, size=(nsp + ntaps - 1) * ne * nch * 2).astype(np.int8)
    win = oracle.window_hamming_sinc(nch, ntaps)
    V64 = oracle.fx(iq, win, ne, nch, ntaps, nsp)
    V32 = oracle.fx(iq, win, ne, nch, ntaps, nsp, double=False)
    assert rel_fro(V32, V64) < 1e-5


def test_xengine_matches_einsum(oracle):
    ne, nch, nsp = 6, 5, 9
    rng = np.random.default_rng(3)
    X = rng.standard_normal((nch, nsp, ne)) + 1j * rng.standard_normal((nch, nsp, ne))
    V = oracle.xengine(X, ne, nch, nsp, 1.0 / nsp)
    ref = np.einsum("csr,csq->cqr", X, np.conj(X)) / nsp
    np.testing.assert_allclose(V, ref, rtol=1e-13, atol=1e-13)


def test_xengine_i8_exact(oracle):
    ne, nch, nsp = 7, 3, 50
    rng = np.random.default_rng(4)
    X = rng.integers(-127, 128, size=(nch, nsp, ne, 2)).astype(np.int8)
    V = oracle.xengine_i8(X, ne, nch, nsp)
    x = X[..., 0].astype(np.int64) + 1j * X[..., 1].astype(np.int64)
    ref = np.einsum("csr,csq->cqr", x, np.conj(x))
    assert np.array_equal(V[..., 0], ref.real.astype(np.int64))
    assert np.array_equal(V[..., 1], ref.imag.astype(np.int64))
