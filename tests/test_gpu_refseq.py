"""Second parity check: the reference's own GPU sequence on the same inputs.

The reference's kernels (PpS_Batch, ReorderFOutput, PFB_Window_min4term_BH),
compiled from the reference source for sm_103a (baseline/build_ref_gpu.sh),
run with NVIDIA's cuFFT and cuBLAS as the reference client calls them
(MDT_OneStation_client.cu:1083,1105,1114,1128; baseline/refseq.cu), stage by
stage, on the int8 I/Q converted to complex64.  Against them:
  * the drop-in PpS_Batch on the same complex64 input: bit-exact;
  * the drop-in ReorderFOutput on the reference's FFT output: bit-exact;
  * this library's FFT against cuFFT on the reference's PpS output, both
    against the FP64 FFT: <= 3e-7 * log2(Nch) relative per row;
  * the fused FP32 plan's visibilities against cuBLAS's: <= 1e-5 relative
    (max over channels, Frobenius), and both against the FP64 oracle;
  * the drop-in window kernel against the reference's: <= 5e-7 absolute.
Shapes: configuration 1 in full (NE=10, Nch=1024, Ntaps=4, Nsp=1000) and
configuration 2 with 256 of its 4096 spectra (NE=40, Nch=2048, Ntaps=8)."""
import numpy as np
import pytest
import torch

from conftest import ROOT, rel_fro  # noqa: F401  (ROOT puts the repo on sys.path)

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5


def cdiv(a, b):
    return (a + b - 1) // b


def _refseq():
    from baseline import refseq
    if not refseq.available():
        pytest.skip("reference kernels not compiled (baseline/build_ref_gpu.sh needs the "
                    "reference checkout)")
    # the harness must call NVIDIA's libraries, not libmdtfx.so's same-named shim
    fft_file, blas_file, fft_ver, blas_ver = refseq.libraries()
    print("cuFFT %d from %s; cuBLAS %d from %s" % (fft_ver, fft_file, blas_ver, blas_file))
    assert "libcufft" in fft_file and "libcublas" in blas_file
    assert "mdtfx" not in fft_file + blas_file
    return refseq


def _shapes(mdt):
    return [mdt.configs.C1, mdt.configs.small(mdt.configs.C2, nspectra=256, nint=1)]


@pytest.mark.parametrize("which", [0, 1])
def test_reference_sequence_stage_by_stage(mdt, cuda, oracle, which):
    from test_gpu_pipeline import gen_iq, to_c64, window
    refseq = _refseq()
    cfg = _shapes(mdt)[which]
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    iq = gen_iq(mdt, cfg, 0, nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    rs = refseq.RefSeq(ne, nch, ntaps, nsp)
    try:
        rs.set_input(iq, win)
        fin = to_c64(iq)
        # the harness's complex64 input is the exact conversion of the int8 samples
        got_in = rs.read(refseq.FINPUT, torch.empty_like(fin))
        assert torch.equal(got_in, fin)

        # PpS_Batch: reference kernel vs drop-in, bit for bit
        rs.stage(0)
        pps_ref = rs.read(refseq.FOUTPUT, torch.empty(nsp * ne * nch, dtype=torch.complex64,
                                                      device="cuda"))
        pps = torch.full_like(pps_ref, float("nan"))
        mdt.PpS_Batch((cdiv(nch, 1024), nsp, ne), (1024,), nch, ntaps, win, fin, pps)
        torch.cuda.synchronize()
        assert torch.equal(pps.view(torch.int64), pps_ref.view(torch.int64))

        # FFT: cuFFT vs this library's FFT, each against FP64
        rs.stage(1)
        fft_ref = rs.read(refseq.FOUTPUT, torch.empty_like(pps_ref))
        ours = torch.empty_like(pps_ref)
        mdt.fft_c2c(pps_ref, ours, nsp * ne, nch, -1)
        torch.cuda.synchronize()
        exact = oracle.fft_rows(pps_ref.cpu().numpy().astype(np.complex128), nch)
        exact = exact.reshape(-1, nch)
        tol = 3e-7 * np.log2(nch)
        for name, y in (("cuFFT", fft_ref), ("library FFT", ours)):
            y = y.cpu().numpy().reshape(-1, nch)
            err = np.linalg.norm(y - exact, axis=1) / np.linalg.norm(exact, axis=1)
            print("%s %s: max row rel err %.3e" % (cfg.name, name, err.max()))
            assert err.max() < tol, name

        # ReorderFOutput: reference kernel vs drop-in on the reference's FFT output
        rs.stage(2)
        xin_ref = rs.read(refseq.XINPUT, torch.empty_like(pps_ref))
        xin = torch.full_like(xin_ref, float("nan"))
        mdt.ReorderFOutput((cdiv(ne, 32), cdiv(nch, 32), nsp), (32, 32), ne, nch, fft_ref, xin)
        torch.cuda.synchronize()
        assert torch.equal(xin.view(torch.int64), xin_ref.view(torch.int64))

        # cublasCgemmBatched vs the fused FP32 plan, both vs the FP64 oracle
        rs.stage(3)
        vis_ref = rs.read(refseq.XOUTPUT, torch.empty(nch, ne, ne, dtype=torch.complex64,
                                                      device="cuda")).cpu().numpy()
        plan = mdt.FxPlan(ne, nch, ntaps, nsp)
        plan.set_window(win)
        vis = torch.empty(nch, ne, ne, dtype=torch.complex64, device="cuda")
        plan.execute(iq, 1, vis)
        torch.cuda.synchronize()
        plan.close()
        vis = vis.cpu().numpy()
        e_lib = rel_fro(vis, vis_ref.astype(np.complex128))
        sel = np.array(sorted({0, 1, 137 % nch, nch // 2, nch - 1} |
                              {c for c, _ in cfg.tone_channels()}), np.int32)
        o = oracle.fx(iq.cpu().numpy(), win.cpu().numpy(), ne, nch, ntaps, nsp, channels=sel)
        e_ref, e_ours = rel_fro(vis_ref[sel], o), rel_fro(vis[sel], o)
        print("%s: plan vs cuBLAS %.3e; vs FP64: cuBLAS %.3e, plan %.3e" %
              (cfg.name, e_lib, e_ref, e_ours))
        assert e_lib < TOL_FP32 and e_ref < TOL_FP32 and e_ours < TOL_FP32
    finally:
        rs.close()


def test_reference_window_kernel(mdt, cuda):
    refseq = _refseq()
    for nch, ntaps in ((1024, 4), (2048, 8), (32, 4)):
        rs = refseq.RefSeq(3, nch, ntaps, 2)
        try:
            ref = rs.window_bh(torch.empty(nch * ntaps, dtype=torch.float32, device="cuda"))
        finally:
            rs.close()
        ours = torch.empty_like(ref)
        n = nch * ntaps
        mdt.PFB_Window_min4term_BH((cdiv(n, 1024),), (1024,), nch, ntaps, ours)
        torch.cuda.synchronize()
        d = (ours - ref).abs().max().item()
        same = int((ours.view(torch.int32) == ref.view(torch.int32)).sum().item())
        print("window Nch=%d Ntaps=%d: max abs diff %.2e, %d of %d bit-equal" %
              (nch, ntaps, d, same, n))
        assert d <= 5e-7
