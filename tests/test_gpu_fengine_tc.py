"""Tensor-core F-engine (mdt_fengine_tc, Nch = 1024): its X16 output against
the FP64 F-output of the oracle (PFB -> FFT, reference PpS_Batch ->
cufftExecC2C) and against the SIMT f16 F-engine on the same inputs, for
ragged NE, Nsp not a multiple of 8 or 32, runs longer than one work item,
Ntaps 4 and 8, f16 and bf16 output.  The DFT runs on f16 operands with FP32
accumulation, so the tolerance is stated per case (relative Frobenius error
of the scaled F-output)."""
import numpy as np
import pytest
import torch

from x16util import unswizzle_x16

pytestmark = pytest.mark.gpu

TOL_F16 = 1.5e-3   # F-output, f16 DFT operands + f16 output rounding
TOL_BF16 = 8e-3    # bf16 output rounding dominates


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def fp64_fout(oracle, iq, win, ne, nch, ntaps, nsp):
    x = iq.astype(np.float64).reshape(nsp + ntaps - 1, ne, nch, 2)
    x = x[..., 0] + 1j * x[..., 1]
    w = win.astype(np.float64).reshape(ntaps, nch)
    P = sum(w[i][None, None, :] * x[i:i + nsp] for i in range(ntaps))
    return oracle.fft_rows(P.reshape(-1, nch), nch).reshape(nsp, ne, nch)


@pytest.mark.parametrize("ne,ntaps,nsp,bf16", [(5, 8, 100, False), (3, 4, 33, False),
                                               (18, 8, 600, False), (7, 4, 264, True)])
def test_fengine_tc_vs_fp64_and_simt(mdt, cuda, oracle, ne, ntaps, nsp, bf16):
    nch = 1024
    iq = oracle.synth_iq(ne * 31 + nsp, ne, nch, 0, nsp + ntaps - 1,
                         np.full(ne, 16 * 256, np.int32))
    win = oracle.window_hamming_sinc(nch, ntaps)
    scale = 0.125
    nep = (ne + 15) // 16 * 16
    nb = mdt.x16_bytes(ne, nch, nsp)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    X_tc = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    X_simt = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    mdt.fengine_tc(ne, nch, ntaps, nsp, dev(iq), dev(win), X_tc, err, ab_fmt=int(bf16),
                   scale=scale)
    mdt.fengine_x16(ne, nch, ntaps, nsp, dev(iq), dev(win), X_simt, ab_fmt=int(bf16), scale=scale)
    torch.cuda.synchronize()
    assert err.item() == 0
    got = unswizzle_x16(X_tc.cpu().numpy(), nch, nsp, ne, nep, bf16)     # [c][s][e][2]
    simt = unswizzle_x16(X_simt.cpu().numpy(), nch, nsp, ne, nep, bf16)
    F = fp64_fout(oracle, iq, win, ne, nch, ntaps, nsp) * scale          # [s][e][c]
    want = np.stack([F.real, F.imag], -1).transpose(2, 0, 1, 3)
    e_tc, e_simt = rel(got, want), rel(simt, want)
    print("F-output rel err: tensor-core %.2e, SIMT %.2e" % (e_tc, e_simt))
    assert e_tc < (TOL_BF16 if bf16 else TOL_F16)
    # padding: chunk positions past Nsp in the last 32-spectrum chunk stay zero
    nkc = (nsp + 31) // 32
    raw = X_tc.cpu().numpy().reshape(nkc, nch, nep, 128)
    assert not raw[:, :, ne:, :].any()   # rows NE..NEp-1 untouched (zeroed by the caller)


def test_plan_fp16_uses_tensor_core_fengine(mdt, cuda, oracle):
    """The plan's FP16 path at Nch = 1024 (tensor-core F-engine + X-engine),
    streamed with history, against the FP64 oracle."""
    cfg = mdt.configs.small(mdt.configs.C3, nelements=24, nchannels=1024, nspectra=512)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    ssig, sdel = cfg.sources()
    nint = 2
    iq = oracle.synth_iq(cfg.seed, ne, nch, 0, nint * nsp + ntaps - 1, cfg.sigma_q8(), None, ssig,
                         sdel)
    win = oracle.window_hamming_sinc(nch, ntaps)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=mdt.MDT_PREC_FP16)
    plan.set_window(dev(win))
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(dev(iq), nint, vis)
    plan.check()
    sb = ne * nch * 2
    for j in range(nint):
        seg = iq[j * nsp * sb:(j * nsp + nsp + ntaps - 1) * sb]
        sel = [0, 1, 511, 512, 1023]
        ref = oracle.fx(seg, win, ne, nch, ntaps, nsp, channels=sel)
        got = vis[j].cpu().numpy()[sel]
        e = max(rel(got[k], ref[k]) for k in range(len(sel)))
        print("integration %d: max channel rel err %.2e" % (j, e))
        assert e < 1e-3
    plan.close()


def test_fengine_tc_q8_within_one_lsb(mdt, cuda, oracle):
    """int8 requantisation on the tensor-core F-engine: within 1 LSB of the
    FP64 F-output quantised with the same scales (the f16 DFT moves values
    that sit within ~0.01 LSB of a rounding boundary)."""
    ne, nch, ntaps, nsp = 6, 1024, 8, 96
    iq = oracle.synth_iq(77, ne, nch, 0, nsp + ntaps - 1, np.full(ne, 16 * 256, np.int32))
    win = oracle.window_hamming_sinc(nch, ntaps)
    F = fp64_fout(oracle, iq, win, ne, nch, ntaps, nsp)           # [s][e][c]
    rms = np.sqrt(np.mean(np.abs(F) ** 2, axis=(0, 1)))
    qs = (20.0 / rms).astype(np.float32)
    want_re = np.clip(np.rint(F.real * qs.astype(np.float64)), -127, 127)
    want_im = np.clip(np.rint(F.imag * qs.astype(np.float64)), -127, 127)
    nep = (ne + 15) // 16 * 16
    X16 = torch.zeros(mdt.x16_bytes(ne, nch, nsp), dtype=torch.uint8, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    mdt.fengine_tc_q8(ne, nch, ntaps, nsp, dev(iq), dev(win), X16, dev(qs), err)
    torch.cuda.synchronize()
    assert err.item() == 0
    got = unswizzle_x16(X16.cpu().numpy(), nch, nsp, ne, nep)
    gre = np.transpose(got[..., 0], (1, 2, 0))
    gim = np.transpose(got[..., 1], (1, 2, 0))
    assert np.all(gre == np.rint(gre)) and np.all(np.abs(gre) <= 127)
    d = np.maximum(np.abs(gre - want_re), np.abs(gim - want_im))
    print("int8 F-output: %.4f of values exact" % np.mean(d == 0))
    assert d.max() <= 1
    assert np.mean(d == 0) > 0.97


def test_plan_int8_at_1024_channels(mdt, cuda, oracle):
    """The plan's INT8 path at Nch = 1024 runs the tensor-core F-engine with
    requantisation: identical to the stages called directly with its scales,
    and within the int8 quantisation error of FP64."""
    cfg = mdt.configs.small(mdt.configs.C3, nelements=20, nchannels=1024, nspectra=256)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    ssig, sdel = cfg.sources()
    iq_h = oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(), None, ssig, sdel)
    iq = dev(iq_h)
    win = dev(oracle.window_hamming_sinc(nch, ntaps))
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=mdt.MDT_PREC_INT8)
    plan.set_window(win)
    vis = torch.empty(nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(iq, 1, vis)
    plan.check()
    qs = torch.empty(nch, dtype=torch.float32, device="cuda")
    plan.get_channel_scales(qs)
    X16 = torch.zeros(mdt.x16_bytes(ne, nch, nsp), dtype=torch.uint8, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    mdt.fengine_tc_q8(ne, nch, ntaps, nsp, iq, win, X16, qs, err)
    v2 = torch.empty_like(vis)
    mdt.xengine_q8(ne, nch, nsp, X16, qs, vis=v2, err=err)
    torch.cuda.synchronize()
    assert err.item() == 0
    assert torch.equal(v2.view(torch.int64), vis.view(torch.int64))
    sel = [0, 7, 511, 1023]
    ref = oracle.fx(iq_h, win.cpu().numpy(), ne, nch, ntaps, nsp, channels=sel)
    e = max(rel(vis.cpu().numpy()[k], ref[i]) for i, k in enumerate(sel))
    print("int8 plan at 1024 channels: max channel rel err %.3e" % e)
    assert e < 2e-2
    plan.close()
