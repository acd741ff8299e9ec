"""Exact int8 path: the F-engine requantises each channel to integers in
[-127, 127] (per-channel scales), the tensor-core X-engine sums them exactly
(f16 MMAs over 512-spectrum FP32-exact windows folded into int32).
* int32 visibilities bit-exact against the integer oracle on the same int8
  F-output, including saturated +-127 data across several windows;
* the int8 F-output within +-1 LSB of the FP64 oracle's quantisation;
* the plan's INT8 path, its calibration, and its error against FP64 (stated)."""
import numpy as np
import pytest
import torch

from conftest import rel_fro
from x16util import swizzle_x16, unswizzle_x16

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("ne,nch,nsp", [(40, 3, 1100), (130, 2, 600), (3, 4, 33)])
def test_xengine_q8_exact_on_saturated_data(mdt, cuda, oracle, ne, nch, nsp):
    rng = np.random.default_rng(ne * 7 + nsp)
    X = rng.integers(-127, 128, size=(nch, nsp, ne, 2))
    sat = rng.random(X.shape) < 0.5
    X[sat] = np.where(rng.random(X.shape)[sat] < 0.5, -127, 127)
    nep = (ne + 15) // 16 * 16
    X16 = dev(swizzle_x16(X, nep))
    qs = torch.ones(nch, dtype=torch.float32, device="cuda")
    raw = torch.full((nch, ne, ne, 2), -1, dtype=torch.int32, device="cuda")
    vis = torch.empty(nch, ne, ne, dtype=torch.complex64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    mdt.xengine_q8(ne, nch, nsp, X16, qs, vis=vis, vis_i32=raw, err=err)
    torch.cuda.synchronize()
    assert err.item() == 0
    ref = oracle.xengine_i8(X.astype(np.int8).reshape(nch, nsp, ne, 2), ne, nch, nsp)
    got = raw.cpu().numpy().astype(np.int64)
    assert np.array_equal(got, ref)
    v = vis.cpu().numpy()
    np.testing.assert_allclose(v.real, ref[..., 0] / nsp, rtol=1e-6, atol=1e-6)


def test_fengine_q8_within_one_lsb_of_fp64(mdt, cuda, oracle):
    cfg = mdt.configs.small(mdt.configs.C3, nelements=8, nchannels=256, nspectra=64)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    ssig, sdel = cfg.sources()
    iq = oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(), None, ssig, sdel)
    win = oracle.window_hamming_sinc(nch, ntaps)
    # FP64 F-output: PFB (tap i on spectrum s+i) then FFT
    x = iq.astype(np.float64).reshape(nsp + ntaps - 1, ne, nch, 2)
    x = x[..., 0] + 1j * x[..., 1]
    w = win.astype(np.float64).reshape(ntaps, nch)
    P = sum(w[i][None, None, :] * x[i:i + nsp] for i in range(ntaps))
    F = oracle.fft_rows(P.reshape(-1, nch), nch).reshape(nsp, ne, nch)
    rms = np.sqrt(np.mean(np.abs(F) ** 2, axis=(0, 1)))
    qs = (20.0 / rms).astype(np.float32)
    want_re = np.clip(np.rint(F.real * qs.astype(np.float64)), -127, 127)
    want_im = np.clip(np.rint(F.imag * qs.astype(np.float64)), -127, 127)
    nep = (ne + 15) // 16 * 16
    X16 = torch.zeros(mdt.x16_bytes(ne, nch, nsp), dtype=torch.uint8, device="cuda")
    wd = dev(win)
    mdt.fengine_q8(ne, nch, ntaps, nsp, dev(iq), wd, X16, dev(qs))
    torch.cuda.synchronize()
    got = unswizzle_x16(X16.cpu().numpy(), nch, nsp, ne, nep)  # [c][s][e][2]
    gre = np.transpose(got[..., 0], (1, 2, 0))
    gim = np.transpose(got[..., 1], (1, 2, 0))
    assert np.all(gre == np.rint(gre)) and np.all(np.abs(gre) <= 127)
    d = np.maximum(np.abs(gre - want_re), np.abs(gim - want_im))
    assert d.max() <= 1
    assert np.mean(d == 0) > 0.99


def test_plan_int8_vs_fp64_and_stage_consistency(mdt, cuda, oracle):
    cfg = mdt.configs.small(mdt.configs.C3, nelements=64, nchannels=256, nspectra=1024)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    ssig, sdel = cfg.sources()
    iq_h = oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(), None, ssig,
                           sdel)
    iq = dev(iq_h)
    win = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, win)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=mdt.MDT_PREC_INT8)
    plan.set_window(win)
    vis = torch.full((nch, ne, ne), float("nan"), dtype=torch.complex64, device="cuda")
    plan.execute(iq, 1, vis)
    plan.check()
    qs = torch.empty(nch, dtype=torch.float32, device="cuda")
    plan.get_channel_scales(qs)
    # the same stages called directly with the plan's scales give the same bits
    X16 = torch.zeros(mdt.x16_bytes(ne, nch, nsp), dtype=torch.uint8, device="cuda")
    mdt.fengine_q8(ne, nch, ntaps, nsp, iq, win, X16, qs)
    v2 = torch.empty_like(vis)
    raw = torch.empty(nch, ne, ne, 2, dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    mdt.xengine_q8(ne, nch, nsp, X16, qs, vis=v2, vis_i32=raw, err=err)
    torch.cuda.synchronize()
    assert torch.equal(v2.view(torch.int64), vis.view(torch.int64))
    # calibrated scales put the F-output near 20 LSB rms
    got = unswizzle_x16(X16.cpu().numpy(), nch, nsp, ne, (ne + 15) // 16 * 16)
    rms = np.sqrt(np.mean(got[..., 0] ** 2 + got[..., 1] ** 2))
    assert 15 < rms < 25
    sel = [0, 5, 100, 128, 255]
    ref = oracle.fx(iq_h, win.cpu().numpy(), ne, nch, ntaps, nsp, channels=sel)
    e = rel_fro(vis.cpu().numpy()[sel], ref)
    print("int8 path rel err vs FP64 %.3e" % e)
    assert e < 2e-2  # int8 quantisation of the F-output (1 LSB at 20 LSB rms)
    plan.close()
