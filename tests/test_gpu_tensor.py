"""Tensor-core path (f16 / bf16 F-engine output, tcgen05 X-engine, FP32
accumulate) against the FP64 oracle: <= 1e-3 relative visibility error (max
over channels of the Frobenius norm), plus structure, streaming and FP64
cross-integration accumulation."""
import numpy as np
import pytest
import torch

from conftest import rel_fro

pytestmark = pytest.mark.gpu

TOL_TC = 1e-3   # f16 operands, FP32 accumulation
# bf16 keeps 8 significand bits (rounding error up to 2^-9 per F-output
# value); cross-correlations of noise do not average that error down, so on
# short integrations the Frobenius error sits near 1.5e-3.
TOL_BF16 = 4e-3


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gen(mdt, cfg, nsp_total):
    out = torch.empty(nsp_total * cfg.nelements * cfg.nchannels * 2, dtype=torch.int8,
                      device="cuda")
    tone = cfg.tone_q16()
    ssig, sdel = cfg.sources()
    mdt.synth_iq(cfg.seed, cfg.nelements, cfg.nchannels, 0, nsp_total, dev(cfg.sigma_q8()), out,
                 tone_q16=None if tone is None else dev(tone),
                 src_sigma_q8=None if ssig is None else dev(ssig),
                 src_delay=None if sdel is None else dev(sdel))
    return out


def window(mdt, nch, ntaps):
    w = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, w)
    return w


def run_plan(mdt, prec, ne, nch, ntaps, nsp, iq, win, nint=1):
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=prec)
    plan.set_window(win)
    vis = torch.full((nint, nch, ne, ne), float("nan"), dtype=torch.complex64, device="cuda")
    plan.execute(iq, nint, vis)
    plan.check()
    return plan, vis


CASES = [
    # (config, ne, nch, ntaps, nsp)
    ("c3_array256", 256, 1024, 8, 256),
    ("c5_gaincal64", 64, 512, 4, 200),
    ("c2_station40", 40, 2048, 8, 96),
    ("c1_snap10", 10, 1024, 4, 100),
    ("c3_array256", 130, 256, 8, 64),
    ("c1_snap10", 3, 32, 4, 2),
]


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("case", CASES)
def test_tensor_path_vs_oracle(mdt, cuda, oracle, prec, case):
    name, ne, nch, ntaps, nsp = case
    cfg = mdt.configs.small(mdt.configs.CONFIGS[name], nelements=ne, nchannels=nch, ntaps=ntaps,
                            nspectra=nsp)
    iq = gen(mdt, cfg, nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    plan, vis = run_plan(mdt, prec, ne, nch, ntaps, nsp, iq, win)
    v = vis[0].cpu().numpy()
    rng = np.random.default_rng(ne + nch)
    sel = sorted(set([0, nch - 1, nch // 2] + list(rng.integers(0, nch, 13))))
    ref = oracle.fx(iq.cpu().numpy(), win.cpu().numpy(), ne, nch, ntaps, nsp, channels=sel)
    err = rel_fro(v[sel], ref)
    print("%s prec=%d ne=%d nch=%d nsp=%d rel err %.3e scale %g" % (name, prec, ne, nch, nsp,
                                                                   err, plan.scale()))
    assert err < (TOL_TC if prec == 1 else TOL_BF16)
    assert np.all(np.isfinite(v))
    assert np.array_equal(v, np.conj(np.transpose(v, (0, 2, 1))))
    assert np.all(np.diagonal(v, axis1=1, axis2=2).imag == 0)
    plan.close()


def test_tensor_vs_fp32_full_c3_shape(mdt, cuda):
    """Full c3 channel count and array size (NE=256, Nch=1024, Ntaps=8), 512
    spectra: the f16 tensor path against the FP32 path on every channel."""
    cfg = mdt.configs.small(mdt.configs.C3, nspectra=512)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    iq = gen(mdt, cfg, nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    p16, v16 = run_plan(mdt, 1, ne, nch, ntaps, nsp, iq, win)
    p32, v32 = run_plan(mdt, 0, ne, nch, ntaps, nsp, iq, win)
    err = rel_fro(v16[0].cpu().numpy(), v32[0].cpu().numpy().astype(np.complex128))
    print("c3 shape f16 vs fp32 rel err %.3e" % err)
    assert err < TOL_TC
    p16.close()
    p32.close()


def test_tensor_streaming_and_fp64_accumulator(mdt, cuda):
    ne, nch, ntaps, nsp, nint = 64, 256, 8, 64, 3
    cfg = mdt.configs.small(mdt.configs.C5, nelements=ne, nchannels=nch, ntaps=ntaps,
                            nspectra=nsp, nint=nint)
    iq = gen(mdt, cfg, nint * nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=1)
    plan.set_window(win)
    acc = torch.zeros(nch, ne, ne, dtype=torch.complex128, device="cuda")
    plan.set_accumulator(acc)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(iq, nint, vis)
    plan.set_accumulator(None)
    vs = torch.empty_like(vis)
    sb = ne * nch * 2
    plan.stream_push(iq[:(nsp + ntaps - 1) * sb].clone(), vs[0])
    for j in range(1, nint):
        lo = (j * nsp + ntaps - 1) * sb
        plan.stream_push(iq[lo:lo + nsp * sb].clone(), vs[j])
    plan.check()
    assert torch.equal(vs.view(torch.int64), vis.view(torch.int64))
    want = vis.to(torch.complex128).sum(dim=0)
    assert torch.allclose(acc, want, rtol=1e-12, atol=1e-9)
    plan.close()


def test_tensor_plan_rejects_large_nch(mdt, cuda):
    with pytest.raises(mdt.MdtError) as e:
        mdt.FxPlan(16, 8192, 4, 64, precision=1)
    assert e.value.code == 2


def test_tensor_path_deterministic(mdt, cuda):
    """c3 shape: every sum of the tensor path has a fixed order, so two runs
    agree bit for bit; the last channels agree with the FP32 path."""
    cfg = mdt.configs.small(mdt.configs.C3, nspectra=512)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    iq = gen(mdt, cfg, nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    p1, v1 = run_plan(mdt, 1, ne, nch, ntaps, nsp, iq, win)
    p2, v2 = run_plan(mdt, 1, ne, nch, ntaps, nsp, iq, win)
    assert torch.equal(v1, v2)
    p32, v32 = run_plan(mdt, 0, ne, nch, ntaps, nsp, iq, win)
    tail = slice(nch - 64, nch)
    err = rel_fro(v1[0, tail].cpu().numpy(), v32[0, tail].cpu().numpy().astype(np.complex128))
    print("c3 shape, last 64 channels: f16 vs fp32 rel err %.3e" % err)
    assert err < TOL_TC
    for p in (p1, p2, p32):
        p.close()


def test_tc_peak_f16_microbenchmark(mdt, cuda):
    """The kind::f16 tcgen05.mma throughput measurement runs, its completion
    wait does not time out, and it lands between a tenth of the nominal 2.25
    PFLOP/s dense figure and the 8192 flops per SM cycle at 2.07 GHz on 152 SMs
    (2.58 PFLOP/s)."""
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    for n, per_sm in ((256, 1), (128, 2)):
        ms, tflops = mdt.tc_peak_f16(n, per_sm, iters=2000, reps=2, err=err)
        print("kind::f16 M128 N%d, %d CTA/SM: %.1f TFLOP/s (%.3f ms)" % (n, per_sm, tflops, ms))
        assert int(err.item()) == 0
        assert 225.0 < tflops < 2580.0


def test_fp32_peak_microbenchmark(mdt, cuda):
    """The FP32 FMA throughput measurement runs for both instruction forms and
    lands between a tenth of the 152 SMs x 128 lanes x 2 flops at 2.07 GHz
    (80.5 TFLOP/s) and twice that figure (a packed f32x2 FMA might retire two
    lanes' worth per lane and cycle)."""
    for packed in (True, False):
        ms, tflops = mdt.fp32_peak(packed, iters=20000, reps=2)
        print("FP32 FMA (%s): %.1f TFLOP/s (%.3f ms)" % ("f32x2" if packed else "f32", tflops, ms))
        assert 8.0 < tflops < 161.0
