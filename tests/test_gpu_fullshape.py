"""Parity at the benchmarked shapes, not reduced ones.

Configuration 3 in full (NE=256, Nch=1024, Ntaps=8, Nsp=8192, 8 integrations
streamed with the PFB history carried), checked on 16 channels (0, Nch/2,
Nch-1 and 13 seeded ones) against the FP64 oracle run on the same samples:
  * f16 and bf16 tensor paths on the first integration (<= 1e-3, <= 4e-3);
  * the exact int8 path at the full K = 8192: the int32 sums of the int8
    F-output bit-exact against the integer oracle on the same channels, the
    stages equal to the plan's visibilities bit for bit, and the plan within
    the int8 quantisation error (<= 2e-2) of FP64;
  * all 8 integrations streamed into the plan's FP64 accumulator against the
    sum of the oracle's per-integration visibilities (<= 1e-3), and against
    the sum of the plan's own per-integration outputs (<= 1e-12).
Configuration 4 in full: the 24 ragged_jobs() in one graph-captured batch,
replayed, bit-equal to single-job plans and within 1e-3 of the FP64 oracle
on 3 channels per job.
The oracle's cost is bounded by the channel subset; the F-engine rows of
every (spectrum, element) are still computed in FP64."""
import numpy as np
import pytest
import torch

from conftest import rel_fro

pytestmark = pytest.mark.gpu

TOL_F16, TOL_BF16, TOL_INT8 = 1e-3, 4e-3, 2e-2


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gen(mdt, cfg, s0, nsp_total):
    out = torch.empty(nsp_total * cfg.nelements * cfg.nchannels * 2, dtype=torch.int8,
                      device="cuda")
    tone = cfg.tone_q16()
    ssig, sdel = cfg.sources()
    mdt.synth_iq(cfg.seed, cfg.nelements, cfg.nchannels, s0, nsp_total, dev(cfg.sigma_q8()),
                 out, tone_q16=None if tone is None else dev(tone),
                 src_sigma_q8=None if ssig is None else dev(ssig),
                 src_delay=None if sdel is None else dev(sdel))
    return out


def window(mdt, nch, ntaps):
    w = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, w)
    return w


class C3Full:
    """The c3 stream on the device and the oracle's per-integration results
    on the channel subset, computed once per module (lazily)."""

    def __init__(self, mdt, oracle):
        self.mdt, self.oracle = mdt, oracle
        self.cfg = cfg = mdt.configs.C3
        self.ne, self.nch, self.ntaps, self.nsp = (cfg.nelements, cfg.nchannels, cfg.ntaps,
                                                   cfg.nspectra)
        self.sb = self.ne * self.nch * 2
        rng = np.random.default_rng(2024)
        extra = rng.choice(np.setdiff1d(np.arange(self.nch), [0, self.nch // 2, self.nch - 1]),
                           13, replace=False)
        self.sel = np.sort(np.concatenate([[0, self.nch // 2, self.nch - 1], extra])).astype(
            np.int32)
        self.iq = gen(mdt, cfg, 0, cfg.total_spectra())
        self.win = window(mdt, self.nch, self.ntaps)
        self.win_h = self.win.cpu().numpy()
        self._ref = {}

    def segment(self, j):
        lo = j * self.nsp * self.sb
        return self.iq[lo:lo + (self.nsp + self.ntaps - 1) * self.sb]

    def ref(self, j):
        if j not in self._ref:
            self._ref[j] = self.oracle.fx(self.segment(j).cpu().numpy(), self.win_h, self.ne,
                                          self.nch, self.ntaps, self.nsp, channels=self.sel)
        return self._ref[j]


@pytest.fixture(scope="module")
def c3(mdt, oracle, cuda):
    state = C3Full(mdt, oracle)
    yield state
    del state.iq
    torch.cuda.empty_cache()


@pytest.mark.parametrize("prec,tol", [(1, TOL_F16), (2, TOL_BF16)])
def test_c3_full_tensor_path_vs_fp64(mdt, c3, prec, tol):
    plan = mdt.FxPlan(c3.ne, c3.nch, c3.ntaps, c3.nsp, precision=prec)
    plan.set_window(c3.win)
    vis = torch.full((c3.nch, c3.ne, c3.ne), float("nan"), dtype=torch.complex64, device="cuda")
    plan.execute(c3.segment(0), 1, vis)
    plan.check()
    plan.close()
    v = vis.cpu().numpy()
    err = rel_fro(v[c3.sel], c3.ref(0))
    print("c3 full shape (K=8192) prec=%d rel err vs FP64 %.3e" % (prec, err))
    assert err < tol
    assert np.all(np.isfinite(v))
    assert np.array_equal(v, np.conj(np.transpose(v, (0, 2, 1))))


def _decode_x16_channels(X16, sel, nch, nsp, ne):
    """int8-valued F-output [k][s][e][2] of the selected channels, decoded
    from the tensor operand rows X16[kc][c][e][128 B] (f16 values, 16-byte
    chunk j of row e stored at j ^ (e & 7))."""
    nep, nkc = (ne + 15) // 16 * 16, (nsp + 31) // 32
    idx = torch.from_numpy(np.asarray(sel, np.int64)).cuda()
    rows = X16.view(nkc, nch, nep, 128)[:, idx].cpu().numpy().view(np.float16)
    rows = rows.reshape(nkc, len(sel), nep, 64)
    L = np.arange(64)
    X = np.zeros((len(sel), nkc * 32, ne, 2), np.float32)
    for e in range(ne):
        p = (((L >> 3) ^ (e & 7)) << 3) | (L & 7)
        lg = rows[:, :, e, :][:, :, p].transpose(1, 0, 2)
        X[:, :, e, 0] = lg[:, :, :32].reshape(len(sel), -1)
        X[:, :, e, 1] = lg[:, :, 32:].reshape(len(sel), -1)
    return X[:, :nsp]


def test_c3_full_int8_exact_sums(mdt, oracle, c3):
    ne, nch, ntaps, nsp = c3.ne, c3.nch, c3.ntaps, c3.nsp
    iq0 = c3.segment(0)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=mdt.MDT_PREC_INT8)
    plan.set_window(c3.win)
    vis = torch.full((nch, ne, ne), float("nan"), dtype=torch.complex64, device="cuda")
    plan.execute(iq0, 1, vis)
    plan.check()
    qs = torch.empty(nch, dtype=torch.float32, device="cuda")
    plan.get_channel_scales(qs)
    plan.close()
    # the plan's stages with its scales: the tensor-core F-engine's int8 output
    X16 = torch.zeros(mdt.x16_bytes(ne, nch, nsp), dtype=torch.uint8, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    mdt.fengine_tc_q8(ne, nch, ntaps, nsp, iq0, c3.win, X16, qs, err)
    raw = torch.empty(nch, ne, ne, 2, dtype=torch.int32, device="cuda")
    v2 = torch.empty_like(vis)
    mdt.xengine_q8(ne, nch, nsp, X16, qs, vis=v2, vis_i32=raw, err=err)
    torch.cuda.synchronize()
    assert err.item() == 0
    assert torch.equal(v2.view(torch.int64), vis.view(torch.int64))
    X = _decode_x16_channels(X16, c3.sel, nch, nsp, ne)
    del X16
    assert np.all(X == np.rint(X)) and np.abs(X).max() <= 127
    ref = oracle.xengine_i8(X.astype(np.int8), ne, len(c3.sel), nsp)
    got = raw[torch.from_numpy(c3.sel.astype(np.int64)).cuda()].cpu().numpy().astype(np.int64)
    assert np.array_equal(got, ref)
    e = rel_fro(vis.cpu().numpy()[c3.sel], c3.ref(0))
    print("c3 full shape int8 path: int32 sums exact on %d channels; rel err vs FP64 %.3e"
          % (len(c3.sel), e))
    assert e < TOL_INT8


def test_c3_eight_integrations_fp64_accumulator(mdt, c3):
    ne, nch, ntaps, nsp, nint = c3.ne, c3.nch, c3.ntaps, c3.nsp, c3.cfg.nint
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=mdt.MDT_PREC_FP16)
    plan.set_window(c3.win)
    acc = torch.zeros(nch, ne, ne, dtype=torch.complex128, device="cuda")
    plan.set_accumulator(acc)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.stream_reset()
    plan.stream_push(c3.segment(0), vis[0])
    for j in range(1, nint):
        lo = (j * nsp + ntaps - 1) * c3.sb
        plan.stream_push(c3.iq[lo:lo + nsp * c3.sb], vis[j])
    plan.check()
    plan.close()
    idx = torch.from_numpy(c3.sel.astype(np.int64)).cuda()
    # the accumulator is the FP64 sum of the per-integration outputs
    want = vis[:, idx].to(torch.complex128).sum(dim=0)
    assert torch.allclose(acc[idx], want, rtol=1e-12, atol=1e-9)
    total = sum(c3.ref(j) for j in range(nint))
    err = rel_fro(acc[idx].cpu().numpy(), total)
    per = [rel_fro(vis[j, idx].cpu().numpy(), c3.ref(j)) for j in range(nint)]
    print("c3 8 integrations: FP64 accumulator rel err %.3e; per integration max %.3e"
          % (err, max(per)))
    assert err < TOL_F16 and max(per) < TOL_F16


def test_c4_all_ragged_jobs(mdt, oracle, cuda):
    jobs = mdt.configs.ragged_jobs()
    shapes = [(j.nelements, j.nchannels, j.ntaps, j.nspectra) for j in jobs]
    batch = mdt.FxBatch(shapes)
    batch.autotune()
    iqs = [gen(mdt, j, 0, j.nspectra + j.ntaps - 1) for j in jobs]
    vis = [torch.full((j.nchannels, j.nelements, j.nelements), float("nan"),
                      dtype=torch.complex64, device="cuda") for j in jobs]
    batch.execute(iqs, vis)           # capture and first replay
    again = [torch.empty_like(v) for v in vis]
    batch.execute(iqs, again)         # replay of the captured graph
    batch.check()
    batch.close()
    worst_plan, worst_oracle = 0.0, 0.0
    for k, j in enumerate(jobs):
        ne, nch, nt, nsp = j.nelements, j.nchannels, j.ntaps, j.nspectra
        assert torch.equal(again[k].view(torch.int64), vis[k].view(torch.int64)), j.name
        win = window(mdt, nch, nt)
        plan = mdt.FxPlan(ne, nch, nt, nsp, precision=mdt.MDT_PREC_FP16)
        plan.set_window(win)
        ref = torch.empty_like(vis[k])
        plan.execute(iqs[k], 1, ref)
        plan.check()
        plan.close()
        v = vis[k].cpu().numpy()
        assert np.all(np.isfinite(v)), j.name
        assert torch.equal(vis[k].view(torch.int64), ref.view(torch.int64)), j.name
        e_plan = rel_fro(v, ref.cpu().numpy().astype(np.complex128))
        sel = [0, nch // 3, nch - 1]
        o = oracle.fx(iqs[k].cpu().numpy(), win.cpu().numpy(), ne, nch, nt, nsp, channels=sel)
        e_or = rel_fro(v[sel], o)
        worst_plan, worst_oracle = max(worst_plan, e_plan), max(worst_oracle, e_or)
        assert e_or < TOL_F16, (j.name, e_or)
    print("c4 24 jobs: batch vs single plans max %.2e, vs FP64 max %.2e"
          % (worst_plan, worst_oracle))
