"""Batched jobs of uneven shape (one graph-captured launch set, persistent
tensor-core X-engine, autotuned tiles) against the single-job f16 plan and
the FP64 oracle."""
import numpy as np
import pytest
import torch

from conftest import rel_fro

pytestmark = pytest.mark.gpu

JOBS = [(8, 256, 4, 64), (40, 512, 8, 100), (130, 256, 8, 70), (17, 1024, 4, 33),
        (64, 512, 4, 300), (3, 2048, 8, 2)]


def gen(mdt, cfg, total):
    out = torch.empty(total * cfg.nelements * cfg.nchannels * 2, dtype=torch.int8, device="cuda")
    tone = cfg.tone_q16()
    mdt.synth_iq(cfg.seed, cfg.nelements, cfg.nchannels, 0, total,
                 torch.from_numpy(cfg.sigma_q8()).cuda(), out,
                 tone_q16=None if tone is None else torch.from_numpy(tone).cuda())
    return out


def inputs(mdt, seed_shift=0):
    iqs, cfgs = [], []
    for k, (ne, nch, nt, nsp) in enumerate(JOBS):
        cfg = mdt.configs.Config("job%d" % k, ne, nch, nt, nsp, 1, seed=900 + k + seed_shift,
                                 sigma=(12.0, 20.0), tones=[(None, 8.0)])
        iqs.append(gen(mdt, cfg, nsp + nt - 1))
        cfgs.append(cfg)
    return iqs, cfgs


def test_batch_matches_single_job_plans_and_oracle(mdt, cuda, oracle):
    batch = mdt.FxBatch(JOBS)
    maxw, cost_order = batch.autotune()
    assert maxw in (64, 128)
    iqs, _ = inputs(mdt)
    vis = [torch.full((nch, ne, ne), float("nan"), dtype=torch.complex64, device="cuda")
           for ne, nch, nt, nsp in JOBS]
    batch.execute(iqs, vis, use_graph=True)
    batch.check()
    direct = [torch.empty_like(v) for v in vis]
    batch.execute(iqs, direct, use_graph=False)
    batch.check()
    for k, (ne, nch, nt, nsp) in enumerate(JOBS):
        v = vis[k].cpu().numpy()
        assert np.all(np.isfinite(v)), k
        assert torch.equal(direct[k].view(torch.int64), vis[k].view(torch.int64)), k
        win = torch.empty(nch * nt, dtype=torch.float32, device="cuda")
        mdt.window_hamming_sinc(nch, nt, win)
        plan = mdt.FxPlan(ne, nch, nt, nsp, precision=mdt.MDT_PREC_FP16)
        plan.set_window(win)
        ref = torch.empty_like(vis[k])
        plan.execute(iqs[k], 1, ref)
        plan.check()
        plan.close()
        r = ref.cpu().numpy()
        assert rel_fro(v, r.astype(np.complex128)) < 1e-6, k
        sel = [0, nch // 3, nch - 1]
        o = oracle.fx(iqs[k].cpu().numpy(), win.cpu().numpy(), ne, nch, nt, nsp, channels=sel)
        assert rel_fro(v[sel], o) < 1e-3, k
    batch.close()


def test_batch_replay_with_new_buffers(mdt, cuda):
    batch = mdt.FxBatch(JOBS)
    iqs, _ = inputs(mdt)
    vis = [torch.empty((nch, ne, ne), dtype=torch.complex64, device="cuda")
           for ne, nch, nt, nsp in JOBS]
    batch.execute(iqs, vis)
    iqs2, _ = inputs(mdt, seed_shift=50)
    vis2 = [torch.empty_like(v) for v in vis]
    batch.execute(iqs2, vis2)  # the same captured graph, new pointers in the job tables
    batch.check()
    vis3 = [torch.empty_like(v) for v in vis]
    batch.execute(iqs2, vis3, use_graph=False)
    batch.check()
    for a, b, c in zip(vis, vis2, vis3):
        assert torch.equal(b.view(torch.int64), c.view(torch.int64))
        assert not torch.equal(a.view(torch.int64), b.view(torch.int64))
    batch.close()


def test_batch_rejects_unsupported_jobs(mdt, cuda):
    with pytest.raises(mdt.MdtError):
        mdt.FxBatch([(8, 256, 6, 64)])  # Ntaps 6
    with pytest.raises(mdt.MdtError):
        mdt.FxBatch([(8, 4096, 4, 64)])  # Nch above 2048
