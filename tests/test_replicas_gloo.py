"""Replicas-only multi-GPU host logic on CPU ranks (gloo, world size 2):
each rank generates only its own span of one I/Q stream (the generator is
counter-based), runs the FP64 oracle pipeline on its integrations, and the
gather at rank 0 equals the single-process run over the whole stream,
bit for bit.  Plus the split arithmetic and the job split."""
import importlib
import os
import socket

import numpy as np
import pytest

from conftest import PKG_NAME, ROOT

torch = pytest.importorskip("torch")


def rep():
    return importlib.import_module(PKG_NAME + ".replicas")


def test_integration_split_covers_stream():
    R = rep()
    for total in (0, 1, 5, 16, 17):
        for world in (1, 2, 3, 8):
            got = [R.integration_split(total, r, world) for r in range(world)]
            assert sum(c for _, c in got) == total
            nxt = 0
            for f, c in got:
                assert f == nxt
                nxt += c
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    assert R.input_span(3, 2, 100, 8) == (300, 207)


def test_job_split_balanced():
    R = rep()
    costs = [float(c) for c in np.random.default_rng(0).integers(1, 100, 24)]
    parts = R.job_split(costs, 4)
    assert sorted(j for p in parts for j in p) == list(range(24))
    loads = [sum(costs[j] for j in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert R.job_split(costs, 4) == parts


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, cfg, out_path):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle
    R = importlib.import_module(PKG_NAME + ".replicas")
    ne, nch, ntaps, nsp, nint, seed = cfg
    first, cnt = R.integration_split(nint, rank, world)
    s0, nspan = R.input_span(first, cnt, nsp, ntaps)
    sig = np.full(ne, 16 * 256, np.int32)
    iq = oracle.synth_iq(seed, ne, nch, s0, nspan, sig).reshape(nspan, -1)
    win = oracle.window_hamming_sinc(nch, ntaps)
    vis = np.stack([oracle.fx(iq[j * nsp:j * nsp + nsp + ntaps - 1].reshape(-1), win, ne, nch,
                              ntaps, nsp) for j in range(cnt)])
    got = R.gather_integrations(torch.from_numpy(vis), nint, rank, world)
    if rank == 0:
        np.save(out_path, got.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_stream_equals_single_process(oracle, tmp_path):
    import torch.multiprocessing as mp
    cfg = (4, 64, 4, 24, 5, 77)  # NE, Nch, Ntaps, Nsp, integrations, seed
    out = str(tmp_path / "gathered.npy")
    mp.start_processes(_worker, args=(2, _free_port(), cfg, out), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(out)
    ne, nch, ntaps, nsp, nint, seed = cfg
    S = nint * nsp + ntaps - 1
    iq = oracle.synth_iq(seed, ne, nch, 0, S, np.full(ne, 16 * 256, np.int32)).reshape(S, -1)
    win = oracle.window_hamming_sinc(nch, ntaps)
    want = np.stack([oracle.fx(iq[j * nsp:j * nsp + nsp + ntaps - 1].reshape(-1), win, ne, nch,
                               ntaps, nsp) for j in range(nint)])
    assert got.shape == want.shape
    assert np.array_equal(got, want)
