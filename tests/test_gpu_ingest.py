"""Streaming ingest pipeline (mdt_ingest_*): int8 packets of several
integrations, reordered within a sliding window, some dropped, pushed in
ragged batches -> popped results bit-identical to the plan run on the same
samples (dropped packets' samples zero), per-window missing counts, late
packets dropped, the output ring's back-pressure, graph replay from the third
integration on."""
import numpy as np
import pytest
import torch

from packets import fmt_dict, groups, packetise

pytestmark = pytest.mark.gpu

STATE = 6  # MDT_ERR_STATE


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def run_case(mdt, oracle, ne, nch, ntaps, nsp, nint, sper, formatted, seed, precision=0):
    rng = np.random.default_rng(seed)
    fd = fmt_dict(sper, bits=8)
    S = nsp * nint + ntaps - 1
    assert S * nch % sper == 0
    iq = oracle.synth_iq(seed, ne, nch, 0, S, np.full(ne, 16 * 256, np.int32))
    iq4 = iq.reshape(S, ne, nch, 2)
    pk, ids = packetise(iq4, ne, nch, range(S * nch // sper), fd)
    # drop a few packets inside integrations 1 and 3
    def win_s(x):  # integration window of element-sample x
        spec = x // nch
        return 0 if spec < ntaps - 1 + nsp else (spec - (ntaps - 1)) // nsp
    cand = [i for i, (_, _, c) in enumerate(ids) if win_s(c * sper) in (1, 3)
            and win_s(c * sper + sper - 1) == win_s(c * sper)]
    drop = set(rng.choice(cand, 6, replace=False).tolist())
    zero = iq4.copy()
    grp = {(st, k): (e0, n) for (st, k, e0, n) in groups(ne, fd)}
    missing = {}
    for i in drop:
        st, k, c = ids[i]
        e0, n = grp[(st, k)]
        for s in range(c * sper, c * sper + sper):
            zero[s // nch, e0:e0 + n, s % nch] = 0
        missing[win_s(c * sper)] = missing.get(win_s(c * sper), 0) + 1
    order = [i for i in range(len(pk)) if i not in drop]
    # network reordering: shuffle inside consecutive blocks of 40 packets
    for b0 in range(0, len(order), 40):
        blk = order[b0:b0 + 40]
        rng.shuffle(blk)
        order[b0:b0 + 40] = blk
    stream = pk[order]
    win = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, win)
    fmt = mdt.packet_format(sper, fd["inputs_per_snap"], fd["inputs_per_station"],
                            fd["words_header"], 8, fd["packet_bytes"])
    ing = mdt.Ingest(ne, nch, ntaps, nsp, fmt, max_packets=64, formatted=formatted,
                     precision=precision)
    ing.set_window(win)
    results = {}
    stats = {}
    buf = np.empty(ing.out_bytes, np.uint8)

    def drain(wait):
        while True:
            it, st = ing.pop(buf, wait=wait)
            if it < 0:
                return
            results[it] = buf.view(np.complex64).copy()
            stats[it] = st

    p = 0
    while p < len(stream):
        n = int(rng.integers(1, 65))
        batch = np.ascontiguousarray(stream[p:p + n])
        try:
            ing.push(batch)
        except mdt.MdtError as e:
            assert e.code == STATE
            drain(True)
            ing.push(batch)
        p += n
        drain(False)
    ing.flush()
    drain(True)
    drain(True)
    # a packet for integration 0 now is late
    ing.push(np.ascontiguousarray(pk[:1]))
    cnt = ing.counters()
    ing.close()
    assert cnt["late"] == 1 and cnt["bad"] == 0
    assert sorted(results) == list(range(nint))
    # expected: the plan over the same samples with the dropped ones zero
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=precision)
    plan.set_window(win)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(dev(zero.reshape(-1)), nint, vis)
    nbl = mdt.num_baselines(ne, 1)
    for n in range(nint):
        if formatted:
            f = torch.empty(nbl, nch, dtype=torch.complex64, device="cuda")
            mdt.format_baselines(ne, 1, nch, vis[n], f)
            want = f.cpu().numpy().reshape(-1)
        else:
            want = vis[n].cpu().numpy().reshape(-1)
        assert np.array_equal(results[n].view(np.uint64), want.view(np.uint64)), n
        assert stats[n]["missing"] == missing.get(n, 0), (n, stats[n])
        assert stats[n]["duplicate"] == 0
    plan.close()


@pytest.mark.parametrize("formatted", [False, True])
def test_ingest_stream_matches_plan(mdt, cuda, oracle, formatted):
    run_case(mdt, oracle, ne=38, nch=256, ntaps=4, nsp=64, nint=6, sper=32,
             formatted=formatted, seed=3 + formatted)


def test_ingest_tensor_path_graphs(mdt, cuda, oracle):
    # f16 tensor path at Nch 1024: the tensor-core F-engine and X-engine run
    # eagerly for two windows, then from graphs replayed per buffer parity
    run_case(mdt, oracle, ne=38, nch=1024, ntaps=8, nsp=64, nint=4, sper=32, formatted=False,
             seed=21, precision=1)


def test_ingest_packets_straddling_windows(mdt, cuda, oracle):
    # 48 samples per packet do not divide Nsp*Nch: packets span two windows
    run_case(mdt, oracle, ne=76, nch=128, ntaps=8, nsp=32, nint=4, sper=48, formatted=False,
             seed=9)


def test_ingest_back_pressure_and_errors(mdt, cuda, oracle):
    ne, nch, ntaps, nsp, sper = 38, 64, 4, 16, 16
    fd = fmt_dict(sper, bits=8)
    fmt = mdt.packet_format(sper, sample_bits=8)
    ing = mdt.Ingest(ne, nch, ntaps, nsp, fmt, max_packets=8)
    win = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    with pytest.raises(mdt.MdtError):      # no window yet
        ing.push(np.zeros((1, fd["packet_bytes"]), np.uint8))
    mdt.window_hamming_sinc(nch, ntaps, win)
    ing.set_window(win)
    S = nsp * 8 + ntaps - 1
    iq = np.zeros((S, ne, nch, 2), np.int8)
    pk, ids = packetise(iq, ne, nch, range(S * nch // sper), fd)
    far = [i for i, (_, _, c) in enumerate(ids) if c * sper // nch == ntaps - 1 + 6 * nsp]
    with pytest.raises(mdt.MdtError) as ei:   # would close windows 0..4: ring holds 3
        ing.push(np.ascontiguousarray(pk[far[:1]]))
    assert ei.value.code == STATE
    with pytest.raises(mdt.MdtError):         # more than max_packets
        ing.push(np.ascontiguousarray(pk[:9]))
    assert ing.counters()["next_window"] == 0
    ing.close()
    with pytest.raises(mdt.MdtError):         # 32-bit packets are for the drop-in path
        mdt.Ingest(ne, nch, ntaps, nsp, mdt.packet_format(sper), max_packets=8)
