"""GPU depacketiser (mdt_depacketise) against the restated rank-1 loop
(oracle.depacketise, MDT_OneStation_client.cu:846-907): bit-exact output,
window edges, bad headers, packet gaps (zero fill and counts), duplicates,
batches delivered over several calls, and packets -> depacketise -> fused plan
equal to the plan on the original int8 I/Q."""
import numpy as np
import pytest
import torch

from packets import fixed19, fmt_dict, groups, packetise

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


class Depack:
    def __init__(self, mdt, fd, ne, nch, sample0, nsp):
        self.mdt, self.ne, self.nch, self.s0, self.nsp = mdt, ne, nch, sample0, nsp
        self.fmt = mdt.packet_format(fd["sper_element"], fd["inputs_per_snap"],
                                     fd["inputs_per_station"], fd["words_header"],
                                     fd["sample_bits"], fd["packet_bytes"])
        n = mdt.depacketise_seen_words(self.fmt, ne, nch, sample0, nsp)
        self.seen = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
        self.stats = torch.zeros(5, dtype=torch.int64, device="cuda")
        if fd["sample_bits"] == 32:
            self.out = torch.full((nsp, ne, nch), complex(7, 7), dtype=torch.complex64,
                                  device="cuda")
        else:
            self.out = torch.full((nsp, ne, nch, 2), 7, dtype=torch.int8, device="cuda")

    def push(self, pk):
        if len(pk):
            self.mdt.depacketise(self.fmt, dev(pk), len(pk), self.ne, self.nch, self.s0,
                                 self.nsp, self.out, self.seen, self.stats)

    def finish(self):
        self.mdt.depacketise_finish(self.fmt, self.ne, self.nch, self.s0, self.nsp, self.out,
                                    self.seen, self.stats)
        torch.cuda.synchronize()
        return dict(zip(self.mdt.STATS_FIELDS, self.stats.cpu().tolist()))


def rand_words(rng, shape):
    w = rng.integers(0, 2 ** 32, size=shape, dtype=np.uint64).astype(np.uint32)
    flat = w.reshape(-1)
    flat[rng.choice(flat.size, 64, replace=False)] = rng.choice(
        np.array([0, 1, 0x7FFFFFFF, 0x80000000, 0x80000001, 0xFFFFFFFF, 0x01000001],
                 np.uint32), 64)
    return w


@pytest.mark.parametrize("ne,nch,sper,s0sp,nsp", [(38, 64, 16, 2, 6), (76, 128, 108, 1, 9),
                                                  (10, 32, 7, 0, 5)])
def test_depack_i32_bit_exact(mdt, cuda, oracle, ne, nch, sper, s0sp, nsp):
    rng = np.random.default_rng(ne + sper)
    fd = fmt_dict(sper)
    total = (s0sp + nsp + 2) * nch
    words = rand_words(rng, (total // nch, ne, nch, 2))
    pk, ids = packetise(words, ne, nch, range(total // sper), fd)
    bad = pk[:2].copy()
    bad[0, 4:8] = np.array([9], np.uint32).view(np.uint8)        # no SNAP 9
    bad[1, 0:4] = np.array([1000], np.uint32).view(np.uint8)     # no station 1000
    pk = np.concatenate([pk, bad])[rng.permutation(len(pk) + 2)]
    d = Depack(mdt, fd, ne, nch, s0sp * nch, nsp)
    d.push(pk[: len(pk) // 2])
    d.push(pk[len(pk) // 2:])
    st = d.finish()
    want, ost = oracle.depacketise(fd, pk, len(pk), ne, nch, s0sp * nch, nsp)
    got = d.out.cpu().numpy()
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    assert [st["accepted"], st["outside"], st["bad"]] == ost
    assert st["missing"] == 0 and st["duplicate"] == 0
    # and the oracle is the reference's conversion of the words
    ref = fixed19(words[s0sp:s0sp + nsp, ..., 0]) + 1j * fixed19(words[s0sp:s0sp + nsp, ..., 1])
    assert np.array_equal(want, ref.astype(np.complex64))


def test_depack_gaps_and_duplicates(mdt, cuda, oracle):
    ne, nch, sper, nsp = 38, 64, 16, 4
    rng = np.random.default_rng(5)
    fd = fmt_dict(sper)
    words = rand_words(rng, (nsp, ne, nch, 2))
    pk, ids = packetise(words, ne, nch, range(nsp * nch // sper), fd)
    drop = set(rng.choice(len(pk), 5, replace=False).tolist())
    keep = [p for p in range(len(pk)) if p not in drop]
    dup = keep[:3]
    sel = pk[keep + dup]
    d = Depack(mdt, fd, ne, nch, 0, nsp)
    d.push(sel)
    st = d.finish()
    assert st["missing"] == 5 and st["duplicate"] == 3
    assert st["accepted"] == len(sel)
    want, _ = oracle.depacketise(fd, sel, len(sel), ne, nch, 0, nsp)   # zeros where missing
    assert np.array_equal(d.out.cpu().numpy().view(np.uint64), want.view(np.uint64))
    # the next window starts clean: all packets present, nothing missing
    d.stats.zero_()
    d.push(pk)
    st = d.finish()
    assert st["missing"] == 0 and st["duplicate"] == 0


def test_depack_i8_into_plan(mdt, cuda, oracle):
    """Packets carrying int8 I/Q -> depacketise -> FP32 plan equals the plan
    run on the I/Q directly (bit-identical visibilities)."""
    ne, nch, ntaps, nsp, sper = 38, 256, 4, 64, 32
    fd = fmt_dict(sper, bits=8)
    S = nsp + ntaps - 1
    iq = oracle.synth_iq(17, ne, nch, 0, S, np.full(ne, 16 * 256, np.int32))
    iq4 = iq.reshape(S, ne, nch, 2)
    pk, _ = packetise(iq4, ne, nch, range(S * nch // sper), fd)
    pk = pk[np.random.default_rng(2).permutation(len(pk))]
    d = Depack(mdt, fd, ne, nch, 0, S)
    d.push(pk)
    st = d.finish()
    assert st["missing"] == 0 and st["accepted"] == len(pk)
    assert np.array_equal(d.out.cpu().numpy(), iq4)
    win = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, win)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp)
    plan.set_window(win)
    v1 = torch.empty(nch, ne, ne, dtype=torch.complex64, device="cuda")
    v2 = torch.empty_like(v1)
    plan.execute(d.out.view(-1), 1, v1)
    plan.execute(dev(iq), 1, v2)
    torch.cuda.synchronize()
    assert torch.equal(v1.view(torch.int64), v2.view(torch.int64))
    plan.close()


def test_depack_rejects_bad_formats(mdt, cuda):
    out = torch.zeros(16, dtype=torch.complex64, device="cuda")
    seen = torch.zeros(16, dtype=torch.int32, device="cuda")
    stats = torch.zeros(5, dtype=torch.int64, device="cuda")
    pk = torch.zeros(1024, dtype=torch.uint8, device="cuda")
    with pytest.raises(mdt.MdtError):   # window start not a multiple of Nch
        mdt.depacketise(mdt.packet_format(4), pk, 1, 38, 8, 3, 2, out, seen, stats)
    with pytest.raises(mdt.MdtError):   # packet_bytes too small for the largest SNAP
        mdt.depacketise(mdt.packet_format(4, packet_bytes=64), pk, 1, 38, 8, 0, 2, out, seen,
                        stats)
    with pytest.raises(mdt.MdtError):   # SNAP inputs exceed a station
        mdt.depacketise(mdt.packet_format(4, inputs_per_snap=(30, 30)), pk, 1, 38, 8, 0, 2, out,
                        seen, stats)
    assert len(groups(38, fmt_dict(4))) == 4
