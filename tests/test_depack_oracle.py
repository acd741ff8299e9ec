"""The depacketiser oracle (restated rank-1 loop, MDT_OneStation_client.cu:
846-907) on the CPU: known answers of the int32 x 2^-19 conversion, element /
channel placement of a hand-built packet, window handling and the packet
round trip."""
import numpy as np

from packets import fixed19, fmt_dict, groups, packetise


def test_fixed19_known_answers(oracle):
    fmt = fmt_dict(sper=1, snaps=(1,), ips=1)
    cases = {
        0x00000000: 0.0,
        0x00000001: 2.0 ** -19,
        0xFFFFFFFF: -(2.0 ** -19),
        0x00080000: 1.0,
        0xFFF80000: -1.0,
        0x7FFFFFFF: 4096.0,            # 2^31 - 1 rounds to 2^31 in float
        0x80000001: -4096.0,           # -(2^31 - 1) rounds likewise
        0x80000000: 4096.0,            # the reference's int wrap: +4096, not -4096
        0x00FFFFFF: (2 ** 24 - 1) * 2.0 ** -19,
        0x01000001: 2 ** 24 * 2.0 ** -19,  # 2^24 + 1 -> 2^24 (ties to even)
        0x01000003: (2 ** 24 + 4) * 2.0 ** -19,  # 2^24 + 3 -> 2^24 + 4
    }
    ws = np.array(list(cases.keys()), np.uint32)
    words = np.stack([ws, ws[::-1]], axis=-1).reshape(len(ws), 1, 1, 2)
    pk, _ = packetise(words, 1, 1, range(len(ws)), fmt)
    out, st = oracle.depacketise(fmt, pk, len(ws), 1, 1, 0, len(ws))
    want = np.array(list(cases.values()), np.float64)
    assert np.array_equal(out.real.ravel(), want.astype(np.float32))
    assert np.array_equal(out.imag.ravel(), want[::-1].astype(np.float32))
    assert np.array_equal(fixed19(ws), want.astype(np.float32))
    assert st == [len(ws), 0, 0]


def test_placement_of_one_packet(oracle):
    fmt = fmt_dict(sper=4)
    ne, nch = 38, 8
    pk = np.zeros((1, fmt["packet_bytes"]), np.uint8)
    pk[0, :12] = np.array([0, 2, 3], np.uint32).view(np.uint8)   # station 0, SNAP 2, counter 3
    pay = np.arange(4 * 10 * 2, dtype=np.uint32) << 19           # sample (i, j) re = 2(10i+j)
    pk[0, 16:16 + pay.nbytes] = pay.view(np.uint8)
    out, st = oracle.depacketise(fmt, pk, 1, ne, nch, 0, 2)
    assert st == [1, 0, 0]
    # samples 12..15 -> spectrum 1, channels 4..7; SNAP 2 -> elements 20..29
    for i in range(4):
        for j in range(10):
            assert out[1, 20 + j, 4 + i] == complex(2 * (10 * i + j), 2 * (10 * i + j) + 1)
    mask = np.zeros(out.shape, bool)
    mask[1, 20:30, 4:8] = True
    assert np.all(out[~mask] == 0)


def test_window_and_bad_headers(oracle):
    fmt = fmt_dict(sper=6)
    ne, nch = 76, 16
    rng = np.random.default_rng(0)
    words = rng.integers(0, 2 ** 32, size=(12, ne, nch, 2), dtype=np.uint64).astype(np.uint32)
    counters = range(0, 12 * nch // 6)
    pk, ids = packetise(words, ne, nch, counters, fmt)
    bad = pk[:2].copy()
    bad[0, 4:8] = np.array([7], np.uint32).view(np.uint8)        # SNAP 7 does not exist
    bad[1, 0:4] = np.array([5], np.uint32).view(np.uint8)        # station 5 > NE
    allp = np.concatenate([pk, bad])
    sample0, nsp = 3 * nch, 5                                     # window: spectra 3..7
    out, st = oracle.depacketise(fmt, allp, len(allp), ne, nch, sample0, nsp)
    assert st[2] == 2
    want = fixed19(words[3:8, ..., 0]) + 1j * fixed19(words[3:8, ..., 1])
    assert np.array_equal(out, want.astype(np.complex64))
    inside = sum(1 for (_, _, c) in ids if c * 6 < sample0 + nsp * nch and c * 6 + 6 > sample0)
    assert st[0] == inside and st[1] == len(ids) - inside


def test_int8_round_trip(oracle):
    fmt = fmt_dict(sper=16, bits=8)
    ne, nch = 38, 32
    rng = np.random.default_rng(1)
    iq = rng.integers(-128, 128, size=(4, ne, nch, 2), dtype=np.int64).astype(np.int8)
    pk, ids = packetise(iq, ne, nch, range(4 * nch // 16), fmt)
    order = rng.permutation(len(pk))
    out, st = oracle.depacketise(fmt, pk[order], len(pk), ne, nch, 0, 4)
    assert np.array_equal(out, iq)
    assert st == [len(pk), 0, 0]
    assert len(groups(ne, fmt)) == 4
