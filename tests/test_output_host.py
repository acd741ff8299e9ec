"""Host writers of the output formatter (no GPU needed): the CSV lines are
byte-identical to the reference's fprintf("%ld,%d,%ld,%d,%ld,%.6f,%.6f\n")
loop (MDT_OneStation_client.cu:1239-1266) over the baseline-major buffer,
for any thread count; the binary form round-trips."""
import numpy as np
import pytest

EDGE = [0.0, -0.0, 0.0078125, 0.0234375, -0.0078125, 1e-9, -1e-9, 5e-7, -5e-7, 4.9999997e-7,
        1.4e-45, -1.4e-45, 1.1754944e-38, 0.1, 0.3333333, 2.5, 123456.789, -98765.4321,
        8589934591.0, 8589934592.0, -8589934592.0, 1e20, -3.4028235e38, float("inf"),
        float("-inf"), 4096.0, 1.9073486e-06]


def ref_lines(F, nel, npol, nch):
    out = []
    b = 0
    for j in range(nel):
        for p in range(npol):
            for k in range(j, nel):
                for q in range(p, npol):
                    for z in range(nch):
                        v = F[b, z]
                        out.append("%d,%d,%d,%d,%d,%.6f,%.6f\n"
                                   % (j, p, k, q, z, float(v.real), float(v.imag)))
                    b += 1
    return "".join(out)


@pytest.mark.parametrize("nel,npol,nch", [(3, 2, 4), (5, 1, 8), (1, 1, 2)])
def test_csv_matches_reference_format(mdt, tmp_path, nel, npol, nch):
    rng = np.random.default_rng(nel * 10 + npol)
    nbl = mdt.num_baselines(nel, npol)
    assert nbl == npol * (npol + 1) // 2 * nel * (nel + 1) // 2
    vals = (rng.standard_normal(2 * nbl * nch) * 10.0 ** rng.integers(-8, 9, 2 * nbl * nch))
    vals = vals.astype(np.float32)
    vals[:min(len(EDGE), vals.size)] = np.array(EDGE, np.float32)[:vals.size]
    F = vals.view(np.complex64).reshape(nbl, nch)
    want = ref_lines(F, nel, npol, nch)
    for nth in (1, 3):
        path = tmp_path / ("v%d.csv" % nth)
        mdt.write_csv(str(path), nel, npol, nch, F, nthreads=nth)
        assert path.read_text() == want
    mdt.write_csv(str(path), nel, npol, nch, F, append=True, nthreads=2)
    assert path.read_text() == want + want


def test_csv_fixed_point_rounding_exhaustive_slice(mdt, tmp_path):
    """Every float32 in a few bit ranges (ties at odd multiples of 2^-7 and of
    2^-8, sub-1e-6 values, large values) formats as Python's correctly rounded
    %.6f does."""
    parts = [np.arange(0x3C000000, 0x3C000000 + 20000, dtype=np.uint32),   # ~0.0078
             np.arange(0x35800000, 0x35800000 + 20000, dtype=np.uint32),   # ~1e-6
             np.arange(0x4F000000 - 10000, 0x4F000000 + 10000, dtype=np.uint32),  # ~2^31
             np.arange(0x50000000 - 10000, 0x50000000 + 10000, dtype=np.uint32)]  # ~2^33
    bits = np.concatenate(parts)
    bits = np.concatenate([bits, bits | np.uint32(0x80000000)])
    n = bits.size // 2 * 2
    F = bits[:n].view(np.float32).view(np.complex64).reshape(-1, 1)
    nbl = F.shape[0]
    nel = int((np.sqrt(8 * nbl + 1) - 1) / 2)
    while nel * (nel + 1) // 2 < nbl:
        nel += 1
    G = np.zeros((nel * (nel + 1) // 2, 1), np.complex64)
    G[:nbl] = F
    path = tmp_path / "x.csv"
    mdt.write_csv(str(path), nel, 1, 1, G, nthreads=4)
    assert path.read_text() == ref_lines(G, nel, 1, 1)


def test_binary_round_trip(mdt, tmp_path):
    nel, npol, nch = 4, 2, 16
    nbl = mdt.num_baselines(nel, npol)
    rng = np.random.default_rng(3)
    F = (rng.standard_normal((nbl, nch)) + 1j * rng.standard_normal((nbl, nch))).astype(np.complex64)
    path = tmp_path / "v.bin"
    mdt.write_binary(str(path), nel, npol, nch, F)
    raw = path.read_bytes()
    assert raw[:8] == b"MDTVIS01"
    hdr = np.frombuffer(raw[8:32], np.int32)
    assert hdr[:4].tolist() == [nel, npol, nch, nbl]
    tab = np.frombuffer(raw[32:32 + 16 * nbl], np.int32).reshape(nbl, 4)
    want = [(j, p, k, q) for j in range(nel) for p in range(npol) for k in range(j, nel)
            for q in range(p, npol)]
    assert [tuple(t) for t in tab.tolist()] == want
    data = np.frombuffer(raw[32 + 16 * nbl:], np.complex64).reshape(nbl, nch)
    assert np.array_equal(data, F)
    with pytest.raises(mdt.MdtError):
        mdt.write_binary(str(tmp_path / "no" / "such" / "dir.bin"), nel, npol, nch, F)
