"""GPU output formatter (mdt_format_baselines) against the reference's output
loop restated in numpy (MDT_OneStation_client.cu:1239-1266): baseline order,
fftshift, column-major element pick; bit-exact (a gather).  End to end:
plan -> format -> CSV equals the reference's lines for the same
visibilities."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def ref_gather(V, nel, npol, nch, shift=True):
    """V: complex64 [Nch][NE*NE] column-major -> [nbl][Nch] in the reference order."""
    ne = nel * npol
    rows = []
    for j in range(nel):
        for p in range(npol):
            for k in range(j, nel):
                for q in range(p, npol):
                    idx = (k * npol + q) * ne + (j * npol + p)
                    chans = ([*range(nch // 2, nch), *range(0, nch // 2)] if shift
                             else list(range(nch)))
                    rows.append(V[chans, idx])
    return np.stack(rows)


@pytest.mark.parametrize("nel,npol,nch", [(5, 1, 64), (37, 1, 96), (6, 2, 32), (40, 2, 16),
                                          (1, 1, 2)])
def test_format_baselines_bit_exact(mdt, cuda, nel, npol, nch):
    ne = nel * npol
    rng = np.random.default_rng(ne + nch)
    V = (rng.standard_normal((nch, ne * ne)) + 1j * rng.standard_normal((nch, ne * ne)))
    V = V.astype(np.complex64)
    nbl = mdt.num_baselines(nel, npol)
    for shift in (True, False):
        out = torch.full((nbl, nch), complex(9, 9), dtype=torch.complex64, device="cuda")
        mdt.format_baselines(nel, npol, nch, torch.from_numpy(V).cuda(), out, fftshift=shift)
        torch.cuda.synchronize()
        want = ref_gather(V, nel, npol, nch, shift)
        assert np.array_equal(out.cpu().numpy().view(np.uint64), want.view(np.uint64))


def test_plan_to_csv(mdt, cuda, oracle, tmp_path):
    ne, nch, ntaps, nsp = 12, 64, 4, 128
    iq = oracle.synth_iq(5, ne, nch, 0, nsp + ntaps - 1, np.full(ne, 16 * 256, np.int32))
    win = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, win)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp)
    plan.set_window(win)
    vis = torch.empty(nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(torch.from_numpy(iq).cuda(), 1, vis)
    nbl = mdt.num_baselines(ne, 1)
    out = torch.empty(nbl, nch, dtype=torch.complex64, device="cuda")
    mdt.format_baselines(ne, 1, nch, vis, out)
    host = out.cpu().numpy()
    plan.close()
    path = tmp_path / "MDT_test.csv"
    mdt.write_csv(str(path), ne, 1, nch, host)
    V = vis.cpu().numpy().reshape(nch, ne * ne)
    want = ref_gather(V, ne, 1, nch)
    lines = []
    b = 0
    for j in range(ne):
        for k in range(j, ne):
            for z in range(nch):
                v = want[b, z]
                lines.append("%d,0,%d,0,%d,%.6f,%.6f\n" % (j, k, z, float(v.real), float(v.imag)))
            b += 1
    assert path.read_text() == "".join(lines)
