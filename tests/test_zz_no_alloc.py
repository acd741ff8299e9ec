"""mdt_fx_integrate_static -- one FP32 FX integration that allocates no device
memory, for callers that cannot allocate (a real-time ingest loop that must
not take cudaMalloc's device synchronisation, a plugin host with a fixed
device-memory budget, a foreign runtime that owns all allocations).  Its
F-engine output and FFT twiddles live in the library's file-scope device
arrays.  Called through the C ABI with ctypes, twice in a row with different
shapes (the second call reuses the scratch the first one left behind), and
checked against the plan entry point mdt_fx_execute within the FP32 path's
tolerance.  This file is collected last so that a stop at its first failure
leaves every other test already run."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_fro

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5  # the FP32 path's tolerance (vs FP64 and between FP32 entry points)
MDT_ERR_INVALID_VALUE = 1


def _entry(mdt):
    f = mdt.lib().mdt_fx_integrate_static
    f.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 4
    f.restype = ctypes.c_int
    return f


def _inputs(mdt, cfg):
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    total = nsp + ntaps - 1
    iq = torch.empty(total * ne * nch * 2, dtype=torch.int8, device="cuda")
    tone = cfg.tone_q16()
    mdt.synth_iq(cfg.seed, ne, nch, 0, total,
                 torch.from_numpy(cfg.sigma_q8()).cuda(), iq,
                 tone_q16=None if tone is None else torch.from_numpy(tone).cuda())
    win = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, win)
    return iq, win


def test_integrate_static_matches_plan_two_calls(mdt, cuda):
    f = _entry(mdt)
    stream = torch.cuda.current_stream().cuda_stream
    cases = [mdt.configs.C1,  # NE=10, Nch=1024, Ntaps=4, Nsp=1000: 82 MB of scratch
             mdt.configs.small(mdt.configs.C2, nspectra=120, nint=1)]  # NE=40, Nch=2048, Ntaps=8
    for cfg in cases:
        ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
        iq, win = _inputs(mdt, cfg)
        vis = torch.full((nch, ne, ne), float("nan"), dtype=torch.complex64, device="cuda")
        rc = f(ne, nch, ntaps, nsp, iq.data_ptr(), win.data_ptr(), vis.data_ptr(), stream)
        assert rc == 0, mdt.lib().mdt_last_error()
        plan = mdt.FxPlan(ne, nch, ntaps, nsp)
        plan.set_window(win)
        ref = torch.full_like(vis, float("nan"))
        plan.execute(iq, 1, ref)
        torch.cuda.synchronize()
        plan.close()
        v, r = vis.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(v))
        assert rel_fro(v, r.astype(np.complex128)) < TOL_FP32, cfg.name


def test_integrate_static_rejects_oversized_request(mdt, cuda):
    f = _entry(mdt)
    ne, nch, ntaps, nsp = 256, 1024, 8, 1024  # 2 GiB of F-output: beyond the scratch
    iq = torch.zeros((nsp + ntaps - 1) * ne * nch * 2, dtype=torch.int8, device="cuda")
    win = torch.zeros(nch * ntaps, dtype=torch.float32, device="cuda")
    vis = torch.zeros(nch * ne * ne, dtype=torch.complex64, device="cuda")
    rc = f(ne, nch, ntaps, nsp, iq.data_ptr(), win.data_ptr(), vis.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    assert rc == MDT_ERR_INVALID_VALUE
    assert b"static scratch" in mdt.lib().mdt_last_error()
