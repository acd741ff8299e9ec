"""mdt_fx_integrate_static -- one FP32 FX integration that allocates no device
memory, for callers that cannot allocate (a real-time ingest loop that must
not take cudaMalloc's device synchronisation, a plugin host with a fixed
device-memory budget, a foreign runtime that owns all allocations).  Its
F-engine output and FFT twiddles live in the library's file-scope device
arrays.

Called through the C ABI with ctypes, several times in a row with different
shapes (each call reuses the scratch the previous one left behind):
  * free device memory is the same before and after the calls that follow
    the first one (the first call on a device loads the module holding the
    arrays);
  * the output equals the plan entry point mdt_fx_execute bit for bit (both
    run the same F-engine and X-engine with the same twiddle values);
  * the output is within the FP32 path's 1e-5 of the FP64 oracle;
  * shapes the entry point cannot serve are rejected with
    MDT_ERR_INVALID_VALUE and a message.
This file is collected last so that a stop at its first failure leaves every
other test already run."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_fro

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5  # the FP32 path's tolerance against the FP64 oracle
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
    vis = torch.full((nch, ne, ne), float("nan"), dtype=torch.complex64, device="cuda")
    return iq, win, vis


def _call(mdt, f, cfg, iq, win, vis):
    rc = f(cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra, iq.data_ptr(),
           win.data_ptr(), vis.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, mdt.lib().mdt_last_error()


def test_integrate_static_matches_plan_and_oracle(mdt, oracle, cuda):
    f = _entry(mdt)
    cases = [mdt.configs.C1,  # NE=10, Nch=1024, Ntaps=4, Nsp=1000: 82 MB of scratch
             mdt.configs.small(mdt.configs.C2, nspectra=120, nint=1)]  # NE=40, Nch=2048, Ntaps=8
    bufs = [_inputs(mdt, cfg) for cfg in cases]
    torch.cuda.synchronize()
    # first call on this device: loads the module holding the static arrays
    _call(mdt, f, cases[0], *bufs[0])
    torch.cuda.synchronize()
    first = bufs[0][2].clone()
    free0, _ = torch.cuda.mem_get_info()
    # then two more calls in a row, the second shape and the first again
    for cfg, b in ((cases[1], bufs[1]), (cases[0], bufs[0])):
        b[2].fill_(float("nan"))
        _call(mdt, f, cfg, *b)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device memory changed across calls: %d -> %d" % (free0, free1)
    assert torch.equal(first.view(torch.int64), bufs[0][2].view(torch.int64)), \
        "repeated call on reused scratch differs"

    for cfg, (iq, win, vis) in zip(cases, bufs):
        ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
        plan = mdt.FxPlan(ne, nch, ntaps, nsp)
        plan.set_window(win)
        ref = torch.full_like(vis, float("nan"))
        plan.execute(iq, 1, ref)
        torch.cuda.synchronize()
        plan.close()
        v = vis.cpu().numpy()
        assert np.all(np.isfinite(v))
        assert np.array_equal(v.view(np.int64), ref.cpu().numpy().view(np.int64)), \
            "%s: static entry point differs from mdt_fx_execute" % cfg.name
        chans = np.array([0, 137 % nch, nch // 2, nch - 1], np.int32)
        o = oracle.fx(iq.cpu().numpy(), win.cpu().numpy(), ne, nch, ntaps, nsp, channels=chans)
        err = rel_fro(v[chans], o)
        assert err < TOL_FP32, "%s: %.3e vs FP64" % (cfg.name, err)


@pytest.mark.parametrize("shape,why", [
    ((256, 1024, 8, 1024), b"static scratch"),  # 2 GiB of F-output
    ((16, 4096, 4, 64), b"Nch must be <= 2048"),
    ((16, 1000, 4, 64), b"power of two"),
])
def test_integrate_static_rejects_unservable_shapes(mdt, cuda, shape, why):
    f = _entry(mdt)
    ne, nch, ntaps, nsp = shape
    iq = torch.zeros((nsp + ntaps - 1) * ne * nch * 2, dtype=torch.int8, device="cuda")
    win = torch.zeros(nch * ntaps, dtype=torch.float32, device="cuda")
    vis = torch.zeros(nch * ne * ne, dtype=torch.complex64, device="cuda")
    rc = f(ne, nch, ntaps, nsp, iq.data_ptr(), win.data_ptr(), vis.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    assert rc == MDT_ERR_INVALID_VALUE
    assert why in mdt.lib().mdt_last_error()
