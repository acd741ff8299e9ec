"""End-to-end FX path on the GPU: the reference call sequence through the
drop-in API (PpS_Batch -> cufftExecC2C -> ReorderFOutput ->
cublasCgemmBatched, MDT_OneStation_client.cu:1083-1128) and the fused plan
API, against the FP64 oracle (<= 1e-5 relative visibility error, max over
channels of the Frobenius norm) and against each other (bit-exact)."""
import numpy as np
import pytest
import torch

from conftest import rel_fro

pytestmark = pytest.mark.gpu

TOL_FP32 = 1e-5  # FP32 path vs FP64 oracle


def cdiv(a, b):
    return (a + b - 1) // b


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gen_iq(mdt, cfg, s0, nsp):
    """int8 I/Q on the GPU from the configuration's generator."""
    out = torch.empty(nsp * cfg.nelements * cfg.nchannels * 2, dtype=torch.int8, device="cuda")
    tone = cfg.tone_q16()
    ssig, sdel = cfg.sources()
    mdt.synth_iq(cfg.seed, cfg.nelements, cfg.nchannels, s0, nsp, dev(cfg.sigma_q8()), out,
                 tone_q16=None if tone is None else dev(tone),
                 src_sigma_q8=None if ssig is None else dev(ssig),
                 src_delay=None if sdel is None else dev(sdel))
    return out


def window(mdt, nch, ntaps):
    w = torch.empty(nch * ntaps, dtype=torch.float32, device="cuda")
    mdt.window_hamming_sinc(nch, ntaps, w)
    return w


def to_c64(iq):
    return torch.view_as_complex(iq.view(-1, 2).float().contiguous())


def ptr_array(base, stride_elems, count):
    return torch.tensor([base.data_ptr() + i * stride_elems * 8 for i in range(count)],
                        dtype=torch.int64, device=base.device)


def dropin_chain(mdt, iq, win, ne, nch, ntaps, nsp):
    """The reference client's rank-2 sequence, launched with its geometry."""
    fin = to_c64(iq)
    fout = torch.empty(nsp * ne * nch, dtype=torch.complex64, device="cuda")
    mdt.PpS_Batch((cdiv(nch, 1024), nsp, ne), (1024,), nch, ntaps, win, fin, fout)
    plan = mdt.cufftPlan1d(nch, mdt.CUFFT_C2C, nsp * ne)
    mdt.cufftSetStream(plan, torch.cuda.current_stream())
    mdt.cufftExecC2C(plan, fout, fout, mdt.CUFFT_FORWARD)
    xin = torch.empty_like(fout)
    mdt.ReorderFOutput((cdiv(ne, 32), cdiv(nch, 32), nsp), (32, 32), ne, nch, fout, xin)
    vis = torch.empty(nch * ne * ne, dtype=torch.complex64, device="cuda")
    h = mdt.cublasCreate()
    mdt.cublasSetStream(h, torch.cuda.current_stream())
    A = ptr_array(xin, ne * nsp, nch)
    C = ptr_array(vis, ne * ne, nch)
    mdt.cublasCgemmBatched(h, mdt.CUBLAS_OP_N, mdt.CUBLAS_OP_C, ne, ne, nsp, 1.0 / nsp, A, ne, A,
                           ne, 0.0, C, ne, nch)
    torch.cuda.synchronize()
    mdt.cublasDestroy(h)
    mdt.cufftDestroy(plan)
    return xin, vis.view(nch, ne, ne)


def test_synth_gpu_matches_oracle(mdt, cuda, oracle):
    for cfg in (mdt.configs.small(mdt.configs.C1, nspectra=4),
                mdt.configs.small(mdt.configs.C3, nelements=16, nchannels=64, nspectra=3)):
        g = gen_iq(mdt, cfg, 7, 5).cpu().numpy()
        ssig, sdel = cfg.sources()
        c = oracle.synth_iq(cfg.seed, cfg.nelements, cfg.nchannels, 7, 5, cfg.sigma_q8(),
                            cfg.tone_q16(), ssig, sdel)
        assert np.array_equal(g, c), cfg.name


def test_c1_dropin_sequence_vs_oracle(mdt, cuda, oracle):
    cfg = mdt.configs.C1  # full size: NE=10, Nch=1024, Ntaps=4, Nsp=1000
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    iq = gen_iq(mdt, cfg, 0, nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    _, vis = dropin_chain(mdt, iq, win, ne, nch, ntaps, nsp)
    ref = oracle.fx(iq.cpu().numpy(), win.cpu().numpy(), ne, nch, ntaps, nsp)
    err = rel_fro(vis.cpu().numpy(), ref)
    print("c1 drop-in rel err %.3e" % err)
    assert err < TOL_FP32
    # the tone at channel 137 dominates the cross-power there
    v = vis.cpu().numpy()
    off = np.abs(v[:, 0, 1])
    assert int(np.argmax(off)) == 137


def test_fused_fengine_bit_identical_to_dropin_chain(mdt, cuda):
    for cfg in (mdt.configs.C1, mdt.configs.small(mdt.configs.C2, nspectra=64, nint=1),
                mdt.configs.small(mdt.configs.C1, nelements=3, nchannels=32, nspectra=2)):
        ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
        iq = gen_iq(mdt, cfg, 0, nsp + ntaps - 1)
        win = window(mdt, nch, ntaps)
        xin, vis = dropin_chain(mdt, iq, win, ne, nch, ntaps, nsp)
        X = torch.full_like(xin, float("nan"))
        mdt.fengine_f32(ne, nch, ntaps, nsp, iq, win, X)
        torch.cuda.synchronize()
        assert torch.equal(X.view(torch.int64), xin.view(torch.int64)), cfg.name
        plan = mdt.FxPlan(ne, nch, ntaps, nsp)
        plan.set_window(win)
        v2 = torch.full_like(vis, float("nan"))
        plan.execute(iq, 1, v2)
        torch.cuda.synchronize()
        assert torch.equal(v2.view(torch.int64), vis.view(torch.int64)), cfg.name
        plan.close()


@pytest.mark.parametrize("ne,nch,ntaps,nsp,nint", [(8, 256, 8, 64, 4), (3, 32, 8, 2, 5),
                                                   (5, 64, 4, 3, 3), (4, 1024, 8, 40, 3),
                                                   (3, 2048, 4, 17, 2)])
def test_streaming_history_vs_oracle(mdt, cuda, oracle, ne, nch, ntaps, nsp, nint):
    cfg = mdt.configs.small(mdt.configs.C2, nelements=ne, nchannels=nch, ntaps=ntaps,
                            nspectra=nsp, nint=nint)
    total = nint * nsp + ntaps - 1
    iq = gen_iq(mdt, cfg, 0, total)
    win = window(mdt, nch, ntaps)
    sb = ne * nch * 2
    plan = mdt.FxPlan(ne, nch, ntaps, nsp)
    plan.set_window(win)
    vis_one = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(iq, nint, vis_one)
    plan.stream_reset()
    vis_stream = torch.empty_like(vis_one)
    # first push carries the lead-in; later pushes only new spectra, from
    # separate buffers so the history must come from the plan
    plan.stream_push(iq[:(nsp + ntaps - 1) * sb].clone(), vis_stream[0])
    for j in range(1, nint):
        lo = (j * nsp + ntaps - 1) * sb
        plan.stream_push(iq[lo:lo + nsp * sb].clone(), vis_stream[j])
    torch.cuda.synchronize()
    assert torch.equal(vis_stream.view(torch.int64), vis_one.view(torch.int64))
    iqh, winh = iq.cpu().numpy(), win.cpu().numpy()
    for j in range(nint):
        seg = iqh[j * nsp * sb:(j * nsp + nsp + ntaps - 1) * sb]
        ref = oracle.fx(seg, winh, ne, nch, ntaps, nsp)
        assert rel_fro(vis_stream[j].cpu().numpy(), ref) < TOL_FP32
    plan.close()


@pytest.mark.parametrize("ne,nch,ntaps,nsp,nint", [(6, 1024, 8, 48, 5), (3, 64, 4, 5, 1)])
def test_execute_host_matches_device_run(mdt, cuda, ne, nch, ntaps, nsp, nint):
    """The host-buffer pipeline (input copies, compute and visibility copies on
    three streams, staging buffers reused from the third integration on)
    returns the device run's visibilities bit for bit, also when called twice."""
    cfg = mdt.configs.small(mdt.configs.C2, nelements=ne, nchannels=nch, ntaps=ntaps,
                            nspectra=nsp, nint=nint)
    total = nint * nsp + ntaps - 1
    iq = gen_iq(mdt, cfg, 0, total)
    win = window(mdt, nch, ntaps)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp)
    plan.set_window(win)
    vis_dev = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(iq, nint, vis_dev)
    torch.cuda.synchronize()
    h_iq = iq.cpu().pin_memory()
    for _ in range(2):
        h_vis = torch.full((nint, nch, ne, ne), float("nan"), dtype=torch.complex64).pin_memory()
        plan.execute_host(h_iq, nint, h_vis)
        assert torch.equal(h_vis.view(torch.int64), vis_dev.cpu().view(torch.int64))
    plan.close()


def test_c2_full_size_channel_subset_vs_oracle(mdt, cuda, oracle):
    cfg = mdt.configs.C2  # NE=40, Nch=2048, Ntaps=8, Nsp=4096 (one integration)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    iq = gen_iq(mdt, cfg, 0, nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp)
    plan.set_window(win)
    vis = torch.empty(nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(iq, 1, vis)
    torch.cuda.synchronize()
    sel = [0, 1, 137, 1023, 1024, 2047] + [c for c, _ in cfg.tone_channels()]
    ref = oracle.fx(iq.cpu().numpy(), win.cpu().numpy(), ne, nch, ntaps, nsp, channels=sel)
    err = rel_fro(vis.cpu().numpy()[sel], ref)
    print("c2 full-size rel err %.3e" % err)
    assert err < TOL_FP32
    # size-independent property over all channels: Hermitian, real positive autos
    v = vis.cpu().numpy()
    assert np.array_equal(v, np.conj(np.transpose(v, (0, 2, 1))))
    d = np.diagonal(v, axis1=1, axis2=2)
    assert np.all(d.imag == 0) and np.all(d.real > 0)
    plan.close()


def test_parseval_checksum_full_c2_stream(mdt, cuda):
    """Size-independent check at the full 16-integration stream: for every
    element, sum_c V_c[e,e] = Nch/Nsp * sum_s sum_c |P[s,e,c]|^2 (Parseval),
    with P the drop-in PpS_Batch output evaluated in FP64 by torch."""
    cfg = mdt.configs.C2
    ne, nch, ntaps, nsp, nint = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra, 4
    win = window(mdt, nch, ntaps)
    iq = gen_iq(mdt, cfg, 0, nint * nsp + ntaps - 1)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp)
    plan.set_window(win)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device="cuda")
    plan.execute(iq, nint, vis)
    sb = ne * nch * 2
    for j in (0, nint - 1):
        seg = iq[j * nsp * sb:(j * nsp + nsp + ntaps - 1) * sb]
        fout = torch.empty(nsp * ne * nch, dtype=torch.complex64, device="cuda")
        mdt.PpS_Batch((cdiv(nch, 1024), nsp, ne), (1024,), nch, ntaps, win, to_c64(seg), fout)
        p = fout.view(nsp, ne, nch).to(torch.complex128)
        power = (p.abs() ** 2).sum(dim=(0, 2)) * nch / nsp
        auto = torch.diagonal(vis[j].to(torch.complex128), dim1=1, dim2=2).real.sum(dim=0)
        rel = ((auto - power).abs() / power).max().item()
        assert rel < 1e-5, rel
    plan.close()


def test_plan_errors(mdt, cuda):
    with pytest.raises(mdt.MdtError):
        mdt.FxPlan(2, 1024, 4, 100)  # NE below the reference minimum
    with pytest.raises(mdt.MdtError):
        mdt.FxPlan(10, 1000, 4, 100)  # Nch not a power of two
    with pytest.raises(mdt.MdtError):
        mdt.FxPlan(10, 1024, 200, 100)  # Ntaps above the maximum
    plan = mdt.FxPlan(4, 64, 4, 8)
    iq = torch.zeros((8 + 3) * 4 * 64 * 2, dtype=torch.int8, device="cuda")
    vis = torch.empty(64 * 16, dtype=torch.complex64, device="cuda")
    with pytest.raises(mdt.MdtError) as e:
        plan.execute(iq, 1, vis)  # no window yet
    assert e.value.code == 6
    plan.close()


@pytest.mark.parametrize("ne,nch,ntaps,nsp", [(40, 2048, 8, 100), (10, 1024, 4, 64), (5, 256, 6, 9),
                                              (3, 32, 4, 2)])
def test_blocked_fengine_matches_reference_layout(mdt, cuda, ne, nch, ntaps, nsp):
    """The spectrum-block F-engine (8-spectrum blocked layout) gives the same
    bits as the element-row F-engine (ReorderFOutput layout), for the
    compile-time tap counts and the runtime-loop fallback (ntaps=6)."""
    cfg = mdt.configs.small(mdt.configs.C2, nelements=ne, nchannels=nch, ntaps=ntaps,
                            nspectra=nsp)
    iq = gen_iq(mdt, cfg, 0, nsp + ntaps - 1)
    win = window(mdt, nch, ntaps)
    X = torch.empty(nsp * ne * nch, dtype=torch.complex64, device="cuda")
    mdt.fengine_f32(ne, nch, ntaps, nsp, iq, win, X)
    nsb = (nsp + 7) // 8
    XB = torch.full((nch * nsb * ne * 8,), float("nan"), dtype=torch.complex64, device="cuda")
    mdt.fengine_c64b(ne, nch, ntaps, nsp, iq, win, XB)
    torch.cuda.synchronize()
    xb = XB.view(nsb, nch, ne, 8).permute(1, 0, 3, 2).reshape(nch, nsb * 8, ne)
    assert torch.all(xb[:, nsp:, :] == 0)
    ref = X.view(nch, nsp, ne)
    assert torch.equal(xb[:, :nsp, :].contiguous().view(torch.int64), ref.view(torch.int64))
