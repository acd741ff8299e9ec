"""The reference client's GPU stage, written against the drop-in header only
(tests/client_stage/client_stage.cu), compiled with nvcc and linked against
libmdtfx.so alone: the link check runs without a GPU, the run on the GPU is
compared with the FP64 oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_pkg, rel_fro

SRC = os.path.join(ROOT, "tests", "client_stage", "client_stage.cu")


def build_client(out_dir):
    mdt = load_pkg()
    mdt.build()
    libdir = os.path.dirname(mdt.LIB_PATH)
    exe = os.path.join(str(out_dir), "client_stage")
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-cudart", "shared", "-I",
           os.path.join(ROOT, "include"), "-o", exe, SRC, "-L", libdir, "-lmdtfx", "-Xlinker",
           "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_client_stage_links_without_cufft_cublas(tmp_path):
    exe = build_client(tmp_path)
    deps = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "libmdtfx.so" in deps
    assert "cufft" not in deps and "cublas" not in deps
    undefined = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    for sym in ("cufftExecC2C", "cublasCgemmBatched", "_Z9PpS_BatchiiPfP6float2S1_",
                "_Z14ReorderFOutputiiP6float2S0_"):
        assert sym in undefined, sym


@pytest.mark.gpu
def test_client_stage_runs_and_matches_oracle(tmp_path, oracle):
    exe = build_client(tmp_path)
    mdt = load_pkg()
    cfg = mdt.configs.small(mdt.configs.C1, nelements=12, nchannels=256, nspectra=200)
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    iq = oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(), cfg.tone_q16())
    win = oracle.window_hamming_sinc(nch, ntaps)
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(iq.tobytes())
        f.write(win.tobytes())
    r = subprocess.run([exe, str(ne), str(nch), str(ntaps), str(nsp), str(inp), str(outp)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    vis = np.fromfile(outp, np.complex64).reshape(nch, ne, ne)
    ref = oracle.fx(iq, win, ne, nch, ntaps, nsp)
    assert rel_fro(vis, ref) < 1e-5
