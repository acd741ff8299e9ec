"""Generate the committed golden fixtures in tests/golden/ from the reference's
own kernel code.

The reference ships no tests, fixtures or known-answer vectors. Its kernels
(PFB_Window_min4term_BH, PpS_Batch, ReorderFOutput in
MDT_OneStation_client/MDT_device_functions.cu) are compiled for the CPU by
oracle/build_ref.sh and run here, block by block, with the launch geometry
the reference documents (MDT_device_functions.cu:44-49, 105-110, 175-180;
ReorderFOutput always with block (32,32), the geometry under which the
reference kernel is correct). The outputs are stored with their seeded
inputs in ref_kernels.npz.

Run in the build container (needs the reference checkout):
    python tests/golden/make_golden.py
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle  # noqa: E402

REF_SO = os.path.join(ROOT, "oracle", "_ref", "libmdt_ref_emu.so")


def ref_lib():
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    L = ctypes.CDLL(REF_SO)
    u, i, P = ctypes.c_uint, ctypes.c_int, ctypes.c_void_p
    L.ref_PFB_Window_min4term_BH.argtypes = [u, u, i, i, P]
    L.ref_PpS_Batch.argtypes = [u, u, u, u, i, i, P, P, P]
    L.ref_ReorderFOutput.argtypes = [u, u, u, u, u, i, i, P, P]
    for f in (L.ref_PFB_Window_min4term_BH, L.ref_PpS_Batch, L.ref_ReorderFOutput):
        f.restype = i
    return L


def p(a):
    return ctypes.c_void_p(a.ctypes.data)


def cdiv(a, b):
    return (a + b - 1) // b


def main():
    L = ref_lib()
    rng = np.random.default_rng(20210301)
    out = {}
    # (nch, ntaps, ne, nsp, block_x): reference minima (MDT_host_functions.h:39-46),
    # a 40-element station row, and a non-multiple-of-32 element count.
    pps_cases = [(32, 4, 3, 2, 1024), (64, 8, 40, 3, 1024), (128, 4, 10, 5, 64),
                 (96, 5, 7, 3, 32)]
    for k, (nch, ntaps, ne, nsp, bx) in enumerate(pps_cases):
        if k % 2 == 0:
            # int8-valued samples (the synthetic inputs' value set)
            iq = rng.integers(-127, 128, size=(nsp + ntaps - 1) * ne * nch * 2).astype(np.float32)
        else:
            # wide dynamic range to exercise fmaf rounding
            iq = (rng.standard_normal((nsp + ntaps - 1) * ne * nch * 2) *
                  np.exp2(rng.integers(-20, 20, size=(nsp + ntaps - 1) * ne * nch * 2))
                  ).astype(np.float32)
        insig = iq.view(np.complex64).copy()
        win = oracle.window_hamming_sinc(nch, ntaps) if k % 2 == 0 else \
            rng.standard_normal(ntaps * nch).astype(np.float32)
        res = np.zeros(nsp * ne * nch, np.complex64)
        rc = L.ref_PpS_Batch(cdiv(nch, bx), nsp, ne, bx, nch, ntaps, p(win), p(insig), p(res))
        assert rc == 0
        out["pps%d_shape" % k] = np.array([nch, ntaps, ne, nsp, bx], np.int64)
        out["pps%d_win" % k] = win
        out["pps%d_in" % k] = insig
        out["pps%d_out" % k] = res

    reorder_cases = [(3, 32, 2), (40, 64, 3), (10, 96, 4), (33, 40, 2)]
    for k, (ne, nch, nsp) in enumerate(reorder_cases):
        F = (rng.standard_normal(nsp * ne * nch * 2)).astype(np.float32).view(np.complex64)
        X = np.full(nsp * ne * nch, np.nan + 1j * np.nan, np.complex64)
        rc = L.ref_ReorderFOutput(cdiv(ne, 32), cdiv(nch, 32), nsp, 32, 32, ne, nch, p(F), p(X))
        assert rc == 0
        out["reorder%d_shape" % k] = np.array([ne, nch, nsp], np.int64)
        out["reorder%d_in" % k] = F
        out["reorder%d_out" % k] = X

    for k, (nch, ntaps) in enumerate([(32, 4), (64, 8), (1024, 4)]):
        w = np.zeros(nch * ntaps, np.float32)
        rc = L.ref_PFB_Window_min4term_BH(cdiv(nch * ntaps, 256), 256, nch, ntaps, p(w))
        assert rc == 0
        out["window%d_shape" % k] = np.array([nch, ntaps], np.int64)
        out["window%d_out" % k] = w

    path = os.path.join(HERE, "ref_kernels.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
