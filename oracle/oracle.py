"""ctypes binding of the oracle (oracle/mdt_oracle.c).

TEST INFRASTRUCTURE ONLY. Results are checked against the oracle in tests/,
the smoke check in __graft_entry__ and the CPU-baseline leg of bench.py; the
product library never uses it.

build() compiles the C restatement into oracle/_build/libmdt_oracle.so with
gcc/cc (-O3 -fopenmp -ffp-contract=off; without -ffast-math no sum is
reassociated, so vectorisation does not change a result).  Every function takes numpy arrays and
returns numpy arrays; complex arrays are numpy complex64/complex128.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libmdt_oracle.so")
_SRC = [os.path.join(_HERE, "mdt_oracle.c"), os.path.join(_HERE, "mdt_oracle_core.h")]
_lib = None


def build(force=False):
    """Compile the oracle shared library (a few seconds)."""
    os.makedirs(_BUILD, exist_ok=True)
    if not force and os.path.exists(_LIB_PATH):
        newest = max(os.path.getmtime(p) for p in _SRC)
        if os.path.getmtime(_LIB_PATH) >= newest:
            return _LIB_PATH
    cc = os.environ.get("CC", "gcc")
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [cc, "-O3", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC", "-std=c11",
           _SRC[0], "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i, l, d, u64 = ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_uint64
        L.mdt_oracle_window_bh4.argtypes = [i, i, P]
        L.mdt_oracle_window_hamming_sinc.argtypes = [i, i, P]
        L.mdt_oracle_pps_f32_exact.argtypes = [i, i, i, i, P, P, P]
        L.mdt_oracle_reorder_c64.argtypes = [i, i, i, P, P]
        L.mdt_oracle_xengine_i8.argtypes = [i, i, i, P, P]
        L.mdt_oracle_synth_iq.argtypes = [u64, i, i, l, l, P, P, i, P, P, P]
        for suf in ("_f64", "_f32"):
            getattr(L, "mdt_oracle_fft_rows" + suf).argtypes = [l, i, P]
            getattr(L, "mdt_oracle_fft_rows" + suf).restype = i
            getattr(L, "mdt_oracle_fx" + suf).argtypes = [i, i, i, i, P, P, i, P, P]
            getattr(L, "mdt_oracle_fx" + suf).restype = i
        L.mdt_oracle_depacketise.argtypes = [i, i, i, i, P, i, l, P, i, i, i,
                                             ctypes.c_longlong, i, P, P]
        L.mdt_oracle_xengine_f64.argtypes = [i, i, i, P, d, P]
        L.mdt_oracle_xengine_f32.argtypes = [i, i, i, P, ctypes.c_float, P]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def window_bh4(nch, ntaps):
    """Blackman-Harris windowed sinc (float64), PFB_Window_min4term_BH."""
    w = np.empty(ntaps * nch, np.float64)
    lib().mdt_oracle_window_bh4(nch, ntaps, _p(w))
    return w


def window_hamming_sinc(nch, ntaps):
    """Hamming windowed sinc (float32), the benchmark configurations' window."""
    w = np.empty(ntaps * nch, np.float32)
    lib().mdt_oracle_window_hamming_sinc(nch, ntaps, _p(w))
    return w


def pps_f32_exact(win, insig, nch, ntaps, ne, nsp):
    """PpS_Batch in float with the reference's fmaf order (bit-exact)."""
    win = np.ascontiguousarray(win, np.float32)
    insig = np.ascontiguousarray(insig, np.complex64)
    assert insig.size == (nsp + ntaps - 1) * ne * nch
    out = np.empty(nsp * ne * nch, np.complex64)
    lib().mdt_oracle_pps_f32_exact(nch, ntaps, ne, nsp, _p(win), _p(insig), _p(out))
    return out


def reorder_c64(F, ne, nch, nsp):
    """ReorderFOutput index map (bit moves)."""
    F = np.ascontiguousarray(F, np.complex64)
    X = np.empty(nsp * ne * nch, np.complex64)
    lib().mdt_oracle_reorder_c64(ne, nch, nsp, _p(F), _p(X))
    return X


def fft_rows(data, n, double=True):
    """Batched unnormalised forward FFT over contiguous rows of n."""
    dt = np.complex128 if double else np.complex64
    x = np.array(data, dtype=dt, copy=True).reshape(-1)
    rows = x.size // n
    f = lib().mdt_oracle_fft_rows_f64 if double else lib().mdt_oracle_fft_rows_f32
    if f(rows, n, _p(x)) != 0:
        raise ValueError("n must be a power of two")
    return x


def fx(iq, win, ne, nch, ntaps, nsp, channels=None, double=True):
    """Full FX pipeline int8 I/Q -> visibilities (column-major per channel).

    iq: int8 array of (nsp+ntaps-1)*ne*nch*2 values; returns complex array
    [nsel, ne(q), ne(r)] where V[k, q, r] = (1/nsp) sum_s X[r] conj(X[q])."""
    iq = np.ascontiguousarray(iq, np.int8).reshape(-1)
    assert iq.size == (nsp + ntaps - 1) * ne * nch * 2
    win = np.ascontiguousarray(win, np.float32)
    dt = np.complex128 if double else np.complex64
    if channels is None:
        nsel, sel = nch, None
    else:
        sel = np.ascontiguousarray(channels, np.int32)
        nsel = sel.size
    V = np.empty((nsel, ne, ne), dt)
    f = lib().mdt_oracle_fx_f64 if double else lib().mdt_oracle_fx_f32
    rc = f(ne, nch, ntaps, nsp, _p(iq), _p(win), nsel, None if sel is None else _p(sel), _p(V))
    if rc != 0:
        raise ValueError("oracle fx failed: %d" % rc)
    return V


def xengine(X, ne, nch, nsp, alpha, double=True):
    """X-engine on the channel-major layout X[c][s][e]."""
    dt = np.complex128 if double else np.complex64
    X = np.ascontiguousarray(X, dt).reshape(-1)
    V = np.empty((nch, ne, ne), dt)
    if double:
        lib().mdt_oracle_xengine_f64(ne, nch, nsp, _p(X), float(alpha), _p(V))
    else:
        lib().mdt_oracle_xengine_f32(ne, nch, nsp, _p(X), ctypes.c_float(alpha), _p(V))
    return V


def xengine_i8(X, ne, nch, nsp):
    """Exact integer visibilities from int8 I/Q channel-major input; int64."""
    X = np.ascontiguousarray(X, np.int8).reshape(-1)
    assert X.size == nch * nsp * ne * 2
    V = np.empty((nch, ne, ne, 2), np.int64)
    lib().mdt_oracle_xengine_i8(ne, nch, nsp, _p(X), _p(V))
    return V


def synth_iq(seed, ne, nch, s0, nsp, sigma_q8, tone_q16=None, src_sigma_q8=None,
             src_delay=None):
    """Deterministic int8 I/Q samples, spectra s0..s0+nsp-1 (see mdt_oracle.c)."""
    sigma_q8 = np.ascontiguousarray(sigma_q8, np.int32)
    assert sigma_q8.size == ne
    tone = None if tone_q16 is None else np.ascontiguousarray(tone_q16, np.int32)
    if tone is not None:
        assert tone.size == ne * nch * 2
    nsrc = 0 if src_sigma_q8 is None else len(src_sigma_q8)
    ss = None if nsrc == 0 else np.ascontiguousarray(src_sigma_q8, np.int32)
    sd = None if nsrc == 0 else np.ascontiguousarray(src_delay, np.int32)
    out = np.empty(nsp * ne * nch * 2, np.int8)
    lib().mdt_oracle_synth_iq(ctypes.c_uint64(seed), ne, nch, s0, nsp, _p(sigma_q8),
                              None if tone is None else _p(tone), nsrc,
                              None if ss is None else _p(ss),
                              None if sd is None else _p(sd), _p(out))
    return out


def depacketise(fmt, pkts, npkt, ne, nch, sample0, nspectra, out=None):
    """Restated rank-1 depacketise loop (MDT_OneStation_client.cu:846-907)
    into a window; fmt is a dict with words_header, sper_element,
    inputs_per_station, inputs_per_snap (list), sample_bits, packet_bytes.
    Returns (out, [accepted, outside, bad]); out is complex64
    [nspectra][ne][nch] (32-bit samples) or int8 [nspectra][ne][nch][2],
    zero where no packet wrote (unless `out` is given)."""
    bits = fmt["sample_bits"]
    if out is None:
        out = (np.zeros((nspectra, ne, nch), np.complex64) if bits == 32
               else np.zeros((nspectra, ne, nch, 2), np.int8))
    ips = np.ascontiguousarray(fmt["inputs_per_snap"], np.int32)
    pk = np.ascontiguousarray(pkts).view(np.uint8)
    stats = np.zeros(3, np.int64)
    lib().mdt_oracle_depacketise(fmt["words_header"], fmt["sper_element"],
                                 fmt["inputs_per_station"], len(ips), _p(ips), bits,
                                 fmt["packet_bytes"], _p(pk), npkt, ne, nch, sample0, nspectra,
                                 _p(out), _p(stats))
    return out, stats.tolist()
