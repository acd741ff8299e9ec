"""ctypes binding of libmdtfx.so (declarations: include/mdt_fx.h,
include/MDT_device_functions.h, include/mdt_cufft_cublas_shim.h).

Every function raises MdtError on a non-success status; the cuFFT / cuBLAS
subset raises with the library status code in MdtError.code, the way the
reference client treats any non-success code as fatal
(MDT_OneStation_client.cu:622-627,1130-1135).
"""
import ctypes
import os

from . import _build

LIB_PATH = _build.LIB

CUFFT_FORWARD = -1
CUFFT_INVERSE = 1
CUFFT_C2C = 0x29
CUBLAS_OP_N, CUBLAS_OP_T, CUBLAS_OP_C = 0, 1, 2
MDT_PREC_FP32, MDT_PREC_FP16, MDT_PREC_BF16, MDT_PREC_INT8 = 0, 1, 2, 3

_P = ctypes.c_void_p
_I = ctypes.c_int
_U = ctypes.c_uint
_L = ctypes.c_long
_F = ctypes.c_float

_lib = None


class MdtError(RuntimeError):
    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


class _CuComplex(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


def build(force=False, verbose=False):
    """Compile libmdtfx.so in-tree for sm_103a (nvcc)."""
    return _build.build(force=force, verbose=verbose)


def _declare(L):
    grid6 = [_U] * 6
    sig = {
        "mdt_version": ([], _I),
        "mdt_last_error": ([], ctypes.c_char_p),
        "mdt_launch_PFB_Window_min4term_BH": (grid6 + [_P, _I, _I, _P], _I),
        "mdt_launch_PpS_Batch": (grid6 + [_P, _I, _I, _P, _P, _P], _I),
        "mdt_launch_ReorderFOutput": (grid6 + [_P, _I, _I, _P, _P], _I),
        "mdt_window_hamming_sinc": ([_I, _I, _P, _P], _I),
        "mdt_fft_c2c": ([_P, _P, _L, _I, _I, _P], _I),
        "mdt_xengine_f32": ([_I, _I, _I, _P, _L, _L, _F, _P, _P], _I),
        "mdt_fengine_f32": ([_I, _I, _I, _I, _P, _P, _P, _P], _I),
        "mdt_fengine_x16": ([_I, _I, _I, _I, _P, _P, _P, _I, _F, _P], _I),
        "mdt_fengine_c64b": ([_I, _I, _I, _I, _P, _P, _P, _P], _I),
        "mdt_xengine_tc": ([_I, _I, _I, _P, _I, _F, _P, _P, _P, _P], _I),
        "mdt_synth_iq": ([ctypes.c_uint64, _I, _I, _L, _L, _P, _P, _I, _P, _P, _P, _P], _I),
        "mdt_fx_create": ([_P, ctypes.POINTER(_P)], _I),
        "mdt_fx_destroy": ([_P], _I),
        "mdt_fx_set_stream": ([_P, _P], _I),
        "mdt_fx_set_window": ([_P, _P], _I),
        "mdt_fx_workspace_bytes": ([_P, ctypes.POINTER(ctypes.c_size_t)], _I),
        "mdt_fx_execute": ([_P, _P, _I, _P], _I),
        "mdt_fx_stream_reset": ([_P], _I),
        "mdt_fx_stream_push": ([_P, _P, _P], _I),
        "mdt_fx_execute_host": ([_P, _P, _I, _P], _I),
        "mdt_fx_set_accumulator": ([_P, _P], _I),
        "mdt_fx_set_channel_scales": ([_P, _P], _I),
        "mdt_fx_get_channel_scales": ([_P, _P], _I),
        "mdt_fengine_tc": ([_I, _I, _I, _I, _P, _P, _P, _I, _F, _P, _P], _I),
        "mdt_fengine_tc_q8": ([_I, _I, _I, _I, _P, _P, _P, _P, _P, _P], _I),
        "mdt_fengine_q8": ([_I, _I, _I, _I, _P, _P, _P, _P, _P], _I),
        "mdt_tc_peak_f16": ([_I, _I, _I, _I, ctypes.POINTER(ctypes.c_float),
                             ctypes.POINTER(ctypes.c_double), _P, _P], _I),
        "mdt_fp32_peak": ([_I, _I, _I, ctypes.POINTER(ctypes.c_float),
                           ctypes.POINTER(ctypes.c_double), _P], _I),
        "mdt_xengine_q8": ([_I, _I, _I, _P, _P, _P, _P, _P, _P, _P], _I),
        "mdt_fx_integrate_static": ([_I, _I, _I, _I, _P, _P, _P, _P], _I),
        "mdt_fx_get_scale": ([_P, ctypes.POINTER(ctypes.c_float)], _I),
        "mdt_fx_check": ([_P], _I),
        "mdt_fx_set_timing": ([_P, _I], _I),
        "mdt_fx_get_timing": ([_P, ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I)], _I),
        "mdt_fx_batch_create": ([_P, _I, ctypes.POINTER(_P)], _I),
        "mdt_fx_batch_destroy": ([_P], _I),
        "mdt_fx_batch_set_window": ([_P, _I, _P], _I),
        "mdt_fx_batch_get_stream": ([_P, ctypes.POINTER(_P)], _I),
        "mdt_fx_batch_autotune": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
        "mdt_fx_batch_execute": ([_P, _P, _P, _I], _I),
        "mdt_fx_batch_check": ([_P], _I),
        "mdt_depacketise_seen_words": ([_P, _I, _I, ctypes.c_longlong, _I,
                                        ctypes.POINTER(ctypes.c_size_t)], _I),
        "mdt_depacketise": ([_P, _P, _I, _I, _I, ctypes.c_longlong, _I, _P, _P, _P, _P], _I),
        "mdt_depacketise_finish": ([_P, _I, _I, ctypes.c_longlong, _I, _P, _P, _P, _P], _I),
        "mdt_num_baselines": ([_I, _I, ctypes.POINTER(_L)], _I),
        "mdt_format_baselines": ([_I, _I, _I, _P, _P, _I, _P], _I),
        "mdt_write_csv": ([ctypes.c_char_p, _I, _I, _I, _P, _I, _I], _I),
        "mdt_write_binary": ([ctypes.c_char_p, _I, _I, _I, _P, _I], _I),
        "mdt_ingest_create": ([_P, _P, _I, _I, ctypes.POINTER(_P)], _I),
        "mdt_ingest_destroy": ([_P], _I),
        "mdt_ingest_set_window": ([_P, _P], _I),
        "mdt_ingest_push": ([_P, _P, _I], _I),
        "mdt_ingest_flush": ([_P], _I),
        "mdt_ingest_pop": ([_P, _P, ctypes.POINTER(ctypes.c_longlong), _P, _I], _I),
        "mdt_ingest_counters": ([_P, ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.c_size_t)], _I),
        "mdt_apply_gains": ([_I, _I, _I, _P, _P, _P, _P], _I),
        "mdt_xengine_adjoint_f32": ([_I, _I, _I, _P, _P, _P, _F, _P], _I),
        "mdt_gain_adjoint": ([_I, _I, _I, _P, _P, _P, _P, _P, _P], _I),
        "mdt_pfb_tap_grad": ([_I, _I, _I, _I, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
        "cufftPlan1d": ([ctypes.POINTER(_I), _I, _I, _I], _I),
        "cufftSetStream": ([_I, _P], _I),
        "cufftExecC2C": ([_I, _P, _P, _I], _I),
        "cufftDestroy": ([_I], _I),
        "cufftGetVersion": ([ctypes.POINTER(_I)], _I),
        "cublasCreate_v2": ([ctypes.POINTER(_P)], _I),
        "cublasDestroy_v2": ([_P], _I),
        "cublasSetStream_v2": ([_P, _P], _I),
        "cublasGetStream_v2": ([_P, ctypes.POINTER(_P)], _I),
        "cublasCgemmBatched": ([_P, _I, _I, _I, _I, _I, ctypes.POINTER(_CuComplex), _P, _I, _P,
                                _I, ctypes.POINTER(_CuComplex), _P, _I, _I], _I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res


def lib():
    """The loaded libmdtfx.so; builds it first if it is missing or stale."""
    global _lib
    if _lib is None:
        if not _build.up_to_date():
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise MdtError("libmdtfx.so is missing and could not be built")
        L = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
        _declare(L)
        _lib = L
    return _lib


def check(status, what):
    if status != 0:
        msg = lib().mdt_last_error().decode(errors="replace")
        raise MdtError("%s failed (mdt_status %d): %s" % (what, status, msg), status)


def ptr(x):
    """Device address of a torch tensor / integer / None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if hasattr(x, "is_cuda") and not x.is_cuda:
            raise MdtError("expected a CUDA tensor")
        return x.data_ptr()
    raise TypeError("cannot take a device address of %r" % type(x))


def _host_ptr(x):
    if hasattr(x, "ctypes"):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return int(x)


def stream_handle(stream=None):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _g6(grid, block):
    g = tuple(grid) + (1,) * (3 - len(grid))
    b = tuple(block) + (1,) * (3 - len(block))
    return list(g) + list(b)


# ----------------------------------------------------------- drop-in kernels
def PFB_Window_min4term_BH(grid, block, Nchannels, Ntaps, Window, stream=None):
    check(lib().mdt_launch_PFB_Window_min4term_BH(*_g6(grid, block), stream_handle(stream),
                                                  Nchannels, Ntaps, ptr(Window)),
          "PFB_Window_min4term_BH")


def PpS_Batch(grid, block, Nchannels, Ntaps, Window, InSignal, PolyStruct, stream=None):
    check(lib().mdt_launch_PpS_Batch(*_g6(grid, block), stream_handle(stream), Nchannels, Ntaps,
                                     ptr(Window), ptr(InSignal), ptr(PolyStruct)), "PpS_Batch")


def ReorderFOutput(grid, block, NpolsxNelements, Nchannels, FOutput, XInput, stream=None):
    check(lib().mdt_launch_ReorderFOutput(*_g6(grid, block), stream_handle(stream),
                                          NpolsxNelements, Nchannels, ptr(FOutput), ptr(XInput)),
          "ReorderFOutput")


# ----------------------------------------------------------- cuFFT subset
def _cufft(rc, what):
    if rc != 0:
        raise MdtError("%s returned cufftResult %d" % (what, rc), rc)


def cufftPlan1d(nx, fft_type, batch):
    h = _I(0)
    _cufft(lib().cufftPlan1d(ctypes.byref(h), nx, fft_type, batch), "cufftPlan1d")
    return h.value


def cufftSetStream(plan, stream):
    _cufft(lib().cufftSetStream(plan, stream_handle(stream)), "cufftSetStream")


def cufftExecC2C(plan, idata, odata, direction):
    _cufft(lib().cufftExecC2C(plan, ptr(idata), ptr(odata), direction), "cufftExecC2C")


def cufftDestroy(plan):
    _cufft(lib().cufftDestroy(plan), "cufftDestroy")


def cufftGetVersion():
    v = _I(0)
    _cufft(lib().cufftGetVersion(ctypes.byref(v)), "cufftGetVersion")
    return v.value


# ----------------------------------------------------------- cuBLAS subset
def _cublas(rc, what):
    if rc != 0:
        raise MdtError("%s returned cublasStatus %d" % (what, rc), rc)


def cublasCreate():
    h = _P()
    _cublas(lib().cublasCreate_v2(ctypes.byref(h)), "cublasCreate")
    return h.value


def cublasSetStream(handle, stream):
    _cublas(lib().cublasSetStream_v2(handle, stream_handle(stream)), "cublasSetStream")


def cublasDestroy(handle):
    _cublas(lib().cublasDestroy_v2(handle), "cublasDestroy")


def cublasCgemmBatched(handle, transa, transb, m, n, k, alpha, Aarray, lda, Barray, ldb, beta,
                       Carray, ldc, batchCount):
    """Aarray/Barray/Carray: device arrays of device pointers (e.g. int64 CUDA
    tensors); alpha/beta: Python complex numbers (host pointer mode)."""
    a = _CuComplex(complex(alpha).real, complex(alpha).imag)
    b = _CuComplex(complex(beta).real, complex(beta).imag)
    _cublas(lib().cublasCgemmBatched(handle, transa, transb, m, n, k, ctypes.byref(a),
                                     ptr(Aarray), lda, ptr(Barray), ldb, ctypes.byref(b),
                                     ptr(Carray), ldc, batchCount), "cublasCgemmBatched")


# ----------------------------------------------------------- stage entry points
def window_hamming_sinc(nchannels, ntaps, window, stream=None):
    check(lib().mdt_window_hamming_sinc(nchannels, ntaps, ptr(window), stream_handle(stream)),
          "window_hamming_sinc")


def fft_c2c(inp, out, rows, n, direction=CUFFT_FORWARD, stream=None):
    check(lib().mdt_fft_c2c(ptr(inp), ptr(out), rows, n, direction, stream_handle(stream)),
          "fft_c2c")


def xengine_f32(ne, nch, nsp, X, ld, xstride, alpha, V, stream=None):
    check(lib().mdt_xengine_f32(ne, nch, nsp, ptr(X), ld, xstride, alpha, ptr(V),
                                stream_handle(stream)), "xengine_f32")


def fengine_f32(ne, nch, ntaps, nsp, iq, window, X, stream=None):
    check(lib().mdt_fengine_f32(ne, nch, ntaps, nsp, ptr(iq), ptr(window), ptr(X),
                                stream_handle(stream)), "fengine_f32")


def fengine_c64b(ne, nch, ntaps, nsp, iq, window, XB, stream=None):
    """FP32 F-engine into XB[s/8][c][e][s%8] complex64 (ceil(nsp/8) blocks of 8
    spectra, spectra past nsp zero), bit-identical to fengine_f32."""
    check(lib().mdt_fengine_c64b(ne, nch, ntaps, nsp, ptr(iq), ptr(window), ptr(XB),
                                 stream_handle(stream)), "fengine_c64b")


def fengine_x16(ne, nch, ntaps, nsp, iq, window, X16, ab_fmt=0, scale=1.0, stream=None):
    check(lib().mdt_fengine_x16(ne, nch, ntaps, nsp, ptr(iq), ptr(window), ptr(X16), ab_fmt,
                                scale, stream_handle(stream)), "fengine_x16")


def xengine_tc(ne, nch, nsp, X16, vis, vis_acc=None, err=None, ab_fmt=0, scale=1.0,
               stream=None):
    check(lib().mdt_xengine_tc(ne, nch, nsp, ptr(X16), ab_fmt, scale, ptr(vis), ptr(vis_acc),
                               ptr(err), stream_handle(stream)), "xengine_tc")


def fengine_tc(ne, nch, ntaps, nsp, iq, window, X16, err, ab_fmt=0, scale=1.0, stream=None):
    """Tensor-core F-engine (Nch 1024): same output layout as fengine_x16."""
    check(lib().mdt_fengine_tc(ne, nch, ntaps, nsp, ptr(iq), ptr(window), ptr(X16), ab_fmt, scale,
                               ptr(err), stream_handle(stream)), "fengine_tc")


def fp32_peak(packed=True, iters=100000, reps=5, stream=None):
    """Measured FP32 FMA throughput (best of `reps` launches): (ms, TFLOP/s)."""
    ms = ctypes.c_float(0.0)
    tf = ctypes.c_double(0.0)
    check(lib().mdt_fp32_peak(1 if packed else 0, iters, reps, ctypes.byref(ms), ctypes.byref(tf),
                              stream_handle(stream)), "fp32_peak")
    return ms.value, tf.value


def tc_peak_f16(n=256, ctas_per_sm=1, iters=20000, reps=5, err=None, stream=None):
    """Measured kind::f16 tcgen05.mma throughput (best of `reps` launches):
    (ms, TFLOP/s).  `err` is a device int32 tensor (a wait timeout sets it)."""
    ms = ctypes.c_float(0.0)
    tf = ctypes.c_double(0.0)
    check(lib().mdt_tc_peak_f16(n, ctas_per_sm, iters, reps, ctypes.byref(ms), ctypes.byref(tf),
                                ptr(err), stream_handle(stream)), "tc_peak_f16")
    return ms.value, tf.value


def fengine_tc_q8(ne, nch, ntaps, nsp, iq, window, X16, qscales, err, stream=None):
    """Tensor-core F-engine with int8 requantisation (Nch 1024)."""
    check(lib().mdt_fengine_tc_q8(ne, nch, ntaps, nsp, ptr(iq), ptr(window), ptr(X16),
                                  ptr(qscales), ptr(err), stream_handle(stream)), "fengine_tc_q8")


def fengine_q8(ne, nch, ntaps, nsp, iq, window, X16, qscales, stream=None):
    check(lib().mdt_fengine_q8(ne, nch, ntaps, nsp, ptr(iq), ptr(window), ptr(X16), ptr(qscales),
                               stream_handle(stream)), "fengine_q8")


def xengine_q8(ne, nch, nsp, X16, qscales, vis=None, vis_acc=None, vis_i32=None, err=None,
               stream=None):
    check(lib().mdt_xengine_q8(ne, nch, nsp, ptr(X16), ptr(qscales), ptr(vis), ptr(vis_acc),
                               ptr(vis_i32), ptr(err), stream_handle(stream)), "xengine_q8")


def x16_bytes(ne, nch, nsp):
    """Size of the X16 tensor-core operand buffer."""
    return nch * ((nsp + 31) // 32) * ((ne + 15) // 16 * 16) * 128


def synth_iq(seed, ne, nch, s0, nsp, sigma_q8, out, tone_q16=None, src_sigma_q8=None,
             src_delay=None, stream=None):
    nsrc = 0 if src_sigma_q8 is None else int(src_sigma_q8.numel())
    check(lib().mdt_synth_iq(seed, ne, nch, s0, nsp, ptr(sigma_q8), ptr(tone_q16), nsrc,
                             ptr(src_sigma_q8), ptr(src_delay), ptr(out), stream_handle(stream)),
          "synth_iq")


def fx_integrate_static(ne, nch, ntaps, nsp, iq, window, vis, stream=None):
    """One FP32 integration with no device allocation (mdt_fx_integrate_static)."""
    check(lib().mdt_fx_integrate_static(ne, nch, ntaps, nsp, ptr(iq), ptr(window), ptr(vis),
                                        stream_handle(stream)), "mdt_fx_integrate_static")


# ----------------------------------------------------------- depacketiser
MDT_MAX_SNAPS = 8
STATS_FIELDS = ("accepted", "outside", "bad", "duplicate", "missing")


class PacketFormat(ctypes.Structure):
    """mdt_packet_format (include/mdt_fx.h)."""
    _fields_ = [("words_header", _I), ("sper_element", _I), ("inputs_per_station", _I),
                ("nsnap", _I), ("inputs_per_snap", _I * MDT_MAX_SNAPS), ("sample_bits", _I),
                ("packet_bytes", _I)]


def packet_format(sper_element, inputs_per_snap=(10, 10, 10, 8), inputs_per_station=38,
                  words_header=4, sample_bits=32, packet_bytes=None):
    """A packet format; the defaults are the reference's SNAP layout
    (MDT_OneStation_client.h:64-68) and its packet size, which fits the
    largest SNAP ((2 + 10*SperElement)*2 words, MDT_OneStation_client.cu:353)."""
    f = PacketFormat()
    f.words_header = words_header
    f.sper_element = sper_element
    f.inputs_per_station = inputs_per_station
    f.nsnap = len(inputs_per_snap)
    for k, n in enumerate(inputs_per_snap):
        f.inputs_per_snap[k] = n
    f.sample_bits = sample_bits
    if packet_bytes is None:
        per = 8 if sample_bits == 32 else 2
        packet_bytes = 4 * words_header + sper_element * max(inputs_per_snap) * per
        packet_bytes = (packet_bytes + 3) // 4 * 4
    f.packet_bytes = packet_bytes
    return f


def depacketise_seen_words(fmt, ne, nch, sample0, nspectra):
    n = ctypes.c_size_t()
    check(lib().mdt_depacketise_seen_words(ctypes.byref(fmt), ne, nch, sample0, nspectra,
                                           ctypes.byref(n)), "depacketise_seen_words")
    return n.value


def depacketise(fmt, packets, npackets, ne, nch, sample0, nspectra, out, seen, stats,
                stream=None):
    """stats: device int64 tensor of 5 counters (STATS_FIELDS)."""
    check(lib().mdt_depacketise(ctypes.byref(fmt), ptr(packets), npackets, ne, nch, sample0,
                                nspectra, ptr(out), ptr(seen), ptr(stats),
                                stream_handle(stream)), "depacketise")


def depacketise_finish(fmt, ne, nch, sample0, nspectra, out, seen, stats, stream=None):
    check(lib().mdt_depacketise_finish(ctypes.byref(fmt), ne, nch, sample0, nspectra, ptr(out),
                                       ptr(seen), ptr(stats), stream_handle(stream)),
          "depacketise_finish")


class _DepackStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_ulonglong) for n in STATS_FIELDS]


class Ingest:
    """Streaming ingest pipeline (mdt_ingest_*): host int8 packets in,
    integrations out, in order."""

    def __init__(self, nelements, nchannels, ntaps, nspectra, fmt, max_packets,
                 formatted=False, precision=MDT_PREC_FP32):
        self._h = None
        d = _Desc(nelements, nchannels, ntaps, nspectra, precision)
        self.fmt = fmt
        h = _P()
        check(lib().mdt_ingest_create(ctypes.byref(d), ctypes.byref(fmt), max_packets,
                                      1 if formatted else 0, ctypes.byref(h)), "ingest_create")
        self._h = h
        self.out_bytes = self.counters()["out_bytes"]

    def set_window(self, window):
        check(lib().mdt_ingest_set_window(self._h, ptr(window)), "ingest_set_window")

    def push(self, packets, npackets=None):
        """packets: host numpy uint8 [n][packet_bytes] (or a raw address)."""
        n = len(packets) if npackets is None else npackets
        check(lib().mdt_ingest_push(self._h, _host_ptr(packets), n), "ingest_push")

    def flush(self):
        check(lib().mdt_ingest_flush(self._h), "ingest_flush")

    def pop(self, out=None, wait=True):
        """Returns (integration index or -1, stats dict); fills `out` (host
        buffer of out_bytes) when given."""
        it = ctypes.c_longlong()
        st = _DepackStats()
        check(lib().mdt_ingest_pop(self._h, None if out is None else _host_ptr(out),
                                   ctypes.byref(it), ctypes.byref(st), 1 if wait else 0),
              "ingest_pop")
        return it.value, {n: getattr(st, n) for n in STATS_FIELDS}

    def counters(self):
        late, bad, nxt = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        ob = ctypes.c_size_t()
        check(lib().mdt_ingest_counters(self._h, ctypes.byref(late), ctypes.byref(bad),
                                        ctypes.byref(nxt), ctypes.byref(ob)), "ingest_counters")
        return dict(late=late.value, bad=bad.value, next_window=nxt.value, out_bytes=ob.value)

    def close(self):
        if self._h:
            check(lib().mdt_ingest_destroy(self._h), "ingest_destroy")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------- output
def num_baselines(nelements, npols=1):
    n = _L()
    check(lib().mdt_num_baselines(nelements, npols, ctypes.byref(n)), "num_baselines")
    return n.value


def format_baselines(nelements, npols, nch, vis, out, fftshift=True, stream=None):
    check(lib().mdt_format_baselines(nelements, npols, nch, ptr(vis), ptr(out),
                                     1 if fftshift else 0, stream_handle(stream)),
          "format_baselines")


def write_csv(path, nelements, npols, nch, formatted, append=False, nthreads=0):
    """formatted: host buffer (numpy complex64 [nbl][Nch] or a CPU tensor)."""
    check(lib().mdt_write_csv(os.fsencode(path), nelements, npols, nch, _host_ptr(formatted),
                              1 if append else 0, nthreads), "write_csv")


def write_binary(path, nelements, npols, nch, formatted, append=False):
    check(lib().mdt_write_binary(os.fsencode(path), nelements, npols, nch,
                                 _host_ptr(formatted), 1 if append else 0), "write_binary")


# ----------------------------------------------------------- adjoints
def apply_gains(ne, nch, nsp, X, gains, Y, stream=None):
    check(lib().mdt_apply_gains(ne, nch, nsp, ptr(X), ptr(gains), ptr(Y), stream_handle(stream)),
          "apply_gains")


def xengine_adjoint_f32(ne, nch, nsp, G, Y, dY, scale, stream=None):
    check(lib().mdt_xengine_adjoint_f32(ne, nch, nsp, ptr(G), ptr(Y), ptr(dY), scale,
                                        stream_handle(stream)), "xengine_adjoint_f32")


def gain_adjoint(ne, nch, nsp, dY, X=None, gains=None, dgains=None, dF=None, stream=None):
    check(lib().mdt_gain_adjoint(ne, nch, nsp, ptr(dY), ptr(X), ptr(gains), ptr(dgains), ptr(dF),
                                 stream_handle(stream)), "gain_adjoint")


def pfb_tap_grad(ne, nch, ntaps, nsp, gradP, iq, gradW, workspace, stream=None):
    nbytes = workspace.numel() * workspace.element_size()
    check(lib().mdt_pfb_tap_grad(ne, nch, ntaps, nsp, ptr(gradP), ptr(iq), ptr(gradW),
                                 ptr(workspace), nbytes, stream_handle(stream)), "pfb_tap_grad")


# ----------------------------------------------------------- plan API
class _Desc(ctypes.Structure):
    _fields_ = [("nelements", _I), ("nchannels", _I), ("ntaps", _I), ("nspectra", _I),
                ("precision", _I)]


class FxPlan:
    """Fused F-engine + X-engine plan (mdt_fx_*)."""

    def __init__(self, nelements, nchannels, ntaps, nspectra, precision=MDT_PREC_FP32,
                 stream=None):
        self.ne, self.nch, self.ntaps, self.nsp = nelements, nchannels, ntaps, nspectra
        d = _Desc(nelements, nchannels, ntaps, nspectra, precision)
        h = _P()
        check(lib().mdt_fx_create(ctypes.byref(d), ctypes.byref(h)), "mdt_fx_create")
        self._h = h
        self.set_stream(stream)

    def set_stream(self, stream=None):
        check(lib().mdt_fx_set_stream(self._h, stream_handle(stream)), "mdt_fx_set_stream")

    def set_window(self, window):
        check(lib().mdt_fx_set_window(self._h, ptr(window)), "mdt_fx_set_window")

    def set_accumulator(self, acc):
        """FP64 cross-integration accumulator (complex128 CUDA tensor) or None."""
        check(lib().mdt_fx_set_accumulator(self._h, ptr(acc)), "mdt_fx_set_accumulator")

    def set_channel_scales(self, scales):
        """INT8 plans: per-channel requantisation scales (CUDA float tensor) or
        None to recalibrate at the next integration."""
        check(lib().mdt_fx_set_channel_scales(self._h, ptr(scales)), "mdt_fx_set_channel_scales")

    def get_channel_scales(self, out):
        check(lib().mdt_fx_get_channel_scales(self._h, ptr(out)), "mdt_fx_get_channel_scales")

    def scale(self):
        v = ctypes.c_float(0)
        check(lib().mdt_fx_get_scale(self._h, ctypes.byref(v)), "mdt_fx_get_scale")
        return v.value

    def check(self):
        """Synchronise and raise on a device-side wait timeout."""
        check(lib().mdt_fx_check(self._h), "mdt_fx_check")

    def workspace_bytes(self):
        v = ctypes.c_size_t(0)
        check(lib().mdt_fx_workspace_bytes(self._h, ctypes.byref(v)), "mdt_fx_workspace_bytes")
        return v.value

    def execute(self, iq, nint, vis):
        check(lib().mdt_fx_execute(self._h, ptr(iq), nint, ptr(vis)), "mdt_fx_execute")

    def stream_reset(self):
        check(lib().mdt_fx_stream_reset(self._h), "mdt_fx_stream_reset")

    def stream_push(self, iq, vis):
        check(lib().mdt_fx_stream_push(self._h, ptr(iq), ptr(vis)), "mdt_fx_stream_push")

    def execute_host(self, h_iq, nint, h_vis):
        """h_iq / h_vis: host buffers (numpy arrays or pinned torch CPU tensors)."""
        check(lib().mdt_fx_execute_host(self._h, _host_ptr(h_iq), nint, _host_ptr(h_vis)),
              "mdt_fx_execute_host")

    def set_timing(self, enable=True):
        check(lib().mdt_fx_set_timing(self._h, 1 if enable else 0), "mdt_fx_set_timing")

    def get_timing(self):
        """(F-engine ms, X-engine ms, integrations) recorded since set_timing."""
        f, x, n = ctypes.c_double(0), ctypes.c_double(0), _I(0)
        check(lib().mdt_fx_get_timing(self._h, ctypes.byref(f), ctypes.byref(x), ctypes.byref(n)),
              "mdt_fx_get_timing")
        return f.value, x.value, n.value

    def close(self):
        if self._h:
            check(lib().mdt_fx_destroy(self._h), "mdt_fx_destroy")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FxBatch:
    """Many independent jobs (mdt_fx_batch_*): jobs = [(NE, Nch, Ntaps, Nsp), ...],
    f16 tensor-core path, one graph-captured batch launch per integration."""

    def __init__(self, jobs):
        self.jobs = [tuple(int(v) for v in j) for j in jobs]
        arr = (_Desc * len(self.jobs))(*[_Desc(ne, nch, nt, nsp, MDT_PREC_FP16)
                                         for ne, nch, nt, nsp in self.jobs])
        h = _P()
        check(lib().mdt_fx_batch_create(arr, len(self.jobs), ctypes.byref(h)), "mdt_fx_batch_create")
        self._h = h

    @property
    def stream(self):
        s = _P()
        check(lib().mdt_fx_batch_get_stream(self._h, ctypes.byref(s)), "mdt_fx_batch_get_stream")
        return s.value

    def set_window(self, job, window):
        check(lib().mdt_fx_batch_set_window(self._h, job, ptr(window)), "mdt_fx_batch_set_window")

    def autotune(self):
        w, o = _I(0), _I(0)
        check(lib().mdt_fx_batch_autotune(self._h, ctypes.byref(w), ctypes.byref(o)),
              "mdt_fx_batch_autotune")
        return w.value, bool(o.value)

    def execute(self, iqs, viss, use_graph=True):
        n = len(self.jobs)
        a = (_P * n)(*[ptr(x) for x in iqs])
        b = (_P * n)(*[ptr(x) for x in viss])
        check(lib().mdt_fx_batch_execute(self._h, a, b, 1 if use_graph else 0),
              "mdt_fx_batch_execute")

    def check(self):
        check(lib().mdt_fx_batch_check(self._h), "mdt_fx_batch_check")

    def close(self):
        if self._h:
            check(lib().mdt_fx_batch_destroy(self._h), "mdt_fx_batch_destroy")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
