"""ctypes binding of baseline/refseq.cu: the reference's own GPU FX sequence.

NOT PART OF THE PRODUCT.  The reference's PpS_Batch, ReorderFOutput and
PFB_Window_min4term_BH, compiled from the reference source for sm_103a by
baseline/build_ref_gpu.sh (baseline/_ref/mdt_ref_kernels.fatbin), run with
NVIDIA's cuFFT and cuBLAS exactly as the reference client's rank 2 calls them
(MDT_OneStation_client.cu:1083,1105,1114,1128).  tests/ use it as the second
parity check and bench.py times it as the library bar.

build() compiles refseq.cu into baseline/_build/librefseq.so (nvcc, sm_103a,
linked against libcuda; cuFFT and cuBLAS are opened at run time with
dlopen(RTLD_LOCAL | RTLD_DEEPBIND), so that their entry points cannot be
bound to the same-named shim that libmdtfx.so exports).
"""
import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "refseq.cu")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "librefseq.so")
FATBIN = os.path.join(HERE, "_ref", "mdt_ref_kernels.fatbin")

STAGES = ("PpS_Batch", "cufftExecC2C", "ReorderFOutput", "cublasCgemmBatched", "history_copy")
FINPUT, FOUTPUT, XINPUT, XOUTPUT, WINDOW = range(5)

_lib = None


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(_nvcc()))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
           "-Xcompiler", "-fPIC", "-shared", "-o", tmp, SRC,
           "-L", os.path.join(cuda, "lib64"), "-L", os.path.join(cuda, "lib64", "stubs"),
           "-lcuda", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("refseq build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


def available():
    """True when the reference kernels have been compiled (the fatbin exists)."""
    return os.path.exists(FATBIN)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P, I = ctypes.c_void_p, ctypes.c_int
        L.refseq_last_error.restype = ctypes.c_char_p
        L.refseq_create.argtypes = [ctypes.c_char_p, I, I, I, I, ctypes.POINTER(P)]
        L.refseq_destroy.argtypes = [P]
        L.refseq_ptr.argtypes = [P, I]
        L.refseq_ptr.restype = P
        L.refseq_read.argtypes = [P, I, P, ctypes.c_size_t]
        L.refseq_set_input.argtypes = [P, P, P]
        L.refseq_stage.argtypes = [P, I]
        L.refseq_sync.argtypes = [P]
        L.refseq_run.argtypes = [P, I, I, ctypes.POINTER(ctypes.c_float),
                                 ctypes.POINTER(ctypes.c_float)]
        L.refseq_window_bh.argtypes = [P, P]
        L.refseq_libraries.argtypes = [ctypes.c_char_p, I, ctypes.POINTER(I), ctypes.POINTER(I)]
        _lib = L
    return _lib


class RefSeqError(RuntimeError):
    pass


def libraries():
    """(cuFFT file, cuBLAS file, cuFFT version, cuBLAS version) of the entry
    points the harness calls."""
    buf = ctypes.create_string_buffer(4096)
    fv, bv = ctypes.c_int(), ctypes.c_int()
    _check(lib().refseq_libraries(buf, 4096, ctypes.byref(fv), ctypes.byref(bv)),
           "refseq_libraries")
    a, _, b = buf.value.decode().partition("|")
    return a, b, fv.value, bv.value


def _check(rc, what):
    if rc != 0:
        raise RefSeqError("%s: %s (code %d)" % (what, lib().refseq_last_error().decode(), rc))


class RefSeq:
    """One integration of the reference sequence at shape (NE, Nch, Ntaps, Nsp)
    on the current CUDA device.  Inputs and outputs are torch CUDA tensors."""

    def __init__(self, ne, nch, ntaps, nsp, fatbin=FATBIN):
        self.ne, self.nch, self.ntaps, self.nsp = ne, nch, ntaps, nsp
        h = ctypes.c_void_p()
        _check(lib().refseq_create(fatbin.encode(), ne, nch, ntaps, nsp, ctypes.byref(h)),
               "refseq_create")
        self.h = h

    def set_input(self, iq, window):
        """iq: int8 I/Q [(Nsp+Ntaps-1)*NE*Nch*2] on the device; window: float32
        [Ntaps*Nch] on the device."""
        _check(lib().refseq_set_input(self.h, iq.data_ptr(), window.data_ptr()),
               "refseq_set_input")

    def stage(self, k):
        _check(lib().refseq_stage(self.h, k), "refseq_stage %s" % STAGES[k])
        _check(lib().refseq_sync(self.h), "refseq_sync")

    def read(self, which, out):
        _check(lib().refseq_read(self.h, which, out.data_ptr(),
                                 out.numel() * out.element_size()), "refseq_read")
        return out

    def run(self, reps, history=True):
        """Times `reps` integrations back to back; returns (per-stage ms dict,
        ms per integration)."""
        st = (ctypes.c_float * 5)()
        tot = ctypes.c_float()
        _check(lib().refseq_run(self.h, reps, 1 if history else 0, st, ctypes.byref(tot)),
               "refseq_run")
        n = 5 if history else 4
        return {STAGES[k]: float(st[k]) for k in range(n)}, float(tot.value)

    def window_bh(self, out):
        _check(lib().refseq_window_bh(self.h, out.data_ptr()), "refseq_window_bh")
        return out

    def close(self):
        if self.h:
            lib().refseq_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
