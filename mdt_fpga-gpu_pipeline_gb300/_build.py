"""In-tree build of libmdtfx.so (the C-ABI library) with nvcc for sm_103a.

Every translation unit in csrc/ is compiled in parallel to an object file
under _build/, then linked into libmdtfx.so next to this file, against the
shared CUDA runtime (-cudart shared: the drop-in __global__ kernels are
launched with <<<>>> from the caller's translation units, which only works
when caller and library share one runtime).  No cuFFT, no cuBLAS.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmdtfx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Size of the file-scope scratch array of mdt_fx_integrate_static (96 MiB).
STATIC_SCRATCH_BYTES = 96 << 20
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=default",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills",
              "-DMDT_STATIC_SCRATCH_BYTES=%d" % STATIC_SCRATCH_BYTES]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    dep = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    dep += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return dep


def _compile(src, extra, build_dir):
    obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force=False, verbose=False, extra=None, out=None):
    """Compile and link libmdtfx.so (or `out`); returns its path.  `extra`
    holds additional nvcc flags (e.g. -D tuning macros) for every unit."""
    lib_path = out or LIB
    if not force and out is None and not extra and up_to_date():
        return LIB
    build_dir = BUILD if out is None else out + ".objs"
    os.makedirs(build_dir, exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra, build_dir), srcs))
    if verbose:
        for obj, err in results:
            if err.strip():
                print(err)
    objs = [o for o, _ in results]
    tmp = lib_path + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force=True, verbose=True))
