"""Build the native library ``sde_mc_gb300/lib/libsdemc.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with one
``-gencode arch=compute_103a,code=sm_103a`` target and linked into one shared
object with the CUDA runtime linked statically.  Run ``python -m
sde_mc_gb300.build`` or call :func:`build`.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
LIBNAME = "libsdemc.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: the host code's double arithmetic (the server's regression,
# the control-variate weights) rounds every operation, on x86 and Arm alike.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc_path():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build sde_mc_gb300")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime():
    """Newest modification time of the headers every translation unit may include."""
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(HERE, "..", "include", "sdemc.h"))
    return max(os.path.getmtime(h) for h in hdrs if os.path.exists(h))


def _compile(nvcc, src, extra, deps_mtime):
    obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    stamp = obj + ".cmd"
    # an object is reused when it is newer than its source and every header and
    # was built by the same command line
    if (os.path.exists(obj) and os.path.exists(stamp)
            and os.path.getmtime(obj) > max(os.path.getmtime(src), deps_mtime)
            and open(stamp).read() == " ".join(cmd)):
        return obj, ""
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), res.stderr))
    with open(stamp, "w") as f:
        f.write(" ".join(cmd))
    return obj, res.stderr


def build(verbose=False, extra=()):
    """Compile every CUDA source and link the shared library; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    deps = _deps_mtime()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, list(extra), deps), srcs))
    if verbose:
        for obj, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    out = os.path.join(LIBDIR, LIBNAME)
    tmp = out + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp] + [o for o, _ in results]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
