"""Build the in-tree CUDA library libgbmie.so for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel and linked
into geosmie_gb300/_lib/libgbmie.so.  Only one -gencode target is built
(compute_103a -> sm_103a), so the build is quick on both the x86 build host
and the Arm GPU host.  ``-Xptxas -v`` output is kept in _lib/ptxas.log.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libgbmie.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-v"]


def _nvcc():
    for c in [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "gbmie.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile (when sources changed) and return the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    logs = []

    def one(src):
        obj = os.path.join(OUT_DIR, os.path.basename(src).replace(".cu", ".o"))
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-I", os.path.join(os.path.dirname(HERE), "include"),
                                            "-c", src, "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, p.stdout, p.stderr))
        return obj, p.stderr

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        for obj, log in ex.map(one, srcs):
            objs.append(obj)
            logs.append(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lcuda"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (p.stdout, p.stderr))
    os.replace(tmp, LIB)
    with open(os.path.join(OUT_DIR, "ptxas.log"), "w") as fp:
        fp.write("\n".join(logs))
    for o in objs:
        os.remove(o)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
