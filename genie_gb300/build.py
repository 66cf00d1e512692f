"""Build recipe of the GB300 library: nvcc for sm_103a, in-tree shared object.

    python -m genie_gb300.build          # or genie_gb300.build.build()

Produces genie_gb300/libgenie_gb300.so (C ABI of include/genie_gb300.h).
Translation units compile in parallel; an unchanged tree is not rebuilt.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgenie_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC",
              "-I" + os.path.join(ROOT, "include")] + ARCH
CXX_FLAGS = ["-std=c++17", "-O3", "-fPIC", "-I" + os.path.join(ROOT, "include")]
# GENIE_CHECKED=1 builds the bounds-checked variant (index reports instead of faults)
if os.environ.get("GENIE_CHECKED") == "1":
    NVCC_FLAGS.append("-DGG_CHECKED")


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cc")))


def _fingerprint():
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cc", ".cuh", ".h")):
            with open(os.path.join(CSRC, f), "rb") as fh:
                h.update(f.encode() + fh.read())
    with open(os.path.join(ROOT, "include", "genie_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _compile(src):
    out = os.path.join(OBJ, src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-c", path, "-o", out]
    else:
        cmd = [_nvcc(), "-x", "c++"] + ["-Xcompiler", "-fPIC", "-std=c++17", "-O3",
                                        "-I" + os.path.join(ROOT, "include"), "-c", path, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return out


def build(force=False, verbose=False):
    """Compile every CUDA/C++ source for sm_103a and link libgenie_gb300.so."""
    fp = _fingerprint()
    stamp = os.path.join(OBJ, "fingerprint")
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read() == fp:
                return LIB
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(fp)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
