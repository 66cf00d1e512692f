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


def cuda_home():
    """The CUDA toolkit holding nvcc (its include/ and lib64/)."""
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


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


def cudart_link():
    """Link flags of the CUDA runtime (the legacy interface's headers use it)."""
    for d in ("lib64", "lib", os.path.join("targets", os.uname().machine + "-linux", "lib"),
              os.path.join("targets", "sbsa-linux", "lib")):
        p = os.path.join(cuda_home(), d)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return ["-L" + p, "-lcudart", "-Wl,-rpath," + p]
    return ["-lcudart"]


CPP = os.path.join(HERE, "cpp")
CPP_LIB = os.path.join(HERE, "libgenie.so")
SHIM_TEST = os.path.join(OBJ, "shim_test")
LEGACY_TEST = os.path.join(OBJ, "legacy_test")


def _cpp_fingerprint():
    h = hashlib.sha256()
    files = [os.path.join(CPP, f) for f in sorted(os.listdir(CPP)) if f.endswith((".cc", ".h"))]
    inc = os.path.join(ROOT, "include")
    for d, _, fs in sorted(os.walk(inc)):
        files += [os.path.join(d, f) for f in sorted(fs) if f.endswith(".h")]
    files.append(os.path.join(ROOT, "tests", "cpp", "shim_test.cc"))
    files.append(os.path.join(ROOT, "tests", "cpp", "legacy_test.cc"))
    for path in files:
        if os.path.exists(path):
            with open(path, "rb") as fh:
                h.update(path.encode() + fh.read())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build_cpp(force=False, verbose=False):
    """The C++ interface <genie/genie.h> (genie_gb300/cpp, host C++ over the C
    ABI) as libgenie.so beside libgenie_gb300.so, and its test program."""
    cxx = shutil.which("g++") or "g++"
    fp = _cpp_fingerprint()
    stamp = os.path.join(OBJ, "cpp_fingerprint")
    if not force and all(os.path.exists(p) for p in (CPP_LIB, SHIM_TEST, LEGACY_TEST, stamp)):
        with open(stamp) as f:
            if f.read() == fp:
                return CPP_LIB
    os.makedirs(OBJ, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda_home(), "include")]
    srcs = [os.path.join(CPP, f) for f in sorted(os.listdir(CPP)) if f.endswith(".cc")]
    steps = [
        [cxx, "-std=c++17", "-O2", "-fPIC", "-shared"] + inc + srcs +
        ["-o", CPP_LIB + ".tmp", "-L" + HERE, "-lgenie_gb300", "-Wl,-rpath,$ORIGIN"] + cudart_link(),
    ]
    for cmd in steps:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("C++ interface build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(CPP_LIB + ".tmp", CPP_LIB)
    for src, exe in (("shim_test.cc", SHIM_TEST), ("legacy_test.cc", LEGACY_TEST)):
        cmd = [cxx, "-std=c++17", "-O2"] + inc + [os.path.join(ROOT, "tests", "cpp", src), "-o", exe,
               "-L" + HERE, "-lgenie", "-lgenie_gb300", "-Wl,-rpath,$ORIGIN/.."] + cudart_link()
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("C++ test build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    with open(stamp, "w") as f:
        f.write(fp)
    if verbose:
        print("built", CPP_LIB)
    return CPP_LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    build_cpp(force="--force" in sys.argv, verbose=True)
