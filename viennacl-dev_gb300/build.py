"""Builds libvclgb.so (the GB300 sparse engine) in-tree with nvcc for sm_103a.

Each translation unit under csrc/ is compiled in parallel, then linked into
one shared library exporting only the C ABI of include/vclgb.h.  The CUDA
runtime is linked statically, so the library loads next to any PyTorch build.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvclgb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-Xcompiler", "-O2",
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _newest_header():
    t = 0.0
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".hpp", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(src, extra):
    """(object path, whether it was compiled now).  The object is written under
    a temporary name and renamed, so an interrupted or concurrent build never
    leaves a partial object that looks up to date."""
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and os.path.getmtime(obj) >= _newest_header()):
        return obj, False
    tmp = "%s.%d.tmp" % (obj, os.getpid())
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if os.path.exists(tmp):
            os.remove(tmp)
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    os.replace(tmp, obj)
    return obj, True


def build(verbose=False, extra=None):
    """Compile (incrementally) and link libvclgb.so; returns its path.  The
    library is relinked whenever an object was compiled by this call or is
    newer than it, into a temporary file renamed over the old one."""
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        done = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = [o for o, _ in done]
    compiled = any(c for _, c in done)
    newest = max(os.path.getmtime(o) for o in objs)
    if compiled or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = "%s.%d.tmp" % (LIB, os.getpid())
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            if os.path.exists(tmp):
                os.remove(tmp)
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
