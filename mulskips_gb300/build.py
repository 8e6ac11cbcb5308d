"""Build the in-tree native libraries of mulskips_gb300 for GB300 (sm_103a).

`build_all()` compiles
  _lib/libmulskips_gpu.so   the CUDA engine + C ABI (include/mulskips_gpu.h)
  _lib/mulskips.e           the drop-in host program (reads ./start.dat)
with nvcc for sm_103a only.  No CPU build of the engine exists.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB = os.path.join(PKG, "_lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 engine must be compiled with the CUDA toolkit")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("build failed: " + " ".join(cmd))
    return r.stdout


ENGINE_SOURCES = ("engine.cu", "stacking.cu")


def object_cmd(src, out):
    return [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
            "-I", os.path.join(ROOT, "include"), os.path.join(PKG, "csrc", src), "-o", out]


def link_cmd(objs, out):
    return [nvcc(), *ARCH, "-shared", *objs, "-o", out]


def host_cmd(out, lib):
    src = os.path.join(PKG, "host", "mulskips_main.cpp")
    return [nvcc(), *ARCH, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", out,
            "-L", os.path.dirname(lib), "-lmulskips_gpu", "-Xlinker", "-rpath=$ORIGIN"]


def host_only(out=None):
    out = out or os.path.join(LIB, "mulskips.e")
    return _run(host_cmd(out, os.path.join(LIB, "libmulskips_gpu.so")))


def build_all(verbose=False):
    os.makedirs(LIB, exist_ok=True)
    lib = os.path.join(LIB, "libmulskips_gpu.so")
    objs = [os.path.join(LIB, os.path.splitext(src)[0] + ".o") for src in ENGINE_SOURCES]
    # the translation units compile in parallel, then one link
    with ThreadPoolExecutor(len(objs)) as ex:
        outs = list(ex.map(lambda so: _run(object_cmd(*so)), zip(ENGINE_SOURCES, objs)))
    out = "".join(outs) + _run(link_cmd(objs, lib))
    if verbose:
        print(out)
    host_src = os.path.join(PKG, "host", "mulskips_main.cpp")
    if os.path.exists(host_src):
        _run(host_cmd(os.path.join(LIB, "mulskips.e"), lib))
    return lib


def build_oracle():
    """Compile the test oracle (oracle/Makefile).  Test infrastructure only."""
    return _run(["make", "-C", os.path.join(ROOT, "oracle")])


if __name__ == "__main__":
    with ThreadPoolExecutor(2) as ex:
        f1 = ex.submit(build_all, True)
        f2 = ex.submit(build_oracle)
        f1.result()
        f2.result()
