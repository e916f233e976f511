"""Builds the native library ``blazingsql_gb300/_lib/libgxeval.so`` in-tree.

Every translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel; the device runtime
prelude used by the JIT-compiled plan kernels is embedded as a string.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libgxeval.so")

SOURCES = ["frontend.cpp", "plan.cpp", "jit.cpp", "driver.cpp", "capi.cpp", "runtime.cu", "noalloc.cu", "learned.cu",
           "batch.cu", "aggregate.cu", "str_prepass.cu", "regex.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the evaluator")
    return cand


def _cuda_root(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _embed_prelude() -> str:
    """device_rt.inc: fp64emu.cuh + device_rt.cuh as one raw string literal."""
    dst = os.path.join(BUILD, "device_rt.inc")
    text = ""
    for name in ("fp64emu.cuh", "device_rt.cuh"):
        with open(os.path.join(CSRC, name)) as f:
            text += f.read() + "\n"
    out = 'R"GXRT(' + text + ')GXRT"\n'
    if not os.path.exists(dst) or open(dst).read() != out:
        with open(dst, "w") as f:
            f.write(out)
    return dst


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    root = _cuda_root(nvcc)
    _embed_prelude()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(HERE, "..", "include", "gx_eval.h"))
    headers.append(os.path.join(BUILD, "device_rt.inc"))
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", *ARCH, "-I", CSRC, "-I", BUILD,
              "-I", os.path.join(root, "include")]

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        path = os.path.join(CSRC, src)
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc, *common, "-c", path, "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose:
                print(" ".join(cmd))
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        # the driver API is resolved at run time (cudaGetDriverEntryPointByVersion):
        # no -lcuda, so the library also loads on hosts without a GPU driver
        lib64 = os.path.join(root, "lib64")
        cmd = [nvcc, "-shared", *ARCH, "-cudart", "shared", "-o", LIB, *objs, "-L", lib64, "-lnvrtc",
               "-Xlinker", "-rpath", "-Xlinker", lib64]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(" ".join(cmd))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
