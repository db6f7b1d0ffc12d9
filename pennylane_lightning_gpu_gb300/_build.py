"""In-tree build of the native parts of the engine.

* ``_lib/liblgpu_gb300.so`` — the sm_103a CUDA kernels behind the C ABI in
  ``include/lgpu.h`` (nvcc, one translation unit per kernel family, compiled
  in parallel, ``-gencode arch=compute_103a,code=sm_103a``).
* ``lightning_gpu_qubit_ops*.so`` — the pybind11 module with the drop-in C++
  classes (g++, pybind11 headers shipped with torch, linked to the library
  above through an ``$ORIGIN`` rpath).

No cmake; everything is rebuilt only when a source is newer than its output.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
KERNELS = os.path.join(CSRC, "kernels")
CPP = os.path.join(CSRC, "cpp")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "liblgpu_gb300.so")
EXT_SUFFIX = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
MODULE = os.path.join(PKG, "lightning_gpu_qubit_ops" + EXT_SUFFIX)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + KERNELS]


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _nvcc():
    return os.path.join(_cuda_home(), "bin", "nvcc")


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _pybind_include():
    import torch  # torch ships the pybind11 headers

    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
        return inc
    import pybind11  # pragma: no cover - fallback

    return pybind11.get_include()


def build(verbose=False, jobs=None):
    """Build the kernel library and the pybind module (incremental)."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu = sorted(glob.glob(os.path.join(KERNELS, "*.cu")))
    headers = (glob.glob(os.path.join(KERNELS, "*.cuh")) + glob.glob(os.path.join(KERNELS, "*.h")) +
               [os.path.join(INCLUDE, "lgpu.h")])
    objs = [os.path.join(BUILD, os.path.basename(f)[:-3] + ".o") for f in cu]
    todo = [(src, obj) for src, obj in zip(cu, objs) if _newer(obj, [src] + headers)]

    cpp_headers = glob.glob(os.path.join(CPP, "*.hpp")) + [os.path.join(INCLUDE, "lgpu.h")]
    bind_src = os.path.join(CSRC, "bindings", "Bindings.cpp")
    bind_obj = os.path.join(BUILD, "Bindings.o")
    py_inc = sysconfig.get_paths()["include"]
    cuda_inc = os.path.join(_cuda_home(), "include")

    def compile_cu(pair):
        src, obj = pair
        _run([_nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"], verbose)
        os.replace(obj + ".tmp", obj)

    def compile_bindings():
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-I" + INCLUDE, "-I" + CPP,
              "-I" + _pybind_include(), "-I" + py_inc, "-I" + cuda_inc, "-c", bind_src, "-o", bind_obj + ".tmp"],
             verbose)
        os.replace(bind_obj + ".tmp", bind_obj)

    jobs = jobs or max(2, min(8, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(compile_cu, p) for p in todo]
        if _newer(bind_obj, [bind_src] + cpp_headers):
            futs.append(ex.submit(compile_bindings))
        for f in futs:
            f.result()

    if _newer(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs, verbose)
        os.replace(tmp, LIB)
    if _newer(MODULE, [bind_obj, LIB]):
        tmp = MODULE + ".tmp%d" % os.getpid()
        _run(["g++", "-shared", "-o", tmp, bind_obj, "-L" + LIBDIR, "-llgpu_gb300",
              "-Wl,-rpath,$ORIGIN/_lib"], verbose)
        os.replace(tmp, MODULE)
    return LIB, MODULE


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
