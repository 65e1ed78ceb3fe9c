"""In-tree build of the engine: libamdat_gb300.so (CUDA kernels + C ABI + C++
host classes) and the amdat_gb300 command-line driver, for sm_103a only.

Translation units compile in parallel; objects are rebuilt only when a source
or header is newer.  Outputs go to amdat_gb300/_lib/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libamdat_gb300.so")
CLI = os.path.join(OUT, "amdat_gb300")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(HOST, "*.h"))
            + glob.glob(os.path.join(REPO, "include", "*.h")))


def _stale(obj: str, src: str, hdr_mtime: float) -> bool:
    return (not os.path.exists(obj)
            or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_mtime))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(verbose: bool = False, jobs: int | None = None) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    hdr_mtime = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    inc = ["-I", os.path.join(REPO, "include"), "-I", CSRC, "-I", HOST]
    cu_flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                       "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
    cxx_flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                 "-I", os.path.join(cuda, "include")]
    jobs_list = []
    lib_objs, cli_objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        lib_objs.append(obj)
        if _stale(obj, src, hdr_mtime):
            jobs_list.append([nvcc] + cu_flags + inc + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp")) + glob.glob(os.path.join(HOST, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        (cli_objs if os.path.basename(src) == "amdat_main.cpp" else lib_objs).append(obj)
        if _stale(obj, src, hdr_mtime):
            jobs_list.append(["g++"] + cxx_flags + inc + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for msg in ex.map(_run, jobs_list):
            if verbose and msg:
                print(msg, file=sys.stderr)
    newest = max(os.path.getmtime(o) for o in lib_objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + f".tmp{os.getpid()}"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + lib_objs + ["-lcudart_static", "-lrt",
                                                                   "-lpthread", "-ldl"])
        os.replace(tmp, LIB)
    if cli_objs:
        if not os.path.exists(CLI) or os.path.getmtime(CLI) < max(newest, os.path.getmtime(LIB)):
            tmp = CLI + f".tmp{os.getpid()}"
            _run(["g++", "-o", tmp] + cli_objs + ["-L", OUT, "-lamdat_gb300",
                                                   f"-Wl,-rpath,$ORIGIN"])
            os.replace(tmp, CLI)
    return LIB


TORCH_SRC = os.path.join(PKG, "torch_ext", "amdat_torch.cpp")


def torch_ext_path() -> str:
    import sysconfig
    return os.path.join(OUT, "amdat_torch" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_torch_ext(verbose: bool = False) -> str:
    """The libtorch autograd extension (amdat_torch), compiled with g++ against
    the installed torch and linked to libamdat_gb300.so (no ninja needed)."""
    import sysconfig

    import torch
    from torch.utils import cpp_extension as ce

    lib = build(verbose=verbose)
    out = torch_ext_path()
    deps = [TORCH_SRC, lib, os.path.join(REPO, "include", "amdat_gb300.h")]
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    cuda = _cuda_home()
    torch_lib = os.path.join(os.path.dirname(torch.__file__), "lib")
    flags = ["-O2", "-std=c++17", "-fPIC", "-shared", "-w",
             f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}",
             "-DTORCH_EXTENSION_NAME=amdat_torch", "-DTORCH_API_INCLUDE_EXTENSION_H"]
    abi = getattr(ce, "_get_pybind11_abi_build_flags", None)
    if abi is not None:
        flags += abi()
    incs = []
    for d in ce.include_paths("cuda") + [sysconfig.get_paths()["include"], os.path.join(REPO, "include"),
                                         os.path.join(cuda, "include")]:
        incs += ["-I", d]
    libs = ["-L", torch_lib, "-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu", "-ltorch_cuda",
            "-ltorch_python", "-L", OUT, "-lamdat_gb300", f"-Wl,-rpath,{torch_lib}",
            "-Wl,-rpath,$ORIGIN", "-L", os.path.join(cuda, "lib64"), "-lcudart"]
    tmp = out + f".tmp{os.getpid()}"
    _run(["g++"] + flags + incs + [TORCH_SRC, "-o", tmp] + libs)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
