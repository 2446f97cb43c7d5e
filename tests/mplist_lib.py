"""The multiphase fluid-list layout builder (mf-lbm_gb300/csrc/listlayout.cpp) compiled for
the host through tests/mplist_host.cpp, for the CPU tests of its tables."""
import ctypes as C
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def host_lib():
    """The compiled harness, or None when g++ or the CUDA headers are missing."""
    global _lib
    if _lib is not None:
        return _lib
    gxx = shutil.which("g++")
    inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if gxx is None or not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        return None
    build = os.path.join(HERE, "_build")
    os.makedirs(build, exist_ok=True)
    out = os.path.join(build, "libmplist_host.so")
    tmp = out + f".{os.getpid()}"
    subprocess.run([gxx, "-O2", "-shared", "-fPIC", "-std=c++17", f"-I{inc}", os.path.join(HERE, "mplist_host.cpp"),
                    "-o", tmp], check=True)
    os.replace(tmp, out)
    lib = C.CDLL(out)
    P64 = C.POINTER(C.c_int64)
    lib.mph_check.restype = C.c_int64
    lib.mph_check.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P64, P64,
                              P64, P64]
    lib.mph_build.restype = C.c_int64
    lib.mph_build.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                              C.c_void_p, C.c_int, C.c_void_p]
    lib.mph_get.restype = None
    lib.mph_get.argtypes = [C.c_void_p] * 5
    _lib = lib
    return lib
