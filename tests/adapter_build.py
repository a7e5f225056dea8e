"""Builds tests/adapter_check.cpp (the AMReX-side adapter's test driver)
against the AMReX stand-in, into tests/_build/.  Test infrastructure."""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")


def build(with_lib):
    os.makedirs(OUT, exist_ok=True)
    name = "libadapter_check.so" if with_lib else "libadapter_view.so"
    out = os.path.join(OUT, name)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "oracle", "ref_shim"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "mesoflow_gb300", "adapter"),
           os.path.join(HERE, "adapter_check.cpp"), "-o", out]
    if with_lib:
        from mesoflow_gb300 import abi
        abi.load()  # the library must exist (and be loaded) first
        libdir = os.path.join(ROOT, "mesoflow_gb300", "_lib")
        cmd += ["-L" + libdir, "-lmflo_gpu", "-Wl,-rpath," + libdir]
    else:
        cmd.insert(1, "-DADAPTER_NO_LIB")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("adapter test driver build failed:\n" + r.stdout + r.stderr)
    lib = C.CDLL(out)
    lib.adapter_view_check.restype = C.c_int
    if with_lib:
        PP = C.POINTER(C.c_void_p)
        IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)
        lib.adapter_dsdt.argtypes = [C.c_int, IP, PP, PP, PP, PP, C.c_int, DP, DP, IP, IP, IP, C.c_double,
                                     C.c_double, C.c_void_p]
        lib.adapter_cutcells.argtypes = [C.c_int, IP, PP, PP, PP, PP, C.c_int, DP, DP, IP, IP, IP, C.c_double,
                                         C.c_void_p]
        lib.adapter_register_scale.argtypes = [C.c_int, C.c_int, DP, C.c_double, C.c_double]
        lib.adapter_register_scale.restype = C.c_double
    return lib
