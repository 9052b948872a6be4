"""ctypes access to the C++ FP64 oracle (TEST INFRASTRUCTURE ONLY)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(quiet=True):
    """Compile oracle/oracle.cpp into oracle/_build/liboracle.so."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "oracle.cpp")
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
            build()
        _lib = ctypes.CDLL(LIB)
        _lib.oracle_params_derive.argtypes = [ctypes.c_void_p]
        _lib.oracle_params_derive.restype = ctypes.c_int
        _lib.oracle_simulate.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_int, ctypes.c_int64]
        _lib.oracle_simulate.restype = ctypes.c_int
    return _lib


def derive(params_struct):
    """Fill the derived fields of an rp_params ctypes struct (oracle's own restatement)."""
    rc = lib().oracle_params_derive(ctypes.byref(params_struct))
    if rc != 0:
        raise ValueError(f"oracle_params_derive failed: {rc}")
    return params_struct


def simulate(params_struct, facets_soa, targets_soa, traces, prisms_soa=None,
             nthreads=0, max_targets=0):
    """Run the FP64 oracle.  Returns (complex128 [ns, nr], int64 counts [ns, 2])."""
    f = np.ascontiguousarray(facets_soa, dtype=np.float64)
    t = np.ascontiguousarray(targets_soa, dtype=np.float64).reshape(7, -1)
    tr = np.ascontiguousarray(traces, dtype=np.float64).reshape(-1, 9)
    nf = f.shape[1] if f.size else 0
    nt = t.shape[1]
    if prisms_soa is None or np.size(prisms_soa) == 0:
        pr = np.zeros((7, 0))
    else:
        pr = np.ascontiguousarray(prisms_soa, dtype=np.float64).reshape(7, -1)
    ns = tr.shape[0]
    nr = params_struct.nr
    out = np.zeros((ns, nr, 2), np.float64)
    counts = np.zeros((ns, 2), np.int64)
    rc = lib().oracle_simulate(ctypes.byref(params_struct), f.ctypes.data, nf, t.ctypes.data, nt,
                               pr.ctypes.data, pr.shape[1], tr.ctypes.data, ns, out.ctypes.data,
                               counts.ctypes.data, int(nthreads), int(max_targets))
    if rc != 0:
        raise RuntimeError(f"oracle_simulate failed: {rc}")
    return out[..., 0] + 1j * out[..., 1], counts
