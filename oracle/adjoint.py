"""ctypes wrapper of the FP64 adjoint oracle (oracle/sph_adjoint_oracle.cpp) -- TEST INFRASTRUCTURE.

Only the tests use it, as the checker of the CUDA adjoint: forward(...) and backward(...)
run the differentiable WCSPH step and its reverse mode in double precision on the CPU,
and central finite differences of forward(...) check the oracle itself.
"""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
_LIB = os.path.join(BUILD, "libsph_adj_oracle.so")
_lock = threading.Lock()
_lib = None


class OrcAdjParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("h", "hh", "h2_list", "mass", "rho0", "kgas", "mu", "g", "dt",
                                          "vmax")] + \
               [("lim", C.c_double * 3)] + \
               [(n, C.c_double) for n in ("poly6", "spiky", "visc_lapl", "rmin2")] + \
               [("steps", C.c_int), ("threads", C.c_int)]


def build_adj_oracle(force=False):
    """Compiles oracle/sph_adjoint_oracle.cpp with g++ (OpenMP)."""
    src = os.path.join(HERE, "sph_adjoint_oracle.cpp")
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(src):
        return _LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = _LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp])
    os.replace(tmp, _LIB)
    return _LIB


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build_adj_oracle()
            lib = C.CDLL(_LIB)
            dp = C.POINTER(C.c_double)
            P = C.POINTER(OrcAdjParams)
            lib.orc_adj_forward.argtypes = [P, C.c_int, dp, dp, dp, dp, C.POINTER(C.c_int)]
            lib.orc_adj_backward.argtypes = [P, C.c_int, dp, dp, dp, dp, dp, dp, dp, dp]
            _lib = lib
        return _lib


def make_params(params, derived, container, steps, mu=None, k=None, threads=0):
    """Oracle parameters from an SphParams and its sph_describe() constants, with the float32
    values the CUDA kernels use (h*h and the list radius rounded as there)."""
    f = np.float32
    if not isinstance(derived, dict):
        derived = {n: getattr(derived, n) for n, _ in derived._fields_}
    h = f(derived["h"])
    rmin = f(1e-5)
    if float(rmin) > 1e-5:
        rmin = np.nextafter(rmin, f(0))
    hd = f(round(float(params.support_radius), 6))
    P = OrcAdjParams()
    P.h = float(h)
    P.hh = float(h * h)
    P.h2_list = float(hd * hd)
    P.mass = float(f(derived["mass"]))
    P.rho0 = float(f(params.rest_density))
    P.kgas = float(f(params.gas_stiffness if k is None else k))
    P.mu = float(f(params.k_viscosity if mu is None else mu))
    P.g = -float(f(params.gravity))
    P.dt = float(f(params.time_step))
    P.vmax = float(f(params.max_vel))
    for a in range(3):
        P.lim[a] = float(f(container[a]))
    P.poly6 = float(f(derived["poly6_eval"]))
    P.spiky = float(f(derived["spiky_grad"]))
    P.visc_lapl = float(f(derived["visc_lapl"]))
    P.rmin2 = float(rmin * rmin)
    P.steps = int(steps)
    P.threads = int(threads)
    return P


def _d3(a):
    a = np.asarray(a, dtype=np.float64)
    return np.ascontiguousarray(a[:, :3])


def _p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def forward(P, x0, v0):
    """Returns (xT, vT, largest neighbour count seen), arrays (n, 3) float64."""
    L = _load()
    x0, v0 = _d3(x0), _d3(v0)
    n = len(x0)
    xT, vT = np.zeros((n, 3)), np.zeros((n, 3))
    mx = C.c_int()
    L.orc_adj_forward(C.byref(P), n, _p(x0), _p(v0), _p(xT), _p(vT), C.byref(mx))
    return xT, vT, mx.value


def backward(P, x0, v0, gxT, gvT=None):
    """dict(g_x0, g_v0 (n, 3), g_mu, g_k) for the loss whose dL/dx_T is gxT."""
    L = _load()
    x0, v0, gxT = _d3(x0), _d3(v0), _d3(gxT)
    gvT = _d3(gvT) if gvT is not None else None
    n = len(x0)
    gx0, gv0 = np.zeros((n, 3)), np.zeros((n, 3))
    gm, gk = C.c_double(), C.c_double()
    L.orc_adj_backward(C.byref(P), n, _p(x0), _p(v0), _p(gxT), _p(gvT), _p(gx0), _p(gv0), C.byref(gm),
                       C.byref(gk))
    return dict(g_x0=gx0, g_v0=gv0, g_mu=gm.value, g_k=gk.value)
