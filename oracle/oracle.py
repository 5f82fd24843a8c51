"""ctypes wrapper of the C++ oracle (oracle/sph_oracle.cpp) -- TEST INFRASTRUCTURE."""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
_LIB = os.path.join(BUILD, "libsph_oracle.so")
_lock = threading.Lock()
_lib = None

STAGES = dict(BOUNDARY_SYNC=0, HASHES=1, SORT=2, SHUFFLE=3, CELL_INTERVALS=4, NEIGH_LIST=5,
              SB_NEIGH_LIST=6, WC_DENSITY=7, NORMALS=8, WC_ACCEL=9, WC_INTEGRATE=10,
              PCI_INIT_DENSITY=11, PCI_INIT_FORCES=12, PCI_LOOP=13, PCI_INTEGRATE=14,
              BOUNDARY_FORCES=15, PCI_PREDICT=16, PCI_UPDATE_PRESSURE=17,
              PCI_PRESSURE_FORCE=18)
FIELDS = dict(POS=0, VEL=1, VEL_HALF=2, POS_SORTED=3, VEL_SORTED=4, VEL_HALF_SORTED=5,
              HASHES=6, MASK=7, CELL_INTERVALS=8, NEIGH_LIST=9, NEIGH_LEN=10, SB_NEIGH_LIST=11,
              SB_NEIGH_LEN=12, DENSITY=13, PRESSURE=14, NORMAL=15, ACCEL=16, POS_PRED=17,
              FORCE_OTHER=18, FORCE_PRESSURE=19, DENS_VAR=20, BPOS_SORTED=21, BPHI_SORTED=22,
              BCELL_INTERVALS=23, BHASHES=24, BMASK=25, BPHI=26, BPOS=27, BODY_FORCE=28,
              BODY_TORQUE=29, PCI_ITERS=30, PCI_MAXERR=31, ID=32)
# WCSPHSimulation::simulate order (fluid/simulation/wcsphsimluation.cpp:40-106)
WCSPH_STEP = ["BOUNDARY_SYNC", "HASHES", "SORT", "SHUFFLE", "CELL_INTERVALS", "NEIGH_LIST",
              "SB_NEIGH_LIST", "WC_DENSITY", "NORMALS", "WC_ACCEL", "BOUNDARY_FORCES",
              "WC_INTEGRATE"]


class OrcConfig(C.Structure):
    _fields_ = [("method", C.c_int), ("mode", C.c_int), ("precision", C.c_int), ("neigh_cap", C.c_int),
                ("time_step", C.c_float), ("max_vel", C.c_float), ("particle_radius", C.c_float),
                ("support_radius", C.c_float), ("pci_min_iter", C.c_int), ("pci_max_iter", C.c_int),
                ("pci_error_ratio", C.c_float), ("pci_relax_max_iter", C.c_int),
                ("rest_density", C.c_float), ("k_viscosity", C.c_float), ("gravity", C.c_float),
                ("gas_stiffness", C.c_float), ("surface_tension", C.c_float), ("grid_size", C.c_float),
                ("grid_margin", C.c_float), ("phi_coeff", C.c_float), ("container", C.c_float * 3),
                ("relax_on_add", C.c_int), ("threads", C.c_int), ("kernels", C.c_int)]


class OrcDerived(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("mass", "mass_def", "h", "h_def", "rest_density_def", "poly6_eval",
                                          "poly6_grad", "spiky_grad", "visc_lapl", "st_main", "st_term",
                                          "default_eval", "boundary_eval", "pci_delta")] + \
               [("grid_origin", C.c_float * 3), ("grid_dims", C.c_int * 3), ("grid_wrap", C.c_int),
                ("key_bits", C.c_int)]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_}
        d["grid_origin"] = list(self.grid_origin)
        d["grid_dims"] = list(self.grid_dims)
        return d


def lib_path():
    return _LIB


def kwargs_from_params(p, container):
    """Oracle keywords equal to a solver parameter struct (any object with the sph_params
    field names, e.g. fluids_gb300.capi.SphParams)."""
    return dict(method=p.method, mode=p.mode, container=tuple(container), neigh_cap=p.neigh_cap,
                time_step=p.time_step, max_vel=p.max_vel, particle_radius=p.particle_radius,
                support_radius=p.support_radius, pci_min_iter=p.pcisph_min_iterations,
                pci_max_iter=p.pcisph_max_iterations, pci_error_ratio=p.pcisph_error_ratio,
                pci_relax_max_iter=p.pcisph_relax_max_iterations, rest_density=p.rest_density,
                k_viscosity=p.k_viscosity, gravity=p.gravity, gas_stiffness=p.gas_stiffness,
                surface_tension=p.surface_tension, grid_size=p.grid_size, grid_margin=p.grid_margin,
                phi_coeff=p.boundary_phi_coeff, relax_on_add=p.relax_on_add, kernels=getattr(p, "kernels", 0))


def build_oracle(force=False):
    """Compiles oracle/sph_oracle.cpp with g++ (OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "sph_oracle.cpp")
    hdr = os.path.join(HERE, "sph_oracle.h")
    if (not force and os.path.exists(_LIB)
            and os.path.getmtime(_LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return _LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = _LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                           src, "-o", tmp])
    os.replace(tmp, _LIB)
    return _LIB


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build_oracle()
        lib = C.CDLL(_LIB)
        vp, ip, fp = C.c_void_p, C.c_int, C.POINTER(C.c_float)
        lib.orc_create.restype = vp
        lib.orc_create.argtypes = [C.POINTER(OrcConfig)]
        lib.orc_destroy.argtypes = [vp]
        lib.orc_set_fluid.argtypes = [vp, fp, fp, ip]
        lib.orc_add_boundary.argtypes = [vp, fp, ip, ip, fp, fp, fp, C.c_float]
        lib.orc_run_stage.argtypes = [vp, ip]
        lib.orc_step.argtypes = [vp, ip]
        lib.orc_field_elems.restype = C.c_longlong
        lib.orc_field_elems.argtypes = [vp, ip]
        lib.orc_field_kind.argtypes = [vp, ip]
        lib.orc_get.argtypes = [vp, ip, vp]
        lib.orc_set.argtypes = [vp, ip, vp]
        lib.orc_derived.argtypes = [vp, C.POINTER(OrcDerived)]
        lib.orc_morton3.restype = C.c_uint32
        lib.orc_morton3.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        lib.orc_stable_sort_pairs.argtypes = [vp, vp, ip]
        lib.orc_stats.argtypes = [vp, C.POINTER(C.c_double)]
        lib.orc_set_body_dynamics.argtypes = [vp, ip, ip, fp, C.c_float]
        lib.orc_body_state.argtypes = [vp, ip, fp, fp, fp]
        _lib = lib
        return lib


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def morton3(x, y, z):
    return int(_load().orc_morton3(x, y, z))


def stable_sort_pairs(keys, vals):
    k = np.ascontiguousarray(keys, dtype=np.uint32).copy()
    v = np.ascontiguousarray(vals, dtype=np.int32).copy()
    _load().orc_stable_sort_pairs(k.ctypes.data, v.ctypes.data, len(k))
    return k, v


class Oracle:
    """One oracle solver instance.  ``method``: 0 WCSPH / 1 PCISPH; ``mode``: 0 COMPAT /
    1 PHYSICS; ``precision``: 0 float / 1 double.  Other keywords are OrcConfig fields."""

    def __init__(self, method=0, mode=0, precision=0, container=(2.0, 1.0, 1.0), **kw):
        lib = _load()
        cfg = OrcConfig()
        defaults = dict(neigh_cap=50, time_step=2e-4, max_vel=10.0, particle_radius=0.0075,
                        support_radius=0.03, pci_min_iter=3, pci_max_iter=3, pci_error_ratio=0.01,
                        pci_relax_max_iter=10000, rest_density=1000.0, k_viscosity=0.01, gravity=9.81,
                        gas_stiffness=57142.857, surface_tension=0.001, grid_size=5.0, grid_margin=2.0,
                        phi_coeff=1.0, relax_on_add=0, threads=0, kernels=0)
        defaults.update(kw)
        cfg.method, cfg.mode, cfg.precision = method, mode, precision
        for k, v in defaults.items():
            setattr(cfg, k, v)
        for a in range(3):
            cfg.container[a] = container[a]
        self.cfg = cfg
        self.precision = precision
        self._h = lib.orc_create(C.byref(cfg))
        self._lib = lib

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_destroy(self._h)
            self._h = None

    def set_fluid(self, pos4, vel4=None):
        p = np.ascontiguousarray(pos4, dtype=np.float32).reshape(-1, 4)
        v = None if vel4 is None else np.ascontiguousarray(vel4, dtype=np.float32).reshape(-1, 4)
        self._lib.orc_set_fluid(self._h, _fptr(p), _fptr(v), len(p))

    def add_boundary(self, pos4, can_move=0, rot3x4=None, lin=None, ang=None, mass=0.0):
        p = np.ascontiguousarray(pos4, dtype=np.float32).reshape(-1, 4)
        r = None if rot3x4 is None else np.ascontiguousarray(rot3x4, dtype=np.float32).reshape(12)
        li = None if lin is None else np.ascontiguousarray(lin, dtype=np.float32).reshape(4)
        an = None if ang is None else np.ascontiguousarray(ang, dtype=np.float32).reshape(4)
        self._lib.orc_add_boundary(self._h, _fptr(p), len(p), int(can_move), _fptr(r), _fptr(li), _fptr(an),
                                   float(mass))

    def stage(self, name):
        s = STAGES[name] if isinstance(name, str) else int(name)
        if self._lib.orc_run_stage(self._h, s) != 0:
            raise ValueError("bad stage %r" % (name,))

    def step(self, n=1):
        self._lib.orc_step(self._h, int(n))

    def get(self, field):
        f = FIELDS[field] if isinstance(field, str) else int(field)
        n = self._lib.orc_field_elems(self._h, f)
        if n < 0:
            raise ValueError("bad field %r" % (field,))
        kind = self._lib.orc_field_kind(self._h, f)
        dt = {0: (np.float64 if self.precision else np.float32), 1: np.int32, 2: np.uint32}[kind]
        out = np.empty(int(n), dtype=dt)
        self._lib.orc_get(self._h, f, out.ctypes.data)
        return out

    def set(self, field, arr):
        f = FIELDS[field] if isinstance(field, str) else int(field)
        n = self._lib.orc_field_elems(self._h, f)
        kind = self._lib.orc_field_kind(self._h, f)
        dt = {0: (np.float64 if self.precision else np.float32), 1: np.int32, 2: np.uint32}[kind]
        a = np.ascontiguousarray(arr, dtype=dt).reshape(-1)
        if a.size != n:
            raise ValueError("size mismatch for %r: %d vs %d" % (field, a.size, n))
        self._lib.orc_set(self._h, f, a.ctypes.data)

    def derived(self):
        d = OrcDerived()
        self._lib.orc_derived(self._h, C.byref(d))
        return d.as_dict()

    def set_body_dynamics(self, body, enabled=True, inv_inertia=(0.0, 0.0, 0.0), radius=0.0):
        ii = np.ascontiguousarray(inv_inertia, dtype=np.float32)
        rc = self._lib.orc_set_body_dynamics(self._h, int(body), int(bool(enabled)), _fptr(ii), float(radius))
        if rc != 0:
            raise ValueError("body %d cannot be dynamic (needs can_move and mass > 0)" % body)

    def body_state(self, body):
        rot = np.zeros(12, np.float32)
        lin = np.zeros(4, np.float32)
        ang = np.zeros(4, np.float32)
        self._lib.orc_body_state(self._h, int(body), _fptr(rot), _fptr(lin), _fptr(ang))
        return rot.reshape(3, 4), lin[:3], ang[:3]

    def stats(self):
        out = (C.c_double * 8)()
        self._lib.orc_stats(self._h, out)
        keys = ["mean_compression", "mean_abs_density_error", "max_density_error", "kinetic", "potential",
                "com_x", "com_y", "com_z"]
        return dict(zip(keys, list(out)))
