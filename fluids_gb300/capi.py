"""ctypes binding of the C ABI in include/sph_capi.h (libsph_gb300.so).

This is the Python face of the drop-in boundary: every call goes through the exported
``extern "C"`` entry points.  The library must exist (``fluids_gb300.build()``); on a
machine with a GPU there is no fallback -- a missing library or device raises.
"""
import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB
_lock = threading.Lock()
_lib = None

SPH_WCSPH, SPH_PCISPH = 0, 1
SPH_MODE_COMPAT, SPH_MODE_PHYSICS = 0, 1
SPH_KERNELS_MULLER, SPH_KERNELS_MONAGHAN = 0, 1
SPH_NEIGH_SCAN, SPH_NEIGH_LIST = 0, 1
SPH_FAULT_NONE, SPH_FAULT_BARRIER_STALL, SPH_FAULT_ALLOC_FAIL = 0, 1, 2
FLAGS = dict(NAN=1, ESCAPED=2, TIMEOUT=4, OVERFLOW=8, NONCONVERGED=16, NONSMOOTH=32)
STATUS = {0: "SPH_OK", 1: "SPH_E_INVALID", 2: "SPH_E_CUDA", 3: "SPH_E_NONCONVERGED", 4: "SPH_E_ESCAPED",
          5: "SPH_E_NAN", 6: "SPH_E_TIMEOUT", 7: "SPH_E_OVERFLOW", 8: "SPH_E_STATE", 9: "SPH_E_NOMEM"}
(SPH_OK, SPH_E_INVALID, SPH_E_CUDA, SPH_E_NONCONVERGED, SPH_E_ESCAPED, SPH_E_NAN, SPH_E_TIMEOUT, SPH_E_OVERFLOW,
 SPH_E_STATE, SPH_E_NOMEM) = range(10)
STAGES = dict(BOUNDARY_SYNC=0, HASHES=1, SORT=2, SHUFFLE=3, CELL_INTERVALS=4, NEIGH_LIST=5, SB_NEIGH_LIST=6,
              WC_DENSITY=7, NORMALS=8, WC_ACCEL=9, WC_INTEGRATE=10, PCI_INIT_DENSITY=11, PCI_INIT_FORCES=12,
              PCI_LOOP=13, PCI_INTEGRATE=14, BOUNDARY_FORCES=15, PCI_PREDICT=16, PCI_UPDATE_PRESSURE=17,
              PCI_PRESSURE_FORCE=18)
FIELDS = dict(POS=0, VEL=1, VEL_HALF=2, POS_SORTED=3, VEL_SORTED=4, VEL_HALF_SORTED=5, HASHES=6, MASK=7,
              CELL_INTERVALS=8, NEIGH_LIST=9, NEIGH_LEN=10, SB_NEIGH_LIST=11, SB_NEIGH_LEN=12, DENSITY=13,
              PRESSURE=14, NORMAL=15, ACCEL=16, POS_PRED=17, FORCE_OTHER=18, FORCE_PRESSURE=19, DENS_VAR=20,
              BPOS_SORTED=21, BPHI_SORTED=22, BCELL_INTERVALS=23, BHASHES=24, BMASK=25, BPHI=26, BPOS=27,
              BODY_FORCE=28, BODY_TORQUE=29, PCI_ITERS=30, PCI_MAXERR=31, ID=32)
_KIND = {0: np.float32, 1: np.int32, 2: np.uint32}

# Every symbol include/sph_capi.h declares (checked by tests/test_capi_symbols.py).
EXPORTS = ["sph_default_params", "sph_create", "sph_destroy", "sph_last_error", "sph_reset", "sph_set_stream",
           "sph_set_rect_limits", "sph_add_volume", "sph_add_boundary", "sph_set_body_transform",
           "sph_particle_count", "sph_boundary_particle_count", "sph_simulate", "sph_run_stage",
           "sph_synchronize", "sph_device_flags", "sph_field_elems", "sph_field_kind", "sph_get_field",
           "sph_set_field", "sph_field_device_ptr", "sph_body_forces", "sph_stats", "sph_sort_pairs",
           "sph_scene_box_volume", "sph_scene_fishtank", "sph_scene_cube", "sph_jitter", "sph_cuda_available",
           "sph_describe", "sph_profile_step", "sph_step_kernel_launches", "sph_simulate_host",
           "sph_sort_pairs_noalloc",
           "sph_batch_create",
           "sph_batch_scene_count", "sph_batch_scene_range", "sph_batch_stats", "sph_batch_scene_grid",
           "sph_adj_create", "sph_adj_destroy", "sph_adj_last_error", "sph_adj_forward", "sph_adj_backward",
           "sph_adj_flags", "sph_adj_tape_bytes", "sph_set_block_size", "sph_set_tile_shape",
           "sph_get_tile_shape", "sph_get_field_async",
           "sph_set_field_async",
           "sph_set_body_dynamics", "sph_get_body_state", "sph_render_depth", "sph_filter_bilateral",
           "sph_render_smooth", "sph_filter_curvature_flow", "sph_render_normals", "sph_scene_load_obj",
           "sph_scene_voxelize", "sph_scene_icosphere", "sph_scene_sphere", "sph_save_state", "sph_load_state",
           "sph_inject_fault", "sph_render_shade", "sph_scene_wall", "sph_render_frame",
           "sph_render_particles"]


class SphParams(C.Structure):
    _fields_ = [("method", C.c_int), ("mode", C.c_int), ("time_step", C.c_float), ("max_vel", C.c_float),
                ("particle_radius", C.c_float), ("support_radius", C.c_float),
                ("pcisph_min_iterations", C.c_int), ("pcisph_max_iterations", C.c_int),
                ("pcisph_error_ratio", C.c_float), ("pcisph_relax_max_iterations", C.c_int),
                ("rest_density", C.c_float), ("k_viscosity", C.c_float), ("gravity", C.c_float),
                ("gas_stiffness", C.c_float), ("surface_tension", C.c_float), ("grid_size", C.c_float),
                ("grid_margin", C.c_float), ("boundary_phi_coeff", C.c_float), ("neigh_cap", C.c_int),
                ("relax_on_add", C.c_int), ("neighbor_mode", C.c_int), ("use_graph", C.c_int),
                ("block_size", C.c_int), ("kernels", C.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class SphDerived(C.Structure):
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


class SceneDesc(C.Structure):
    _fields_ = [("container", C.c_float * 3), ("k_viscosity", C.c_float), ("gas_stiffness", C.c_float),
                ("fluid_pos4", C.c_void_p), ("fluid_vel4", C.c_void_p), ("n_fluid", C.c_int),
                ("boundary_pos4", C.c_void_p), ("n_boundary", C.c_int)]


class SphView(C.Structure):
    _fields_ = [("modelview", C.c_float * 16), ("projection", C.c_float * 16), ("point_radius", C.c_float),
                ("point_scale", C.c_float), ("width", C.c_int), ("height", C.c_int)]


def make_view(modelview, projection, point_radius, point_scale, width, height):
    """sph_view from 4x4 matrices in mathematical (row, column) layout; the struct holds
    them column-major like GL uniforms."""
    v = SphView()
    mv = np.asarray(modelview, np.float32).reshape(4, 4).T.reshape(-1)
    pr = np.asarray(projection, np.float32).reshape(4, 4).T.reshape(-1)
    for k in range(16):
        v.modelview[k] = float(mv[k])
        v.projection[k] = float(pr[k])
    v.point_radius = float(point_radius)
    v.point_scale = float(point_scale)
    v.width = int(width)
    v.height = int(height)
    return v


class SphLight(C.Structure):
    _fields_ = [("direction", C.c_float * 3), ("diffuse", C.c_float * 4)]


def make_lights(lights):
    """[(direction (3,), diffuse rgba (4,) in 0..1)] -> ctypes array of SphLight."""
    arr = (SphLight * max(1, len(lights)))()
    for k, (d, c) in enumerate(lights):
        for a in range(3):
            arr[k].direction[a] = float(d[a])
        for a in range(4):
            arr[k].diffuse[a] = float(c[a])
    return arr


SPH_RENDER_PARTICLES, SPH_RENDER_SCREEN_SPACE = 0, 1


class SphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


def lib():
    """Loads libsph_gb300.so (building it in-tree if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            _build.build()
        L = C.CDLL(LIB_PATH)
        vp, ip, fp, cp = C.c_void_p, C.c_int, C.c_void_p, C.c_char_p
        PP = C.POINTER(SphParams)
        sig = {
            "sph_default_params": (None, [ip, PP]),
            "sph_create": (ip, [PP, C.POINTER(vp)]),
            "sph_destroy": (ip, [vp]),
            "sph_last_error": (cp, [vp]),
            "sph_reset": (ip, [vp, PP]),
            "sph_set_stream": (ip, [vp, vp]),
            "sph_set_rect_limits": (ip, [vp, C.c_float, C.c_float, C.c_float]),
            "sph_add_volume": (ip, [vp, fp, fp, ip]),
            "sph_add_boundary": (ip, [vp, fp, ip, ip, fp, fp, fp, C.c_float]),
            "sph_set_body_transform": (ip, [vp, ip, fp, fp, fp]),
            "sph_particle_count": (ip, [vp]),
            "sph_boundary_particle_count": (ip, [vp]),
            "sph_simulate": (ip, [vp, ip]),
            "sph_run_stage": (ip, [vp, ip]),
            "sph_synchronize": (ip, [vp]),
            "sph_device_flags": (ip, [vp, C.POINTER(C.c_uint), ip]),
            "sph_field_elems": (C.c_longlong, [vp, ip]),
            "sph_field_kind": (ip, [ip]),
            "sph_get_field": (ip, [vp, ip, vp, C.c_size_t]),
            "sph_set_field": (ip, [vp, ip, vp, C.c_size_t]),
            "sph_field_device_ptr": (ip, [vp, ip, C.POINTER(vp)]),
            "sph_body_forces": (ip, [vp, fp, fp, ip]),
            "sph_stats": (ip, [vp, C.POINTER(C.c_double)]),
            "sph_sort_pairs": (ip, [vp, vp, ip, ip, vp]),
            "sph_scene_box_volume": (ip, [fp, fp, C.c_float, fp, ip]),
            "sph_scene_fishtank": (ip, [C.c_float, C.c_float, C.c_float, C.c_float, fp, ip]),
            "sph_scene_cube": (ip, [C.c_float, C.c_float, fp, ip]),
            "sph_jitter": (None, [fp, ip, C.c_float, C.c_uint64]),
            "sph_cuda_available": (ip, []),
            "sph_describe": (ip, [PP, fp, C.POINTER(SphDerived)]),
            "sph_profile_step": (ip, [vp, ip, C.POINTER(C.c_float), ip, C.POINTER(ip), C.c_char_p, C.c_size_t]),
            "sph_step_kernel_launches": (ip, [vp, C.POINTER(ip)]),
            "sph_simulate_host": (ip, [vp, fp, fp, fp, ip]),
            "sph_sort_pairs_noalloc": (ip, [vp, vp, vp, vp, ip, ip, vp]),
            "sph_batch_create": (ip, [PP, ip, C.POINTER(SceneDesc), C.POINTER(vp)]),
            "sph_batch_scene_count": (ip, [vp]),
            "sph_batch_scene_range": (ip, [vp, ip, C.POINTER(ip), C.POINTER(ip)]),
            "sph_batch_stats": (ip, [vp, C.POINTER(C.c_double), ip]),
            "sph_batch_scene_grid": (ip, [vp, ip, C.POINTER(C.c_float), C.POINTER(ip), C.POINTER(C.c_longlong)]),
            "sph_adj_create": (ip, [vp, ip, ip, C.POINTER(vp)]),
            "sph_adj_destroy": (ip, [vp]),
            "sph_adj_last_error": (cp, [vp]),
            "sph_adj_forward": (ip, [vp, vp, vp, C.c_float, C.c_float, vp, vp]),
            "sph_adj_backward": (ip, [vp, vp, vp, vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]),
            "sph_adj_flags": (ip, [vp, C.POINTER(C.c_uint)]),
            "sph_adj_tape_bytes": (ip, [vp, C.POINTER(C.c_size_t)]),
            "sph_set_block_size": (ip, [vp, ip]),
            "sph_set_tile_shape": (ip, [vp, ip]),
            "sph_get_tile_shape": (ip, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int)]),
            "sph_get_field_async": (ip, [vp, ip, vp, C.c_size_t]),
            "sph_set_field_async": (ip, [vp, ip, vp, C.c_size_t]),
            "sph_set_body_dynamics": (ip, [vp, ip, ip, fp, C.c_float]),
            "sph_get_body_state": (ip, [vp, ip, fp, fp, fp]),
            "sph_render_depth": (ip, [vp, C.POINTER(SphView), vp]),
            "sph_filter_bilateral": (ip, [vp, vp, ip, ip, vp]),
            "sph_render_smooth": (ip, [vp, vp, ip, ip, ip, vp]),
            "sph_filter_curvature_flow": (ip, [vp, vp, ip, ip, C.c_float, C.c_float, vp]),
            "sph_render_normals": (ip, [vp, vp, ip, ip, C.POINTER(C.c_float), vp]),
            "sph_scene_load_obj": (ip, [C.c_char_p, fp, ip, fp, ip, C.POINTER(ip), C.POINTER(ip)]),
            "sph_scene_voxelize": (ip, [fp, ip, fp, ip, C.c_float, C.c_float, fp, ip]),
            "sph_scene_icosphere": (ip, [C.c_float, ip, fp, ip, fp, ip, C.POINTER(ip), C.POINTER(ip)]),
            "sph_scene_sphere": (ip, [C.c_float, C.c_float, fp, ip]),
            "sph_scene_wall": (ip, [C.c_float, C.c_float, C.c_float, fp, ip]),
            "sph_render_frame": (ip, [vp, C.POINTER(SphView), ip, ip, vp, ip, fp]),
            "sph_render_particles": (ip, [vp, C.POINTER(SphView), vp, ip, vp]),
            "sph_save_state": (ip, [vp, C.c_char_p]),
            "sph_load_state": (ip, [vp, C.c_char_p]),
            "sph_inject_fault": (ip, [vp, ip]),
            "sph_render_shade": (ip, [vp, vp, vp, vp, ip, ip, ip, C.POINTER(C.c_float), C.POINTER(C.c_float), vp,
                                      vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def ptr(a):
    """Address of a contiguous numpy array (None for None)."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


def f4(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if a.ndim == 1:
        a = a.reshape(-1, 4)
    if a.ndim != 2 or a.shape[1] != 4:
        raise ValueError("expected an (n, 4) float32 array, got shape %r" % (a.shape,))
    return a


def default_params(method=SPH_WCSPH):
    p = SphParams()
    lib().sph_default_params(int(method), C.byref(p))
    return p


def make_params(method=SPH_WCSPH, **kw):
    p = default_params(method)
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError("unknown parameter %r" % k)
        setattr(p, k, v)
    return p


def describe(params, container=(0.0, 0.0, 0.0)):
    """Constants and grid a context derives (sph_describe; host only)."""
    c = np.ascontiguousarray(container, np.float32)
    d = SphDerived()
    check(lib().sph_describe(C.byref(params), ptr(c), C.byref(d)))
    return d.as_dict()


def cuda_available():
    return bool(lib().sph_cuda_available())


def last_error(handle=None):
    s = lib().sph_last_error(handle)
    return s.decode() if s else ""


def check(rc, handle=None):
    if rc != 0:
        raise SphError(rc, last_error(handle))
    return rc


class Context:
    """Owns one ``sph_ctx``.  Thin: each method is one C-ABI call."""

    def __init__(self, params):
        self._lib = lib()
        h = C.c_void_p()
        check(self._lib.sph_create(C.byref(params), C.byref(h)))
        self.h = h
        self.params = params

    def close(self):
        for ref in getattr(self, "_dependents", ()):
            dep = ref()
            if dep is not None:
                dep.close()
        if getattr(self, "h", None):
            self._lib.sph_destroy(self.h)
            self.h = None

    def _attach(self, dep):
        """Handles that use this context (an Adjoint) are closed before it."""
        import weakref
        if not hasattr(self, "_dependents"):
            self._dependents = []
        self._dependents.append(weakref.ref(dep))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        return check(rc, self.h)

    def set_stream(self, cuda_stream):
        """Runs this context's work on a caller stream (an integer cudaStream_t)."""
        self._c(self._lib.sph_set_stream(self.h, C.c_void_p(int(cuda_stream))))

    def set_block_size(self, block_size):
        self._c(self._lib.sph_set_block_size(self.h, int(block_size)))

    def set_rect_limits(self, w, h, d):
        self._c(self._lib.sph_set_rect_limits(self.h, w, h, d))

    def add_volume(self, pos4, vel4=None):
        p = f4(pos4)
        v = None if vel4 is None else f4(vel4)
        self._c(self._lib.sph_add_volume(self.h, ptr(p), ptr(v), len(p)))

    def add_boundary(self, pos4, can_move=False, rot3x4=None, lin=None, ang=None, mass=0.0):
        p = f4(pos4)
        r = None if rot3x4 is None else np.ascontiguousarray(rot3x4, np.float32).reshape(12)
        li = None if lin is None else np.ascontiguousarray(lin, np.float32).reshape(4)
        an = None if ang is None else np.ascontiguousarray(ang, np.float32).reshape(4)
        self._c(self._lib.sph_add_boundary(self.h, ptr(p), len(p), int(bool(can_move)), ptr(r), ptr(li), ptr(an),
                                           float(mass)))

    def set_body_transform(self, body, rot3x4=None, lin=None, ang=None):
        r = None if rot3x4 is None else np.ascontiguousarray(rot3x4, np.float32).reshape(12)
        li = None if lin is None else np.ascontiguousarray(lin, np.float32).reshape(4)
        an = None if ang is None else np.ascontiguousarray(ang, np.float32).reshape(4)
        self._c(self._lib.sph_set_body_transform(self.h, int(body), ptr(r), ptr(li), ptr(an)))

    def reset(self, params):
        self.params = params
        self._c(self._lib.sph_reset(self.h, C.byref(params)))

    def simulate(self, steps=1):
        self._c(self._lib.sph_simulate(self.h, int(steps)))

    def stage(self, name):
        s = STAGES[name] if isinstance(name, str) else int(name)
        self._c(self._lib.sph_run_stage(self.h, s))

    def synchronize(self):
        self._c(self._lib.sph_synchronize(self.h))

    def device_flags(self, clear=False):
        f = C.c_uint()
        self._c(self._lib.sph_device_flags(self.h, C.byref(f), int(bool(clear))))
        return int(f.value)

    def particle_count(self):
        return int(self._lib.sph_particle_count(self.h))

    def boundary_particle_count(self):
        return int(self._lib.sph_boundary_particle_count(self.h))

    def get(self, field):
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        n = self._lib.sph_field_elems(self.h, fid)
        if n < 0:
            raise SphError(1, "bad field %r" % (field,))
        out = np.empty(int(n), dtype=_KIND[self._lib.sph_field_kind(fid)])
        self._c(self._lib.sph_get_field(self.h, fid, out.ctypes.data, out.nbytes))
        return out

    def set(self, field, arr):
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        a = np.ascontiguousarray(arr, dtype=_KIND[self._lib.sph_field_kind(fid)]).reshape(-1)
        self._c(self._lib.sph_set_field(self.h, fid, a.ctypes.data, a.nbytes))

    def device_ptr(self, field):
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        p = C.c_void_p()
        self._c(self._lib.sph_field_device_ptr(self.h, fid, C.byref(p)))
        return int(p.value or 0)

    def set_body_dynamics(self, body, enabled=True, inv_inertia=(0.0, 0.0, 0.0), radius=0.0):
        ii = np.ascontiguousarray(inv_inertia, dtype=np.float32)
        self._c(self._lib.sph_set_body_dynamics(self.h, int(body), int(bool(enabled)), ptr(ii), float(radius)))

    def body_state(self, body):
        """(rot3x4 (3, 4), linear velocity (3,), angular velocity (3,))"""
        rot = np.zeros(12, np.float32)
        lin = np.zeros(4, np.float32)
        ang = np.zeros(4, np.float32)
        self._c(self._lib.sph_get_body_state(self.h, int(body), ptr(rot), ptr(lin), ptr(ang)))
        return rot.reshape(3, 4), lin[:3], ang[:3]

    def inject_fault(self, kind):
        """sph_inject_fault (failure-detection tests)."""
        self._c(self._lib.sph_inject_fault(self.h, int(kind)))

    def render_frame(self, view, filter_iterations=2, method=None, lights=()):
        """sph_render_frame: a shaded (h, w, 4) float32 host image of the particles
        (screen-space surface by default; method SPH_RENDER_PARTICLES with lights)."""
        out = np.zeros((view.height, view.width, 4), np.float32)
        m = SPH_RENDER_SCREEN_SPACE if method is None else int(method)
        arr = make_lights(lights)
        self._c(self._lib.sph_render_frame(self.h, C.byref(view), m, int(filter_iterations), C.cast(arr, C.c_void_p),
                                           len(lights), ptr(out)))
        return out

    def render_particles(self, view, lights, d_rgba):
        """sph_render_particles into the device image at d_rgba."""
        arr = make_lights(lights)
        self._c(self._lib.sph_render_particles(self.h, C.byref(view), C.cast(arr, C.c_void_p), len(lights),
                                               C.c_void_p(int(d_rgba))))

    def save_state(self, path):
        """Checkpoint (sph_save_state)."""
        self._c(self._lib.sph_save_state(self.h, str(path).encode()))

    def load_state(self, path):
        """Resume from a checkpoint into a context built from the same scene (sph_load_state)."""
        self._c(self._lib.sph_load_state(self.h, str(path).encode()))

    def render_depth(self, view, d_depth):
        """sph_render_depth into the device image at address d_depth (view: SphView)."""
        self._c(self._lib.sph_render_depth(self.h, C.byref(view), C.c_void_p(int(d_depth))))

    def body_forces(self, nbodies):
        f = np.zeros((nbodies, 4), np.float32)
        t = np.zeros((nbodies, 4), np.float32)
        self._c(self._lib.sph_body_forces(self.h, ptr(f), ptr(t), int(nbodies)))
        return f, t

    def profile_step(self, nsteps):
        """Average device ms per step of each kernel group of the step (sph_profile_step)."""
        ms = (C.c_float * 64)()
        ng = C.c_int()
        names = C.create_string_buffer(4096)
        self._c(self._lib.sph_profile_step(self.h, int(nsteps), ms, 64, C.byref(ng), names, 4096))
        keys = names.value.decode().split(",") if ng.value else []
        return dict(zip(keys, [float(ms[i]) for i in range(ng.value)]))

    def simulate_host(self, pos4, vel4, vhalf4=None, steps=1):
        """sph_simulate_host: steps with the state in host arrays (float32, (N, 4), C order),
        updated in place; waits for the context stream before returning."""
        arrs = [pos4, vel4] + ([vhalf4] if vhalf4 is not None else [])
        for a in arrs:
            if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"] or a.size != 4 * self.particle_count():
                raise ValueError("host state arrays must be C-contiguous float32 of shape (N, 4)")
        self._c(self._lib.sph_simulate_host(self.h, pos4.ctypes.data, vel4.ctypes.data,
                                            vhalf4.ctypes.data if vhalf4 is not None else None, int(steps)))
        self._c(self._lib.sph_synchronize(self.h))

    def step_kernel_launches(self):
        """Kernel launches in one step's CUDA graph (0 without a graph)."""
        n = C.c_int()
        self._c(self._lib.sph_step_kernel_launches(self.h, C.byref(n)))
        return n.value

    def stats(self):
        out = (C.c_double * 8)()
        self._c(self._lib.sph_stats(self.h, out))
        keys = ["mean_compression", "mean_abs_density_error", "max_density_error", "kinetic", "potential",
                "com_x", "com_y", "com_z"]
        return dict(zip(keys, list(out)))


class BatchContext(Context):
    """A batched context (sph_batch_create): ``scenes`` is a list of dicts with keys
    container (w, h, d), mu, kgas, fluid ((n, 4) array), boundary ((m, 4) array) and
    optionally vel."""

    def __init__(self, params, scenes):
        self._lib = lib()
        keep = []
        descs = (SceneDesc * len(scenes))()
        for d, s in zip(descs, scenes):
            fl = f4(s["fluid"])
            bd = f4(s["boundary"]) if s.get("boundary") is not None else None
            vl = f4(s["vel"]) if s.get("vel") is not None else None
            keep += [fl, bd, vl]
            for a in range(3):
                d.container[a] = s["container"][a]
            d.k_viscosity = s["mu"]
            d.gas_stiffness = s["kgas"]
            d.fluid_pos4, d.n_fluid = ptr(fl), len(fl)
            d.fluid_vel4 = ptr(vl)
            d.boundary_pos4, d.n_boundary = (ptr(bd), len(bd)) if bd is not None else (None, 0)
        h = C.c_void_p()
        check(self._lib.sph_batch_create(C.byref(params), len(scenes), descs, C.byref(h)))
        self.h = h
        self.params = params
        self.nscenes = len(scenes)

    def scene_range(self, s):
        a, n = C.c_int(), C.c_int()
        self._c(self._lib.sph_batch_scene_range(self.h, int(s), C.byref(a), C.byref(n)))
        return a.value, n.value

    def scene_grid(self, s):
        o = (C.c_float * 3)()
        d = (C.c_int * 3)()
        base = C.c_longlong()
        self._c(self._lib.sph_batch_scene_grid(self.h, int(s), o, d, C.byref(base)))
        return list(o), list(d), base.value

    def scene_stats(self):
        out = (C.c_double * (8 * self.nscenes))()
        self._c(self._lib.sph_batch_stats(self.h, out, self.nscenes))
        return np.array(out[:], dtype=np.float64).reshape(self.nscenes, 8)

    def set_tile_shape(self, ctas_per_sm):
        """CTAs per SM of the persistent per-scene tile launches (0: 2048 / block size)."""
        self._c(self._lib.sph_set_tile_shape(self.h, int(ctas_per_sm)))

    def tile_shape(self):
        """{tile_particles, ctas_per_sm, tiles, blocks} of the persistent tile launches."""
        v = [C.c_int() for _ in range(4)]
        self._c(self._lib.sph_get_tile_shape(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("tile_particles", "ctas_per_sm", "tiles", "blocks"), [x.value for x in v]))


class Adjoint:
    """Differentiable WCSPH over a context (sph_adj_*): ``forward`` runs ``steps`` steps
    from (x0, v0) with viscosity ``mu`` and Tait stiffness ``k``; ``backward`` takes dL/dx_T
    (and optionally dL/dv_T) and returns the gradients.  Arrays are (n, 4) float32 in
    particle-id order: numpy arrays (host) or integer device addresses."""

    def __init__(self, ctx, steps, checkpoint_every=20):
        self._lib = lib()
        self.ctx = ctx
        self.n = ctx.particle_count()
        self.steps = int(steps)
        h = C.c_void_p()
        check(self._lib.sph_adj_create(ctx.h, int(steps), int(checkpoint_every), C.byref(h)), ctx.h)
        self.h = h
        ctx._attach(self)

    def close(self):
        if getattr(self, "h", None):
            self._lib.sph_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        if rc != 0:
            msg = self._lib.sph_adj_last_error(self.h)
            raise SphError(rc, msg.decode() if msg else "")
        return rc

    @staticmethod
    def _addr(a):
        if a is None:
            return None
        if isinstance(a, int):
            return C.c_void_p(a)
        return C.c_void_p(ptr(a))

    def forward(self, x0, v0, mu, k, out_x=None, out_v=None):
        """Returns (xT, vT) as numpy arrays unless device outputs are given."""
        host_out = out_x is None
        if host_out:
            x0, v0 = f4(x0), f4(v0)
            out_x = np.zeros((self.n, 4), np.float32)
            out_v = np.zeros((self.n, 4), np.float32)
        self._c(self._lib.sph_adj_forward(self.h, self._addr(x0), self._addr(v0), float(mu), float(k),
                                          self._addr(out_x), self._addr(out_v)))
        return (out_x, out_v) if host_out else None

    def backward(self, gxT, gvT=None, out_gx0=None, out_gv0=None):
        """Returns dict(g_x0, g_v0, g_mu, g_k, g_c0); arrays are numpy unless device
        outputs are given."""
        host_out = out_gx0 is None and not isinstance(gxT, int)
        if host_out:
            gxT = f4(gxT)
            gvT = f4(gvT) if gvT is not None else None
            out_gx0 = np.zeros((self.n, 4), np.float32)
            out_gv0 = np.zeros((self.n, 4), np.float32)
        gm, gk, gc = C.c_double(), C.c_double(), C.c_double()
        self._c(self._lib.sph_adj_backward(self.h, self._addr(gxT), self._addr(gvT), self._addr(out_gx0),
                                           self._addr(out_gv0), C.byref(gm), C.byref(gk), C.byref(gc)))
        return dict(g_x0=out_gx0, g_v0=out_gv0, g_mu=gm.value, g_k=gk.value, g_c0=gc.value)

    def flags(self):
        f = C.c_uint()
        self._c(self._lib.sph_adj_flags(self.h, C.byref(f)))
        return f.value

    def tape_bytes(self):
        b = C.c_size_t()
        self._c(self._lib.sph_adj_tape_bytes(self.h, C.byref(b)))
        return b.value


def sort_pairs_device(d_keys, d_vals, n, key_bits=32, stream=None):
    """sph_sort_pairs on device addresses (ints)."""
    check(lib().sph_sort_pairs(C.c_void_p(d_keys), C.c_void_p(d_vals), int(n), int(key_bits),
                               C.c_void_p(stream or 0)))


def filter_bilateral(d_in, d_out, width, height, stream=None):
    """sph_filter_bilateral on device addresses (ints)."""
    check(lib().sph_filter_bilateral(C.c_void_p(d_in), C.c_void_p(d_out), int(width), int(height),
                                     C.c_void_p(stream or 0)))


def render_smooth(d_depth, d_tmp, width, height, iterations, stream=None):
    check(lib().sph_render_smooth(C.c_void_p(d_depth), C.c_void_p(d_tmp), int(width), int(height),
                                  int(iterations), C.c_void_p(stream or 0)))


def filter_curvature_flow(d_in, d_out, width, height, inv_proj_x, inv_proj_y, stream=None):
    check(lib().sph_filter_curvature_flow(C.c_void_p(d_in), C.c_void_p(d_out), int(width), int(height),
                                          float(inv_proj_x), float(inv_proj_y), C.c_void_p(stream or 0)))


def render_normals(d_depth, d_normals4, width, height, inv_projection, stream=None):
    """inv_projection: 4x4 in mathematical layout (passed column-major)."""
    ip = np.ascontiguousarray(np.asarray(inv_projection, np.float32).reshape(4, 4).T.reshape(-1))
    check(lib().sph_render_normals(C.c_void_p(d_depth), C.c_void_p(d_normals4), int(width), int(height),
                                   ip.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(stream or 0)))


def render_shade(d_depth, d_normals4, d_background4, d_cube4, cube_size, width, height, modelview,
                 inv_projection, d_rgba, stream=None):
    """sph_render_shade; matrices in mathematical layout (passed column-major), device
    addresses as ints (0 / None for no background or cube map)."""
    mv = np.ascontiguousarray(np.asarray(modelview, np.float32).reshape(4, 4).T.reshape(-1))
    ip = np.ascontiguousarray(np.asarray(inv_projection, np.float32).reshape(4, 4).T.reshape(-1))
    fpt = C.POINTER(C.c_float)
    check(lib().sph_render_shade(C.c_void_p(d_depth), C.c_void_p(d_normals4), C.c_void_p(d_background4 or 0),
                                 C.c_void_p(d_cube4 or 0), int(cube_size), int(width), int(height),
                                 mv.ctypes.data_as(fpt), ip.ctypes.data_as(fpt), C.c_void_p(d_rgba),
                                 C.c_void_p(stream or 0)))
