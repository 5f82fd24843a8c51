"""ctypes wrapper of oracle/_ref/libref_kernels.so -- the reference's own OpenCL kernels
compiled for the CPU (TEST INFRASTRUCTURE; pins the oracle; available only where the
reference is mounted and ``oracle/build_ref.sh`` has run)."""
import contextlib
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_kernels.so")
_lib = None


def reference_root():
    """Where the reference sources are mounted: the root build_ref.sh resolves (its argument
    default, or $FLUIDS_REFERENCE_ROOT)."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--root"], capture_output=True, text=True)
    return r.stdout.strip()


REFERENCE_ROOT = reference_root()


SRC_COPIES = os.path.join(HERE, "_ref", "src", "grid.cl")


def available():
    return (os.path.exists(LIB) or os.path.isdir(os.path.join(REFERENCE_ROOT, "kernels"))
            or os.path.exists(SRC_COPIES))


def has_mesh_code():
    """The mesh entry points need the reference's own mesh sources at build time."""
    try:
        lib().ref_load_obj
        return True
    except (AttributeError, RuntimeError):
        return False


def build(force=False):
    if os.path.exists(LIB) and not force:
        return LIB
    if not (os.path.isdir(os.path.join(REFERENCE_ROOT, "kernels")) or os.path.exists(SRC_COPIES)):
        return None
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT])
    return LIB if os.path.exists(LIB) else None


def lib():
    global _lib
    if _lib is None:
        if build() is None:
            raise RuntimeError("reference kernels unavailable")
        _lib = C.CDLL(LIB)
    return _lib


# entry points the reference's Monaghan build exports too (name + "_monaghan")
_MONAGHAN = {"ref_wc_density_pressure", "ref_wc_acceleration", "ref_wc_integrate", "ref_compute_normals",
             "ref_pci_initial_density", "ref_pci_initial_forces", "ref_pci_predict_pos", "ref_pci_update_pressure",
             "ref_pci_pressure_force", "ref_pci_integrate", "ref_boundary_phi", "ref_transform_particles",
             "ref_fluid_force"}
_suffix = ""


@contextlib.contextmanager
def monaghan():
    """Inside this block the kernel wrappers run the reference's kernels as built without
    USE_MULLER_KERNELS (the Monaghan kernels of kernels/monaghan_kernels.h)."""
    global _suffix
    old, _suffix = _suffix, "_monaghan"
    try:
        yield
    finally:
        _suffix = old


def _f(name):
    return getattr(lib(), name + (_suffix if name in _MONAGHAN else ""))


def P(a):
    """Pointer to a contiguous numpy array (or NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def f(x):
    return C.c_float(float(x))


def i(x):
    return C.c_int(int(x))


def compute_hashes(pos4, size, h, cps):
    n = len(pos4)
    hs = np.zeros(n, np.uint32)
    mk = np.zeros(n, np.int32)
    _f("ref_compute_hashes")(P(pos4), i(n), f(size), f(h), i(cps), P(hs), P(mk))
    return hs, mk


def compute_cell_intervals(spos4, hashes, size, h, cps, out=None):
    """out: a reused 2 * cps^3 int32 table, zero-filled here as grid.cpp:41 fills it."""
    if out is None:
        iv = np.zeros(2 * cps ** 3, np.int32)
    else:
        iv = out
        _f("ref_fill_zero")(P(iv), C.c_longlong(iv.size))
    _f("ref_compute_cell_intervals")(P(spos4), P(hashes), i(len(spos4)), f(size), f(h), i(cps), P(iv))
    return iv


def compute_neigh_list(ref_pos4, neigh_pos4, intervals, size, h, h_define, cps, cap=50):
    n = len(ref_pos4)
    lst = np.zeros(cap * max(n, 1), np.int32)
    ln = np.zeros(n, np.int32)
    _f("ref_compute_neigh_list")(P(ref_pos4), i(n), P(neigh_pos4), P(intervals), f(size), f(h), f(h_define),
                                 i(cps), P(lst), P(ln))
    return lst, ln


def wc_density_pressure(spos4, flist, flen, bpos4, bphi, blist, blen, mass, h, gas_k, rho0, poly6, h_define):
    n = len(spos4)
    d = np.zeros(n, np.float32)
    p = np.zeros(n, np.float32)
    _f("ref_wc_density_pressure")(P(spos4), i(n), P(d), P(p), f(mass), f(h), f(gas_k), f(rho0), f(poly6),
                                  P(flen), P(flist), P(blist), P(blen), P(bpos4), P(bphi), f(h_define))
    return d, p


def wc_acceleration(spos4, svel4, nrm4, dens, pres, flist, flen, bpos4, bphi, blist, blen, g, mass, h, mu, sigma,
                    rho0, sc9, st_main, st_term, h_define):
    n = len(spos4)
    acc = np.zeros((n, 4), np.float32)
    g4 = np.array([0.0, -g, 0.0, 0.0], np.float32)
    sc = np.ascontiguousarray(sc9, np.float32)
    _f("ref_wc_acceleration")(P(spos4), P(svel4), P(nrm4), P(dens), P(pres), P(acc), i(n), P(g4), f(mass), f(h),
                              f(h * h), f(mu), f(sigma), f(rho0), P(sc), P(flen), P(flist), P(blist), P(blen),
                              P(bpos4), P(bphi), f(st_main), f(st_term), f(h_define))
    return acc


def wc_integrate(spos4, svel4, svh4, acc4, dt, max_vel, limits, h_define):
    n = len(spos4)
    op, ov, ovh = (np.zeros((n, 4), np.float32) for _ in range(3))
    lim = np.array(list(limits) + [0.0], np.float32)
    _f("ref_wc_integrate")(P(spos4), P(svel4), P(svh4), P(acc4), i(n), f(dt), P(op), P(ov), P(ovh), f(max_vel),
                           P(lim), f(h_define))
    return op, ov, ovh


def compute_normals(spos4, dens, flist, flen, w_grad, mass_define, h_define, local_size=64):
    n = len(spos4)
    nrm = np.zeros((n, 4), np.float32)
    _f("ref_compute_normals")(P(spos4), P(dens), P(nrm), i(n), P(flen), P(flist), f(w_grad), f(mass_define),
                              f(h_define), i(local_size))
    return nrm


def pci_initial_density(spos4, flist, flen, bpos4, bphi, blist, blen, w_eval, h_def, m_def, rho_def, local_size=64):
    n = len(spos4)
    d = np.zeros(n, np.float32)
    _f("ref_pci_initial_density")(P(spos4), P(d), i(n), P(flen), P(flist), P(blist), P(blen), P(bpos4), P(bphi),
                                  f(w_eval), f(h_def), f(m_def), f(rho_def), i(local_size))
    return d


def pci_initial_forces(spos4, svel4, dens, nrm4, flist, flen, mu, sigma, visc_lapl, st_main, st_term, h_def, m_def,
                       rho_def, local_size=64):
    n = len(spos4)
    fo = np.zeros((n, 4), np.float32)
    _f("ref_pci_initial_forces")(P(spos4), P(svel4), P(dens), P(nrm4), P(fo), i(n), f(mu), f(sigma), P(flen),
                                 P(flist), f(visc_lapl), f(st_main), f(st_term), f(h_def), f(m_def), f(rho_def),
                                 i(local_size))
    return fo


def pci_predict_pos(spos4, svel4, fo4, fp4, dt, g, max_vel, limits, h_def, m_def, rho_def):
    n = len(spos4)
    pred = np.zeros((n, 4), np.float32)
    g4 = np.array([0.0, -g, 0.0, 0.0], np.float32)
    lim = np.array(list(limits) + [0.0], np.float32)
    _f("ref_pci_predict_pos")(P(spos4), P(svel4), P(fo4), P(fp4), P(pred), i(n), f(dt), P(g4), f(max_vel), P(lim),
                              f(h_def), f(m_def), f(rho_def))
    return pred


def pci_update_pressure(pred4, pres, delta, flist, flen, bpos4, bphi, blist, blen, w_eval, h_def, m_def, rho_def,
                        local_size=64):
    n = len(pred4)
    dv = np.zeros(n, np.float32)
    p = np.ascontiguousarray(pres, np.float32).copy()
    _f("ref_pci_update_pressure")(P(pred4), P(dv), P(p), i(n), f(delta), P(flen), P(flist), P(blist), P(blen),
                                  P(bpos4), P(bphi), f(w_eval), f(h_def), f(m_def), f(rho_def), i(local_size))
    return dv, p


def pci_pressure_force(spos4, dens, pres, size, h, cps, flist, flen, bpos4, bphi, blist, blen, w_grad, h_def, m_def,
                       rho_def, local_size=64):
    n = len(spos4)
    fp = np.zeros((n, 4), np.float32)
    _f("ref_pci_pressure_force")(P(spos4), P(dens), P(pres), P(fp), i(n), f(size), f(h), i(cps), P(flen), P(flist),
                                 P(blist), P(blen), P(bpos4), P(bphi), f(w_grad), f(h_def), f(m_def), f(rho_def),
                                 i(local_size))
    return fp


def pci_integrate(spos4, svel4, fo4, fp4, dt, g, max_vel, limits, h_def, m_def, rho_def):
    n = len(spos4)
    op, ov = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)
    g4 = np.array([0.0, -g, 0.0, 0.0], np.float32)
    lim = np.array(list(limits) + [0.0], np.float32)
    _f("ref_pci_integrate")(P(spos4), P(svel4), P(fo4), P(fp4), P(op), P(ov), i(n), f(dt), P(g4), f(max_vel),
                            P(lim), f(h_def), f(m_def), f(rho_def))
    return op, ov


def boundary_phi(pos4, rho0, w_eval, phi_coeff, h_define):
    n = len(pos4)
    phi = np.zeros(n, np.float32)
    _f("ref_boundary_phi")(P(pos4), P(phi), i(n), f(rho0), f(w_eval), f(phi_coeff), f(h_define))
    return phi


def transform_particles(raw4, rot3x4, lin, ang):
    n = len(raw4)
    out, vel = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)
    r = np.asarray(rot3x4, np.float32).reshape(3, 4)
    m = [np.array([r[k, 0], r[k, 1], r[k, 2], 0.0], np.float32) for k in range(3)]
    cm = np.array([r[0, 3], r[1, 3], r[2, 3], 1.0], np.float32)
    li = np.array(list(lin)[:3] + [0.0], np.float32)
    an = np.array(list(ang)[:3] + [0.0], np.float32)
    _f("ref_transform_particles")(P(raw4), P(out), P(vel), P(m[0]), P(m[1]), P(m[2]), P(li), P(an), P(cm), i(n))
    return out, vel


def fluid_force(bpos4, bphi, fpos4, fdens, fpres, intervals, mass, spiky_grad, size, h, cps, center, fvel4, bvel4,
                visc_lapl, h_define):
    n = len(bpos4)
    force, torque = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)
    c4 = np.array(list(center)[:3] + [1.0], np.float32)
    _f("ref_fluid_force")(P(bpos4), P(bphi), P(fpos4), P(fdens), P(fpres), P(intervals), f(mass), f(spiky_grad),
                          f(size), f(h), i(cps), i(n), P(force), P(torque), P(c4), P(fvel4), P(bvel4), f(visc_lapl),
                          f(h_define))
    return force, torque


def bilateral_filter(depth):
    """kernels/bilateral.cl over a (height, width) float32 image."""
    img = np.ascontiguousarray(depth, np.float32)
    out = np.zeros_like(img)
    _f("ref_bilateral_filter")(P(img), P(out), i(img.shape[1]), i(img.shape[0]))
    return out


def curvature_flow(depth, inv_proj_x, inv_proj_y):
    """kernels/curvatureflow.cl over a (height, width) float32 image."""
    img = np.ascontiguousarray(depth, np.float32)
    out = np.zeros_like(img)
    _f("ref_curvature_flow")(P(img), P(out), i(img.shape[1]), i(img.shape[0]), f(inv_proj_x), f(inv_proj_y))
    return out


def load_obj(path):
    """ModelMesh(path): (vertices (n, 3) float32, indices (m,) uint32 holding its 16-bit values)."""
    nv, ni = C.c_int(), C.c_int()
    if _f("ref_load_obj")(path.encode(), None, 0, None, 0, C.byref(nv), C.byref(ni)) != 0:
        raise RuntimeError("ModelMesh could not load " + path)
    v = np.zeros((nv.value, 3), np.float32)
    ix = np.zeros(ni.value, np.uint32)
    _f("ref_load_obj")(path.encode(), P(v), nv, P(ix), ni, C.byref(nv), C.byref(ni))
    return v, ix


def voxelize(vertices3, indices, spacing, precision):
    """vx_voxelize as Model::surface_sampling calls it: (n, 4) float32 output vertices."""
    v = np.ascontiguousarray(vertices3, np.float32)
    ix = np.ascontiguousarray(indices, np.uint32)
    n = _f("ref_voxelize")(P(v), i(len(v)), P(ix), i(len(ix)), f(spacing), f(precision), None, i(0))
    out = np.zeros((n, 4), np.float32)
    _f("ref_voxelize")(P(v), i(len(v)), P(ix), i(len(ix)), f(spacing), f(precision), P(out), i(n))
    return out


def icosphere(radius, level):
    nv, ni = C.c_int(), C.c_int()
    _f("ref_icosphere")(f(radius), C.c_uint(level), None, 0, None, 0, C.byref(nv), C.byref(ni))
    v = np.zeros((nv.value, 3), np.float32)
    ix = np.zeros(ni.value, np.uint32)
    _f("ref_icosphere")(f(radius), C.c_uint(level), P(v), nv, P(ix), ni, C.byref(nv), C.byref(ni))
    return v, ix


def _sample(fn, *args):
    n = fn(*args, None, i(0))
    out = np.zeros((max(n, 0), 4), np.float32)
    if n > 0:
        fn(*args, P(out), i(n))
    return out


def scene_box_volume(size3, center3, particle_radius):
    """BoxVolume::particles (fluid/simulation/boxvolume.cpp:11-40), the reference's own code."""
    s = np.ascontiguousarray(size3, np.float32).reshape(3)
    c = np.ascontiguousarray(center3, np.float32).reshape(3)
    return _sample(lib().ref_scene_box_volume, P(s), P(c), f(particle_radius))


def scene_fishtank(width, height, depth, spacing):
    """FishTank::surface_sampling (scene/fishtank.cpp:108-141) in body coordinates."""
    return _sample(lib().ref_scene_fishtank, f(width), f(height), f(depth), f(spacing))


def scene_cube(side, spacing):
    """Cube::surface_sampling (scene/cube.cpp:136-171) in body coordinates."""
    return _sample(lib().ref_scene_cube, f(side), f(spacing))
