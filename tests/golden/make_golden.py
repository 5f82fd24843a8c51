"""Generates the golden fixtures in tests/golden/ from the reference's own OpenCL kernels,
compiled for the CPU by oracle/build_ref.sh (oracle/_ref).  Run where the reference is
mounted:

    python tests/golden/make_golden.py

    python tests/golden/make_golden.py render    # only render_small.npz
    python tests/golden/make_golden.py mesh      # only voxel_teapot.npz

Every stage output is produced by chaining reference kernels only (the key sort is the
stable ascending sort clogs performs, numpy's stable argsort; the shuffle is a gather).  The
kernel constants are the host-side derivation restated by the oracle (stored with the
fixture).  The fixtures are small (~2k fluid particles of the seeded small scene) so the
CPU and GPU parity tests can pin against the reference on machines without it.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import Oracle  # noqa: E402  (derived constants only)
from oracle import refkernels as rk  # noqa: E402
from oracle import render as orender  # noqa: E402
from scenes_np import small_scene  # noqa: E402

GRID_SIZE = 5.0


def f4(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, 4))


def compact_lists(lst, ln):
    """Column-major list[k * n + i] with lengths -> (flat entries in (i, k) order, offsets)."""
    n = len(ln)
    cols = lst.reshape(-1, n)
    flat = np.concatenate([cols[:ln[i], i] for i in range(n)]).astype(np.int32) if n else np.zeros(0, np.int32)
    off = np.concatenate([[0], np.cumsum(ln)]).astype(np.int64)
    return flat, off


def compact_intervals(iv):
    iv = iv.reshape(-1, 2)
    nz = np.nonzero(iv[:, 1] > iv[:, 0])[0]
    return nz.astype(np.int64), iv[nz].astype(np.int32)


def grid_chain(fluid, boundary, d, bphi):
    """hashes -> stable sort -> shuffle -> intervals -> fluid and boundary lists."""
    h, cps = d["h"], d["grid_dims"][0]
    out = {}
    bh, _ = rk.compute_hashes(f4(boundary), GRID_SIZE, h, cps)
    border = np.argsort(bh, kind="stable").astype(np.int32)
    bps = f4(boundary[border])
    bphi_s = np.ascontiguousarray(bphi[border])
    biv = rk.compute_cell_intervals(bps, np.ascontiguousarray(bh[border]), GRID_SIZE, h, cps)
    hs, mk = rk.compute_hashes(f4(fluid), GRID_SIZE, h, cps)
    order = np.argsort(hs, kind="stable").astype(np.int32)
    ps = f4(fluid[order])
    iv = rk.compute_cell_intervals(ps, np.ascontiguousarray(hs[order]), GRID_SIZE, h, cps)
    fl, fn = rk.compute_neigh_list(ps, ps, iv, GRID_SIZE, h, d["h_def"], cps)
    bl, bn = rk.compute_neigh_list(ps, bps, biv, GRID_SIZE, h, d["h_def"], cps)
    out.update(hashes=hs, mask_sorted=order, hashes_sorted=hs[order], pos_sorted=ps, bmask_sorted=border,
               bpos_sorted=bps, bphi_sorted=bphi_s)
    out["iv_cells"], out["iv_ranges"] = compact_intervals(iv)
    out["biv_cells"], out["biv_ranges"] = compact_intervals(biv)
    out["nlist"], out["nlist_off"] = compact_lists(fl, fn)
    out["sblist"], out["sblist_off"] = compact_lists(bl, bn)
    return out, (ps, order, iv, fl, fn, bps, bphi_s, bl, bn)


def wcsph(sc):
    kw = dict(time_step=2e-4, max_vel=10.0, k_viscosity=0.01, surface_tension=0.001, gas_stiffness=57142.857)
    o = Oracle(method=0, mode=0, container=sc["container"], **kw)
    d = o.derived()
    fluid, boundary = sc["fluid"], sc["boundary"]
    bphi = rk.boundary_phi(f4(boundary), 1000.0, d["boundary_eval"], 1.0, d["h_def"])
    out, (ps, order, iv, fl, fn, bps, bphi_s, bl, bn) = grid_chain(fluid, boundary, d, bphi)
    vel = np.zeros_like(fluid)
    vel[:, 3] = 0
    dens, pres = rk.wc_density_pressure(ps, fl, fn, bps, bphi_s, bl, bn, d["mass"], d["h"], kw["gas_stiffness"],
                                        1000.0, d["poly6_eval"], d["h_def"])
    # The kernel text gives negative densities (poly6 of r); physical densities and pressures
    # are set before the force stages so their pressure and viscosity branches run.
    phys_d = (1000.0 + 20.0 * np.sin(np.arange(len(ps)))).astype(np.float32)
    phys_p = (kw["gas_stiffness"] * ((phys_d / 1000.0) ** 7 - 1)).clip(0).astype(np.float32)
    nrm = rk.compute_normals(ps, phys_d, fl, fn, d["poly6_grad"], d["mass_def"], d["h_def"])
    sc9 = [d["poly6_eval"], d["poly6_grad"], d["poly6_grad"], 0, 0, d["visc_lapl"], 0, d["spiky_grad"], 0]
    svel = f4(vel[order])
    acc = rk.wc_acceleration(ps, svel, nrm, phys_d, phys_p, fl, fn, bps, bphi_s, bl, bn, 9.81, d["mass"], d["h"],
                             kw["k_viscosity"], kw["surface_tension"], 1000.0, sc9, d["st_main"], d["st_term"],
                             d["h_def"])
    op, ov, ovh = rk.wc_integrate(ps, svel, svel.copy(), acc, kw["time_step"], kw["max_vel"], sc["container"],
                                  d["h_def"])
    out.update(bphi=bphi, density=dens, pressure=pres, phys_density=phys_d, phys_pressure=phys_p, normal=nrm,
               accel=acc, pos_out=op, vel_out=ov, vhalf_out=ovh)
    return out, kw, d


def pcisph(sc):
    kw = dict(time_step=5e-4, max_vel=20.0, k_viscosity=0.01, surface_tension=1.0, pci_max_iter=3)
    o = Oracle(method=1, mode=0, container=sc["container"], **kw)
    d = o.derived()
    fluid, boundary = sc["fluid"], sc["boundary"]
    args = (d["h_def"], d["mass_def"], d["rest_density_def"])
    bphi = rk.boundary_phi(f4(boundary), 1000.0, d["boundary_eval"], 1.0, d["h_def"])
    out, (ps, order, iv, fl, fn, bps, bphi_s, bl, bn) = grid_chain(fluid, boundary, d, bphi)
    sv = f4(np.zeros_like(fluid)[order])
    dens = rk.pci_initial_density(ps, fl, fn, bps, bphi_s, bl, bn, d["default_eval"], *args)
    nrm = rk.compute_normals(ps, dens, fl, fn, d["poly6_grad"], d["mass_def"], d["h_def"])
    fo = rk.pci_initial_forces(ps, sv, dens, nrm, fl, fn, kw["k_viscosity"], kw["surface_tension"], d["visc_lapl"],
                               d["st_main"], d["st_term"], *args)
    fp = np.zeros_like(fo)
    pres = np.zeros(len(ps), np.float32)
    h, cps = d["h"], d["grid_dims"][0]
    maxerr = []
    for _ in range(3):
        pred = rk.pci_predict_pos(ps, sv, fo, fp, kw["time_step"], 9.81, kw["max_vel"], sc["container"], *args)
        dv, pres = rk.pci_update_pressure(pred, pres, d["pci_delta"], fl, fn, bps, bphi_s, bl, bn,
                                          d["default_eval"], *args)
        fp = rk.pci_pressure_force(ps, dens, pres, GRID_SIZE, h, cps, fl, fn, bps, bphi_s, bl, bn, d["spiky_grad"],
                                   *args)
        maxerr.append(dv.max())
    op, ov = rk.pci_integrate(ps, sv, fo, fp, kw["time_step"], 9.81, kw["max_vel"], sc["container"], *args)
    out.update(bphi=bphi, density=dens, normal=nrm, force_other=fo, pos_pred=pred, dens_var=dv, pressure=pres,
               force_pressure=fp, pci_maxerr=np.array(maxerr, np.float32), pos_out=op, vel_out=ov)
    return out, kw, d


def save(name, sc, out, kw, d):
    meta = {k: np.float64(v) for k, v in kw.items()}
    consts = {"c_" + k: np.float64(v) for k, v in d.items() if np.isscalar(v)}
    np.savez_compressed(os.path.join(HERE, name), fluid=sc["fluid"], boundary=sc["boundary"],
                        container=np.array(sc["container"], np.float32), **out,
                        **{"p_" + k: v for k, v in meta.items()}, **consts)
    print("wrote", name, os.path.getsize(os.path.join(HERE, name)), "bytes")


def render_fixture():
    """Screen-space surface of a seeded particle blob seen by the reference's default camera
    (fov 45, near 0.5, far 30: gui/glwidget.cpp:82-88; point size uniforms:
    fluid/render/sspacefluidrenderer.cpp:365-366).  The depth and normals images come from the
    restatement (the GLSL stages cannot run here); the smoothing filters from the
    reference's own OpenCL kernels compiled for the CPU."""
    w, h = 128, 96
    rng = np.random.default_rng(20250601)
    pos = np.zeros((2500, 4), np.float32)
    pos[:, :3] = rng.uniform(0.1, 0.9, (2500, 3))   # inside a container of side 1
    mv = orender.look_at([1.3, 1.5, 2.2], [0.5, 0.5, 0.5], [0.0, 1.0, 0.0])
    pr = orender.perspective(45.0, w / h, 0.5, 30.0)
    ipr = np.linalg.inv(pr.astype(np.float64)).astype(np.float32)
    radius, scale = 0.0625, w * np.tan(np.radians(22.5))
    depth = orender.splat_depth(pos, mv, pr, radius, scale, w, h)
    bil = rk.bilateral_filter(depth)
    smooth = depth
    for _ in range(2):
        smooth = rk.bilateral_filter(rk.bilateral_filter(smooth))
    curv = rk.curvature_flow(depth, ipr[0, 0], ipr[1, 1])
    nrm = orender.depth_normals(smooth, ipr)
    path = os.path.join(HERE, "render_small.npz")
    np.savez_compressed(path, pos=pos, modelview=mv, projection=pr, inv_projection=ipr,
                        point_radius=np.float32(radius), point_scale=np.float32(scale), width=w, height=h,
                        depth=depth, bilateral=bil, smooth2=smooth, curvature=curv, normals=nrm)
    print("wrote render_small.npz", os.path.getsize(path), "bytes; covered", float((depth != 0).mean()))


def mesh_fixture():
    """Model::surface_sampling of the reference's teapot (data/models/teapot.obj read by its
    own ModelMesh) at particle spacing 0.03: the voxelizer's output list, in its order."""
    from oracle.refkernels import REFERENCE_ROOT
    v, ix = rk.load_obj(os.path.join(REFERENCE_ROOT, "data", "models", "teapot.obj"))
    spacing = np.float32(0.03)
    out = rk.voxelize(v, ix, spacing, np.float32(spacing / np.float32(10)))
    path = os.path.join(HERE, "voxel_teapot.npz")
    np.savez_compressed(path, vertices=v, indices=ix, spacing=spacing, precision=np.float32(spacing / np.float32(10)),
                        out=out)
    print("wrote voxel_teapot.npz", os.path.getsize(path), "bytes;", len(out), "particles")


def main():
    if rk.build() is None:
        raise SystemExit("the reference kernels are not available here")
    if sys.argv[1:] == ["render"]:
        render_fixture()
        return
    if sys.argv[1:] == ["mesh"]:
        mesh_fixture()
        return
    render_fixture()
    mesh_fixture()
    sc = small_scene()
    out, kw, d = wcsph(sc)
    save("wcsph_compat_small.npz", sc, out, kw, d)
    out, kw, d = pcisph(sc)
    save("pcisph_compat_small.npz", sc, out, kw, d)


if __name__ == "__main__":
    main()
