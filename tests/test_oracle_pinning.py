"""Pins the oracle against the reference's own OpenCL kernels compiled for the CPU
(oracle/ref_shim + oracle/build_ref.sh).  Each stage of the oracle's step is re-run through
the corresponding reference kernel on the oracle's inputs and must agree bit for bit.

Runs only where the reference is mounted (the shim library cannot be built elsewhere);
tests/golden/ carries fixtures generated from the same kernels for everywhere else."""
import numpy as np
import pytest

from oracle import Oracle
from oracle import refkernels as rk
from scenes_np import small_scene

pytestmark = pytest.mark.skipif(not rk.available(), reason="reference kernels not available here")


def f4(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, 4))


def c(a, dt=None):
    return np.ascontiguousarray(a if dt is None else np.asarray(a, dt))


def make(method, mode, **kw):
    sc = small_scene()
    o = Oracle(method=method, mode=mode, container=sc["container"], **kw)
    o.add_boundary(sc["boundary"])
    o.set_fluid(sc["fluid"])
    return o, sc


def grid_args(o):
    d = o.derived()
    return 5.0, d["h"], d["grid_dims"][0], d


def check_grid_stages(o):
    size, h, cps, d = grid_args(o)
    o.stage("BOUNDARY_SYNC")
    o.stage("HASHES")
    hs, mk = rk.compute_hashes(f4(o.get("POS")), size, h, cps)
    assert np.array_equal(hs, o.get("HASHES")) and np.array_equal(mk, o.get("MASK"))
    o.stage("SORT")
    o.stage("SHUFFLE")
    o.stage("CELL_INTERVALS")
    iv = rk.compute_cell_intervals(f4(o.get("POS_SORTED")), c(o.get("HASHES")), size, h, cps)
    assert np.array_equal(iv, o.get("CELL_INTERVALS"))
    o.stage("NEIGH_LIST")
    o.stage("SB_NEIGH_LIST")
    ps = f4(o.get("POS_SORTED"))
    fl, fn = rk.compute_neigh_list(ps, ps, iv, size, h, d["h_def"], cps)
    assert np.array_equal(fl, o.get("NEIGH_LIST")) and np.array_equal(fn, o.get("NEIGH_LEN"))
    bl, bn = rk.compute_neigh_list(ps, f4(o.get("BPOS_SORTED")), c(o.get("BCELL_INTERVALS")), size, h,
                                   d["h_def"], cps)
    assert np.array_equal(bl, o.get("SB_NEIGH_LIST")) and np.array_equal(bn, o.get("SB_NEIGH_LEN"))
    assert fn.mean() > 20 and bn.sum() > 0


def test_boundary_phi_and_sort_match_reference():
    o, sc = make(0, 0)
    d = o.derived()
    phi = rk.boundary_phi(f4(sc["boundary"]), 1000.0, d["boundary_eval"], 1.0, d["h_def"])
    assert np.array_equal(phi, o.get("BPHI"))
    size, h, cps, _ = grid_args(o)
    hs, mk = rk.compute_hashes(f4(o.get("BPOS")), size, h, cps)
    order = np.argsort(hs, kind="stable")
    assert np.array_equal(o.get("BHASHES"), hs[order]) and np.array_equal(o.get("BMASK"), order)


@pytest.mark.parametrize("steps", [3])
def test_wcsph_compat_stages_match_reference(steps):
    o, sc = make(0, 0)
    d = o.derived()
    lim = sc["container"]
    sc9 = [d["poly6_eval"], d["poly6_grad"], d["poly6_grad"], 0, 0, d["visc_lapl"], 0, d["spiky_grad"], 0]
    for _ in range(steps):
        check_grid_stages(o)
        ps, fl, fn = f4(o.get("POS_SORTED")), c(o.get("NEIGH_LIST")), c(o.get("NEIGH_LEN"))
        bp, bphi, bl, bn = f4(o.get("BPOS_SORTED")), c(o.get("BPHI_SORTED")), c(o.get("SB_NEIGH_LIST")), \
            c(o.get("SB_NEIGH_LEN"))
        o.stage("WC_DENSITY")
        dens, pres = rk.wc_density_pressure(ps, fl, fn, bp, bphi, bl, bn, d["mass"], d["h"], 57142.857, 1000.0,
                                            d["poly6_eval"], d["h_def"])
        assert np.array_equal(dens, o.get("DENSITY")) and np.array_equal(pres, o.get("PRESSURE"))
        # The kernel text gives negative densities (poly6 of r); feed physical densities and
        # pressures so the force branch of compute_acceleration is exercised too.
        phys_d = (1000.0 + 20.0 * np.sin(np.arange(len(ps)))).astype(np.float32)
        phys_p = (57142.857 * ((phys_d / 1000.0) ** 7 - 1)).clip(0).astype(np.float32)
        o.set("DENSITY", phys_d)
        o.set("PRESSURE", phys_p)
        o.stage("NORMALS")
        nrm = rk.compute_normals(ps, phys_d, fl, fn, d["poly6_grad"], d["mass_def"], d["h_def"])
        assert np.array_equal(nrm, f4(o.get("NORMAL")))
        o.stage("WC_ACCEL")
        acc = rk.wc_acceleration(ps, f4(o.get("VEL_SORTED")), nrm, phys_d, phys_p, fl, fn, bp, bphi, bl, bn,
                                 9.81, d["mass"], d["h"], 0.01, 0.001, 1000.0, sc9, d["st_main"], d["st_term"],
                                 d["h_def"])
        assert np.array_equal(acc, f4(o.get("ACCEL")))
        sv, svh = f4(o.get("VEL_SORTED")), f4(o.get("VEL_HALF_SORTED"))
        o.stage("BOUNDARY_FORCES")
        o.stage("WC_INTEGRATE")
        op, ov, ovh = rk.wc_integrate(ps, sv, svh, acc, 2e-4, 10.0, lim, d["h_def"])
        assert np.array_equal(op, f4(o.get("POS")))
        assert np.array_equal(ov, f4(o.get("VEL")))
        assert np.array_equal(ovh, f4(o.get("VEL_HALF")))


@pytest.mark.parametrize("mode", [0, 1])
def test_pcisph_stages_match_reference(mode):
    o, sc = make(1, mode, time_step=5e-4, max_vel=20.0, surface_tension=1.0, k_viscosity=0.01, pci_max_iter=3)
    d = o.derived()
    lim = sc["container"]
    size, h, cps, _ = grid_args(o)
    args = (d["h_def"], d["mass_def"], d["rest_density_def"])
    for _ in range(2):
        if mode == 0:
            check_grid_stages(o)
        else:
            # PHYSICS bins on the container-fitted grid (P7), which the reference kernels
            # cannot express; its float stages are checked on the oracle's own lists.
            for s in ("BOUNDARY_SYNC", "HASHES", "SORT", "SHUFFLE", "CELL_INTERVALS", "NEIGH_LIST",
                      "SB_NEIGH_LIST"):
                o.stage(s)
        ps, sv, fl, fn = f4(o.get("POS_SORTED")), f4(o.get("VEL_SORTED")), c(o.get("NEIGH_LIST")), \
            c(o.get("NEIGH_LEN"))
        bp, bphi, bl, bn = f4(o.get("BPOS_SORTED")), c(o.get("BPHI_SORTED")), c(o.get("SB_NEIGH_LIST")), \
            c(o.get("SB_NEIGH_LEN"))
        o.stage("PCI_INIT_DENSITY")
        dens = rk.pci_initial_density(ps, fl, fn, bp, bphi, bl, bn, d["default_eval"], *args)
        assert np.array_equal(dens, o.get("DENSITY"))
        assert 900 < np.median(dens) < 1300
        o.stage("NORMALS")
        nrm = rk.compute_normals(ps, dens, fl, fn, d["poly6_grad"], d["mass_def"], d["h_def"])
        assert np.array_equal(nrm, f4(o.get("NORMAL")))
        o.stage("PCI_INIT_FORCES")
        fo = rk.pci_initial_forces(ps, sv, dens, nrm, fl, fn, 0.01, 1.0, d["visc_lapl"], d["st_main"],
                                   d["st_term"], *args)
        assert np.array_equal(fo, f4(o.get("FORCE_OTHER")))
        o.stage("PCI_LOOP")
        if mode == 0:
            # the compat stop test always ends after the minimum iteration count
            assert o.get("PCI_ITERS")[0] == 3
        o.stage("BOUNDARY_FORCES")
        pres, fpress = c(o.get("PRESSURE")), f4(o.get("FORCE_PRESSURE"))
        o.stage("PCI_INTEGRATE")
        op, ov = rk.pci_integrate(ps, sv, fo, fpress, 5e-4, 9.81, 20.0, lim, *args)
        assert np.array_equal(op, f4(o.get("POS"))) and np.array_equal(ov, f4(o.get("VEL")))


def test_pcisph_loop_iteration_matches_reference():
    """The oracle's predict/update/force loop equals chaining the reference kernels."""
    o, sc = make(1, 0, time_step=5e-4, max_vel=20.0, surface_tension=1.0, pci_max_iter=3)
    d = o.derived()
    lim = sc["container"]
    size, h, cps, _ = grid_args(o)
    args = (d["h_def"], d["mass_def"], d["rest_density_def"])
    check_grid_stages(o)
    for s in ("PCI_INIT_DENSITY", "NORMALS", "PCI_INIT_FORCES"):
        o.stage(s)
    ps, sv, fl, fn = f4(o.get("POS_SORTED")), f4(o.get("VEL_SORTED")), c(o.get("NEIGH_LIST")), c(o.get("NEIGH_LEN"))
    bp, bphi, bl, bn = f4(o.get("BPOS_SORTED")), c(o.get("BPHI_SORTED")), c(o.get("SB_NEIGH_LIST")), \
        c(o.get("SB_NEIGH_LEN"))
    dens, fo = c(o.get("DENSITY")), f4(o.get("FORCE_OTHER"))
    fp = np.zeros_like(fo)
    pres = np.zeros(len(ps), np.float32)
    maxerr = []
    for _ in range(3):
        pred = rk.pci_predict_pos(ps, sv, fo, fp, 5e-4, 9.81, 20.0, lim, *args)
        dv, pres = rk.pci_update_pressure(pred, pres, d["pci_delta"], fl, fn, bp, bphi, bl, bn, d["default_eval"],
                                          *args)
        fp = rk.pci_pressure_force(ps, dens, pres, size, h, cps, fl, fn, bp, bphi, bl, bn, d["spiky_grad"], *args)
        maxerr.append(dv.max())
    o.stage("PCI_LOOP")
    assert np.array_equal(pred, f4(o.get("POS_PRED")))
    assert np.array_equal(dv, o.get("DENS_VAR"))
    assert np.array_equal(pres, o.get("PRESSURE"))
    assert np.array_equal(fp, f4(o.get("FORCE_PRESSURE")))
    assert np.array_equal(np.array(maxerr, np.float32), o.get("PCI_MAXERR"))


def test_boundary_transform_and_fluid_force_match_reference():
    sc = small_scene()
    th = 0.5
    rot = np.array([[np.cos(th), 0, np.sin(th), 0.01], [0, 1, 0, 0.0], [-np.sin(th), 0, np.cos(th), 0.0]],
                   np.float32)
    lin, ang = [0.1, 0.0, -0.2, 0.0], [0.3, 0.5, -0.1, 0.0]
    o = Oracle(method=1, mode=0, container=sc["container"], time_step=5e-4, max_vel=20.0, pci_max_iter=3)
    o.add_boundary(sc["boundary"], can_move=1, rot3x4=rot, lin=lin, ang=ang, mass=2.0)
    o.set_fluid(sc["fluid"])
    out, vel = rk.transform_particles(f4(sc["boundary"]), rot, lin, ang)
    assert np.array_equal(out, f4(o.get("BPOS")))
    o.step(1)
    d = o.derived()
    size, h, cps, _ = grid_args(o)
    force, torque = rk.fluid_force(f4(o.get("BPOS")), c(o.get("BPHI")), f4(o.get("POS_SORTED")),
                                   c(o.get("DENSITY")), c(o.get("PRESSURE")), c(o.get("CELL_INTERVALS")),
                                   d["mass"], np.float32(-45.0 / (np.pi * np.float32(d["h"]) ** 6)), size, h, cps,
                                   rot[:, 3], f4(o.get("VEL_SORTED")), vel, 0.0, d["h_def"])
    fsum = force.astype(np.float64).sum(0)[:3]
    tsum = torque.astype(np.float64).sum(0)[:3]
    of = o.get("BODY_FORCE")[:3].astype(np.float64)
    ot = o.get("BODY_TORQUE")[:3].astype(np.float64)
    assert np.linalg.norm(fsum) > 0
    assert np.allclose(of, fsum, rtol=1e-5, atol=1e-6 * np.abs(fsum).max())
    assert np.allclose(ot, tsum, rtol=1e-5, atol=1e-6 * np.abs(tsum).max())


# ---- the Monaghan kernels (kernels/monaghan_kernels.h:7-47): the oracle with kernels = 1
# against the reference's kernel files built without USE_MULLER_KERNELS

def test_monaghan_boundary_phi_matches_reference():
    o, sc = make(0, 0, kernels=1)
    d = o.derived()
    with rk.monaghan():
        phi = rk.boundary_phi(f4(sc["boundary"]), 1000.0, d["boundary_eval"], 1.0, d["h_def"])
    assert np.array_equal(phi, o.get("BPHI"))
    o0, _ = make(0, 0)
    assert not np.array_equal(phi, o0.get("BPHI"))   # the kernel family matters


def test_monaghan_wcsph_density_and_normals_match_reference():
    o, sc = make(0, 0, kernels=1)
    d = o.derived()
    check_grid_stages(o)
    ps, fl, fn = f4(o.get("POS_SORTED")), c(o.get("NEIGH_LIST")), c(o.get("NEIGH_LEN"))
    bp, bphi, bl, bn = f4(o.get("BPOS_SORTED")), c(o.get("BPHI_SORTED")), c(o.get("SB_NEIGH_LIST")), \
        c(o.get("SB_NEIGH_LEN"))
    o.stage("WC_DENSITY")
    with rk.monaghan():
        dens, pres = rk.wc_density_pressure(ps, fl, fn, bp, bphi, bl, bn, d["mass"], d["h"], 57142.857, 1000.0,
                                            d["poly6_eval"], d["h_def"])
    assert np.array_equal(dens, o.get("DENSITY")) and np.array_equal(pres, o.get("PRESSURE"))
    phys_d = (1000.0 + 20.0 * np.sin(np.arange(len(ps)))).astype(np.float32)
    o.set("DENSITY", phys_d)
    o.stage("NORMALS")
    with rk.monaghan():
        nrm = rk.compute_normals(ps, phys_d, fl, fn, d["poly6_grad"], d["mass_def"], d["h_def"])
    assert np.array_equal(nrm[:, :3], f4(o.get("NORMAL"))[:, :3])


def test_monaghan_pcisph_stages_match_reference():
    o, sc = make(1, 0, time_step=5e-4, max_vel=20.0, surface_tension=1.0, k_viscosity=0.01, pci_max_iter=3,
                 kernels=1)
    d = o.derived()
    size, h, cps, _ = grid_args(o)
    args = (d["h_def"], d["mass_def"], d["rest_density_def"])
    check_grid_stages(o)
    ps, sv, fl, fn = f4(o.get("POS_SORTED")), f4(o.get("VEL_SORTED")), c(o.get("NEIGH_LIST")), c(o.get("NEIGH_LEN"))
    bp, bphi, bl, bn = f4(o.get("BPOS_SORTED")), c(o.get("BPHI_SORTED")), c(o.get("SB_NEIGH_LIST")), \
        c(o.get("SB_NEIGH_LEN"))
    with rk.monaghan():
        o.stage("PCI_INIT_DENSITY")
        dens = rk.pci_initial_density(ps, fl, fn, bp, bphi, bl, bn, d["default_eval"], *args)
        assert np.array_equal(dens, o.get("DENSITY"))
        o.stage("NORMALS")
        nrm = rk.compute_normals(ps, dens, fl, fn, d["poly6_grad"], d["mass_def"], d["h_def"])
        assert np.array_equal(nrm[:, :3], f4(o.get("NORMAL"))[:, :3])
        # the oracle's normals carry w = 0; the kernel text's Monaghan gradient puts
        # -0.75 r / h^2 into w as well, which no later pass reads
        o.set("NORMAL", nrm)
        o.stage("PCI_INIT_FORCES")
        fo = rk.pci_initial_forces(ps, sv, dens, nrm, fl, fn, 0.01, 1.0, d["visc_lapl"], d["st_main"],
                                   d["st_term"], *args)
        assert np.array_equal(fo[:, :3], f4(o.get("FORCE_OTHER"))[:, :3])
        # one loop iteration's passes on the oracle's inputs
        o.set("FORCE_OTHER", fo)
        lim = sc["container"]
        fp = np.zeros_like(fo)
        o.set("FORCE_PRESSURE", fp)
        o.stage("PCI_PREDICT")
        pred = rk.pci_predict_pos(ps, sv, fo, fp, 5e-4, 9.81, 20.0, lim, *args)
        assert np.array_equal(pred[:, :3], f4(o.get("POS_PRED"))[:, :3])
        pres0 = (50.0 * (1.0 + np.cos(np.arange(len(ps))))).astype(np.float32)
        o.set("PRESSURE", pres0)
        o.stage("PCI_UPDATE_PRESSURE")
        dv, pres = rk.pci_update_pressure(pred, pres0.copy(), d["pci_delta"], fl, fn, bp, bphi, bl, bn,
                                          d["default_eval"], *args)
        assert np.array_equal(dv, o.get("DENS_VAR")) and np.array_equal(pres, o.get("PRESSURE"))
        o.stage("PCI_PRESSURE_FORCE")
        fpr = rk.pci_pressure_force(ps, dens, pres, size, h, cps, fl, fn, bp, bphi, bl, bn, d["spiky_grad"], *args)
        assert np.array_equal(fpr[:, :3], f4(o.get("FORCE_PRESSURE"))[:, :3])
