"""One WCSPH step made of the reference's own OpenCL kernels, run on the host cores by the
CPU runtime of oracle/ref_shim (work-groups spread over the threads) -- TEST INFRASTRUCTURE
and the timed reference arm of bench.py.

The step follows WCSPHSimulation::simulate (fluid/simulation/wcsphsimluation.cpp:40-106)
launch for launch: compute_hashes, the clogs key sort (restated: the stable ascending sort
numpy provides, which is the permutation clogs produces), the clshuffle gathers,
compute_cell_intervals over the reference's 5 m grid (its table cleared every step), the
fluid and boundary neighbour lists, compute_density_pressure, compute_normals (with the
binding the code intends), compute_acceleration and predict_vel_n_pos.  Boundary particles
are static: their hashes, sort, intervals and Psi are computed once (Psi by the oracle's
restatement of compute_boundary_phi, pinned bit for bit to the kernel, whose O(n^2) loop over
a body is too slow for hundreds of thousands of wall particles).  The kernel constants are
the host-side derivation restated by the oracle.
"""
import numpy as np

from . import refkernels as rk
from .oracle import Oracle

GRID_SIZE = 5.0


def _f4(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, 4))


class RefWCSPH:
    def __init__(self, fluid4, boundary4, container, time_step, max_vel, k_viscosity, surface_tension,
                 gas_stiffness, rest_density=1000.0, gravity=9.81, particle_radius=None, support_radius=None):
        kw = dict(time_step=time_step, max_vel=max_vel, k_viscosity=k_viscosity, surface_tension=surface_tension,
                  gas_stiffness=gas_stiffness, rest_density=rest_density, gravity=gravity)
        if particle_radius is not None:
            kw["particle_radius"] = particle_radius
        if support_radius is not None:
            kw["support_radius"] = support_radius
        o = Oracle(method=0, mode=0, container=tuple(container), **kw)
        d = o.derived()
        self.d, self.kw, self.container = d, kw, tuple(float(c) for c in container)
        self.cps = int(d["grid_dims"][0])
        self.pos = _f4(fluid4)
        self.vel = np.zeros_like(self.pos)
        self.vhalf = np.zeros_like(self.pos)
        b = _f4(boundary4)
        o.add_boundary(b)
        o.set_fluid(self.pos[:1])
        o.stage("BOUNDARY_SYNC")
        bphi = np.ascontiguousarray(o.get("BPHI"), np.float32)
        bh, _ = rk.compute_hashes(b, GRID_SIZE, d["h"], self.cps)
        order = np.argsort(bh, kind="stable")
        self.bpos = _f4(b[order])
        self.bphi = np.ascontiguousarray(bphi[order])
        self.biv = rk.compute_cell_intervals(self.bpos, np.ascontiguousarray(bh[order]), GRID_SIZE, d["h"], self.cps)
        self.table = np.empty(2 * self.cps ** 3, np.int32)   # the fluid cell table, cleared each step
        self.sc9 = [d["poly6_eval"], d["poly6_grad"], d["poly6_grad"], 0, 0, d["visc_lapl"], 0, d["spiky_grad"], 0]

    def step(self):
        d, kw = self.d, self.kw
        hs, _ = rk.compute_hashes(self.pos, GRID_SIZE, d["h"], self.cps)
        order = np.argsort(hs, kind="stable")
        ps, vs, vhs = _f4(self.pos[order]), _f4(self.vel[order]), _f4(self.vhalf[order])
        iv = rk.compute_cell_intervals(ps, np.ascontiguousarray(hs[order]), GRID_SIZE, d["h"], self.cps, self.table)
        fl, fn = rk.compute_neigh_list(ps, ps, iv, GRID_SIZE, d["h"], d["h_def"], self.cps)
        bl, bn = rk.compute_neigh_list(ps, self.bpos, self.biv, GRID_SIZE, d["h"], d["h_def"], self.cps)
        dens, pres = rk.wc_density_pressure(ps, fl, fn, self.bpos, self.bphi, bl, bn, d["mass"], d["h"],
                                            kw["gas_stiffness"], kw["rest_density"], d["poly6_eval"], d["h_def"])
        nrm = rk.compute_normals(ps, dens, fl, fn, d["poly6_grad"], d["mass_def"], d["h_def"])
        acc = rk.wc_acceleration(ps, vs, nrm, dens, pres, fl, fn, self.bpos, self.bphi, bl, bn, kw["gravity"],
                                 d["mass"], d["h"], kw["k_viscosity"], kw["surface_tension"], kw["rest_density"],
                                 self.sc9, d["st_main"], d["st_term"], d["h_def"])
        self.pos, self.vel, self.vhalf = rk.wc_integrate(ps, vs, vhs, acc, kw["time_step"], kw["max_vel"],
                                                         self.container, d["h_def"])
