"""Helpers shared by the parity tests: build the same scene in the CUDA context and in the
oracle, and compare fields."""
import numpy as np

from oracle import Oracle
from fluids_gb300 import capi

# FP32 tolerance of the parity bar: max over particles of |a_i - b_i| (norm-wise for
# vectors) relative to the largest |b_i| of the field.
RTOL = 1e-5


def field_relerr(a, b, width=1):
    a = np.asarray(a, np.float64).reshape(-1, width)
    b = np.asarray(b, np.float64).reshape(-1, width)
    if width == 4:
        a, b = a[:, :3], b[:, :3]
    num = np.linalg.norm(a - b, axis=1).max() if len(a) else 0.0
    den = np.linalg.norm(b, axis=1).max() if len(b) else 0.0
    return num / den if den > 0 else num


def assert_close(name, a, b, width=1, rtol=RTOL):
    e = field_relerr(a, b, width)
    assert np.all(np.isfinite(np.asarray(a, np.float64))), "%s: non-finite values" % name
    assert e <= rtol, "%s: field-relative error %.3g > %.1g" % (name, e, rtol)
    return e


def oracle_config(params, container):
    """OrcConfig keywords equal to a capi.SphParams."""
    p = params
    return dict(method=p.method, mode=p.mode, container=container, neigh_cap=p.neigh_cap, time_step=p.time_step,
                max_vel=p.max_vel, particle_radius=p.particle_radius, support_radius=p.support_radius,
                pci_min_iter=p.pcisph_min_iterations, pci_max_iter=p.pcisph_max_iterations,
                pci_error_ratio=p.pcisph_error_ratio, pci_relax_max_iter=p.pcisph_relax_max_iterations,
                rest_density=p.rest_density, k_viscosity=p.k_viscosity, gravity=p.gravity,
                gas_stiffness=p.gas_stiffness, surface_tension=p.surface_tension, grid_size=p.grid_size,
                grid_margin=p.grid_margin, phi_coeff=p.boundary_phi_coeff, relax_on_add=p.relax_on_add)


def make_pair(params, fluid, bodies, container, precision=0, vel=None):
    """(CUDA context, oracle) loaded identically: limits, boundaries, fluid."""
    ctx = capi.Context(params)
    ctx.set_rect_limits(*container)
    orc = Oracle(precision=precision, **oracle_config(params, container))
    for pts, rot, mv, mass in bodies:
        ctx.add_boundary(pts, can_move=mv, rot3x4=rot, mass=mass)
        orc.add_boundary(pts, can_move=mv, rot3x4=rot, mass=mass)
    ctx.add_volume(fluid, vel)
    orc.set_fluid(fluid, vel)
    return ctx, orc
