"""Helpers shared by the parity tests: build the same scene in the CUDA context and in the
oracle, and compare fields."""
import numpy as np

from oracle import Oracle, kwargs_from_params
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
    return kwargs_from_params(params, container)


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


def tait(density, params):
    """compute_density_pressure's equation of state (kernels/wcsph.cl:32-79) in FP32 with
    pown as left-to-right multiplication: p = max(0, k ((rho / rho0)^7 - 1))."""
    with np.errstate(over="ignore", invalid="ignore"):
        q = np.asarray(density, np.float32) / np.float32(params.rest_density)
        pw = q.copy()
        for _ in range(6):
            pw = pw * q
        return np.maximum(np.float32(0), np.float32(params.gas_stiffness) * (pw - np.float32(1)))
