"""Checkpoint / resume (sph_save_state / sph_load_state): A steps, save, B more steps ends
bit-identical to a fresh context built from the same scene that loads the file and runs the
same B steps -- fluid state, ids and a dynamic body's pose; damaged or mismatched files are
refused.  The driver's --save / --resume give the same."""
import json
import subprocess

import numpy as np
import pytest

import fluids_gb300
from fluids_gb300 import capi, workloads
from fluids_gb300.scenes import Cube
from scenes_np import jittered_block

pytestmark = pytest.mark.gpu


DX = 0.015


def build(method, nz=12):
    """A light cube submerged in a fluid block (the fluid inside it removed) over a floor:
    the fluid's pressure pushes the dynamic cube from the first step."""
    if method == capi.SPH_WCSPH:
        p = workloads.wcsph_params(DX, 2e-4, capi.SPH_MODE_PHYSICS, sigma=0.0)
    else:
        p = capi.make_params(capi.SPH_PCISPH, mode=capi.SPH_MODE_PHYSICS, time_step=5e-4, max_vel=10.0,
                             particle_radius=DX / 2, support_radius=2 * DX, k_viscosity=0.01, surface_tension=0.0,
                             pcisph_min_iterations=3, pcisph_max_iterations=8, pcisph_error_ratio=0.01,
                             relax_on_add=0)
    fluid = jittered_block(14, 16, nz, DX, (-0.1, -0.5 + DX, -0.08), seed=2)
    side, mass = 0.06, 0.1
    center = np.array([0.0, -0.5 + DX + 7 * DX, 0.0], np.float32)
    inside = np.all(np.abs(fluid[:, :3] - center) < side / 2 + DX / 2, axis=1)
    fluid = np.ascontiguousarray(fluid[~inside])
    cube = Cube(side, mass=mass, position=tuple(center))
    floor = np.array([[x, -0.5, z, 1.0] for x in np.arange(-0.25, 0.26, DX) for z in np.arange(-0.2, 0.21, DX)],
                     np.float32)
    ctx = capi.Context(p)
    ctx.set_rect_limits(0.5, 1.0, 0.4)
    ctx.add_boundary(floor)
    ctx.add_boundary(cube.surface_sampling(DX), can_move=True, rot3x4=cube.rot3x4(), mass=mass)
    ctx.add_volume(fluid)
    ctx.set_body_dynamics(1, True, [6.0 / (mass * side * side)] * 3, side / 2)
    return ctx


def state(ctx):
    return {f: ctx.get(f) for f in ("POS", "VEL", "VEL_HALF", "ID")}, ctx.body_state(1)


@pytest.mark.parametrize("method", [capi.SPH_WCSPH, capi.SPH_PCISPH])
def test_resume_is_bit_identical(gpu_lib, tmp_path, method):
    path = str(tmp_path / "state.bin")
    a = build(method)
    a.simulate(15)
    a.save_state(path)
    a.simulate(10)
    want, want_body = state(a)
    b = build(method)
    b.load_state(path)
    b.simulate(10)
    got, got_body = state(b)
    for f in want:
        assert np.array_equal(got[f], want[f]), f
    for g, w in zip(got_body, want_body):
        assert np.array_equal(g, w)
    force, _ = b.body_forces(2)
    assert np.abs(force[1, :3]).max() > 0   # the fluid acted on the body


def test_mismatched_or_damaged_files_are_refused(gpu_lib, tmp_path):
    path = tmp_path / "state.bin"
    a = build(capi.SPH_WCSPH)
    a.simulate(2)
    a.save_state(str(path))
    other = build(capi.SPH_WCSPH, nz=10)   # another particle count
    with pytest.raises(capi.SphError, match="counts differ"):
        other.load_state(str(path))
    pci = build(capi.SPH_PCISPH)
    with pytest.raises(capi.SphError, match="parameters differ"):
        pci.load_state(str(path))
    raw = bytearray(path.read_bytes())
    raw[len(raw) // 2] ^= 1
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(raw))
    with pytest.raises(capi.SphError, match="checksum"):
        build(capi.SPH_WCSPH).load_state(str(bad))
    with pytest.raises(capi.SphError):
        build(capi.SPH_WCSPH).load_state(str(tmp_path / "missing.bin"))


CONFIG = """time_step=0.0002
max_vel=10.0
fluid_particle_radius=0.0075
fluid_support_radius=0.03
pcisph_max_iterations=3
pcisph_error_ratio=0.01
method=wcsph
rest_density=1000
k_viscosity=0.01
gravity=9.81
gas_stiffness=57142.857
surface_tension=0.001
"""

SCENE = {"container": {"width": 0.6, "height": 0.6, "depth": 0.4},
         "fluid_volumes": [{"type": "box", "name": "f", "size": [0.2, 0.24, 0.16], "center": [0.15, -0.17, 0.0]}],
         "rigid_bodies": [{"type": "cube", "name": "c", "mass": 0.3, "size": 0.1, "center": [-0.12, -0.1, 0.0],
                           "rotation": [0, 0, 0, 1]}]}


def test_driver_save_and_resume(gpu_lib, tmp_path):
    driver = fluids_gb300.build_driver()
    (tmp_path / "c.wc").write_text(CONFIG)
    (tmp_path / "s.json").write_text(json.dumps(SCENE))
    base = [driver, "--config", str(tmp_path / "c.wc"), "--scene", str(tmp_path / "s.json"), "--container-boundary"]

    def run(*extra):
        r = subprocess.run(base + list(extra), capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        return r

    run("--steps", "30", "--dump", str(tmp_path / "full.bin"))
    run("--steps", "20", "--save", str(tmp_path / "ck.bin"))
    run("--steps", "10", "--resume", str(tmp_path / "ck.bin"), "--dump", str(tmp_path / "resumed.bin"))
    full = np.fromfile(tmp_path / "full.bin", np.float32)
    resumed = np.fromfile(tmp_path / "resumed.bin", np.float32)
    assert full.size > 0 and np.array_equal(full, resumed)
