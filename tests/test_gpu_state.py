"""Checkpoint / resume (sph_save_state / sph_load_state): A steps, save, B more steps ends
bit-identical to a fresh context built from the same scene that loads the file and runs the
same B steps -- fluid state, ids and a dynamic body's pose; damaged or mismatched files are
refused.  The driver's --save / --resume give the same."""
import json
import subprocess

import numpy as np
import pytest

import fluids_gb300
from fluids_gb300 import capi
from fluids_gb300.scenes import BoxVolume, Cube, FishTank

pytestmark = pytest.mark.gpu


def build(method, nfluid_box=(0.2, 0.24, 0.16)):
    kw = dict(time_step=2e-4 if method == capi.SPH_WCSPH else 5e-4, max_vel=10.0, particle_radius=0.0075,
              support_radius=0.03, k_viscosity=0.01, surface_tension=0.001, rest_density=1000.0, gravity=9.81)
    if method == capi.SPH_WCSPH:
        kw["gas_stiffness"] = 57142.857
    else:
        kw.update(pcisph_min_iterations=3, pcisph_max_iterations=8, pcisph_error_ratio=0.01, relax_on_add=0)
    ctx = capi.Context(capi.make_params(method, mode=capi.SPH_MODE_PHYSICS, **kw))
    ctx.set_rect_limits(0.6, 0.6, 0.4)
    ctx.add_boundary(FishTank(0.6, 0.6, 0.4).surface_sampling(0.015))
    # resting on the fluid's surface (top at y = -0.05), so the fluid pushes it from the start
    cube = Cube(0.1, mass=0.3, position=(0.15, 0.005, 0.0))
    ctx.add_boundary(cube.surface_sampling(0.015), can_move=True, rot3x4=cube.rot3x4(), mass=cube.mass)
    ctx.set_body_dynamics(1, True, (6.0 / (0.3 * 0.01),) * 3, 0.05)
    ctx.add_volume(BoxVolume(nfluid_box, (0.15, -0.17, 0.0)).particles(0.0075))
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
    # the body moved: the checkpoint carried a pose the scene file does not have
    assert not np.array_equal(want_body[0][:, 3], np.array([0.15, 0.005, 0.0], np.float32))
    force, _ = b.body_forces(2)
    assert np.abs(force[1, :3]).max() > 0   # the fluid acted on the body


def test_mismatched_or_damaged_files_are_refused(gpu_lib, tmp_path):
    path = tmp_path / "state.bin"
    a = build(capi.SPH_WCSPH)
    a.simulate(2)
    a.save_state(str(path))
    other = build(capi.SPH_WCSPH, nfluid_box=(0.2, 0.24, 0.12))   # another particle count
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
