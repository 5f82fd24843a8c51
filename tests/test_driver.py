"""The C++ host mirror (include/sph_fluid.hpp) and the headless driver built on it: settings
files in the reference's key=value format, scene files in its JSON format, and on the GPU
the same result as the Python API on the same scene."""
import json
import os
import subprocess

import numpy as np
import pytest

import fluids_gb300
from fluids_gb300 import capi
from fluids_gb300 import scenes
from fluids_gb300.scenes import BoxVolume, Cube, FishTank, Sphere

CONFIG = """# Simulation settings
time_step=0.0002
max_vel=10.0
fluid_particle_radius=0.0075
fluid_support_radius=0.03
pcisph_max_iterations=3
pcisph_error_ratio=0.01
method=wcsph

# Physics settings
rest_density=1000
k_viscosity=0.01
gravity=9.81
gas_stiffness=57142.857
surface_tension=0.001
"""

SCENE = {"container": {"width": 0.6, "height": 0.6, "depth": 0.4},
         "fluid_volumes": [{"type": "box", "name": "fluid_1", "size": [0.24, 0.3, 0.2], "center": [0.15, -0.14, 0.0]}],
         "rigid_bodies": [{"type": "cube", "name": "cube_1", "mass": 0.0, "size": 0.1, "center": [-0.15, -0.24, 0.0],
                           "rotation": [0, 0, 0, 1]},
                          {"type": "sphere", "name": "ball", "mass": 0.0, "size": 0.05, "center": [0, 0, 0]}]}


@pytest.fixture(scope="module")
def driver():
    return fluids_gb300.build_driver()


def write(tmp_path, config=CONFIG, scene=SCENE):
    c = tmp_path / "config.wc"
    c.write_text(config)
    s = tmp_path / "scene.json"
    s.write_text(json.dumps(scene))
    return str(c), str(s)


def test_driver_parses_reference_formats(driver, tmp_path):
    c, s = write(tmp_path)
    r = subprocess.run([driver, "--config", c, "--scene", s, "--dry-run", "--container-boundary"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout)
    n = len(BoxVolume((0.24, 0.3, 0.2), (0.15, -0.14, 0.0)).particles(0.0075))
    nb = (len(FishTank(0.6, 0.6, 0.4).surface_sampling(0.015)) + len(Cube(0.1).surface_sampling(0.015)) +
          len(Sphere(0.05).surface_sampling(0.015)))
    assert out["particles"] == n and out["boundary_particles"] == nb
    assert out["method"] == "wcsph" and out["bodies"] == 3 and out["device_sampled_bodies"] == 0


def test_driver_checks_render_method(driver, tmp_path):
    """render_method is particles or screenspace (settings/settings.cpp:47-57)."""
    for val, rc in (("particles", 0), ("screenspace", 0), ("raytraced", 1)):
        c, s = write(tmp_path, config=CONFIG + "render_method=%s\n" % val)
        r = subprocess.run([driver, "--config", c, "--scene", s, "--dry-run"], capture_output=True, text=True)
        assert r.returncode == rc, (val, r.stderr)


def test_driver_rejects_incomplete_settings(driver, tmp_path):
    c, s = write(tmp_path, config=CONFIG.replace("gas_stiffness=57142.857\n", ""))
    r = subprocess.run([driver, "--config", c, "--scene", s, "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 1 and "gas_stiffness" in r.stderr
    c, s = write(tmp_path, config=CONFIG.replace("method=wcsph", "method=flip"))
    r = subprocess.run([driver, "--config", c, "--scene", s, "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 1 and "flip" in r.stderr


@pytest.mark.gpu
def test_driver_matches_python_api(gpu_lib, driver, tmp_path):
    c, s = write(tmp_path)
    dump = str(tmp_path / "pos.bin")
    steps = 30
    r = subprocess.run([driver, "--config", c, "--scene", s, "--steps", str(steps), "--every", "10",
                        "--container-boundary", "--dump", dump], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines()]
    assert [x["step"] for x in lines[:-1]] == [10, 20, 30] and lines[-1]["done"] == steps
    got = np.fromfile(dump, np.float32).reshape(-1, 4)
    # the driver runs PHYSICS mode unless --mode compat (the C ABI's default is COMPAT)
    p = capi.make_params(capi.SPH_WCSPH, mode=capi.SPH_MODE_PHYSICS, time_step=2e-4, max_vel=10.0, particle_radius=0.0075,
                         support_radius=0.03, pcisph_max_iterations=3, pcisph_error_ratio=0.01, rest_density=1000.0,
                         k_viscosity=0.01, gravity=9.81, gas_stiffness=57142.857, surface_tension=0.001)
    ctx = capi.Context(p)
    ctx.set_rect_limits(0.6, 0.6, 0.4)
    ctx.add_boundary(FishTank(0.6, 0.6, 0.4).surface_sampling(0.015))
    cube = Cube(0.1, position=(-0.15, -0.24, 0.0))
    ctx.add_boundary(cube.surface_sampling(0.015), rot3x4=cube.rot3x4())
    ball = Sphere(0.05)
    ctx.add_boundary(ball.surface_sampling(0.015), rot3x4=ball.rot3x4())
    ctx.add_volume(BoxVolume((0.24, 0.3, 0.2), (0.15, -0.14, 0.0)).particles(0.0075))
    ctx.simulate(steps)
    ctx.synchronize()
    pos = ctx.get("POS").reshape(-1, 4)
    ids = ctx.get("ID")
    ref = np.empty_like(pos)
    ref[ids] = pos
    assert np.array_equal(got, ref)
    st = ctx.stats()
    assert lines[-2]["kinetic"] == pytest.approx(st["kinetic"], rel=1e-8)   # printed with 9 digits


@pytest.mark.gpu
def test_driver_moves_bodies_with_mass(gpu_lib, driver, tmp_path):
    """A cube with mass in the scene file is dynamic: it falls under gravity (no fluid near)."""
    scene = {"container": {"width": 0.6, "height": 0.6, "depth": 0.4},
             "fluid_volumes": [{"type": "box", "name": "f", "size": [0.12, 0.12, 0.12], "center": [0.2, -0.2, 0.0]}],
             "rigid_bodies": [{"type": "cube", "name": "falling", "mass": 0.4, "size": 0.1,
                               "center": [-0.15, 0.1, 0.0], "rotation": [0, 0, 0, 1]}]}
    c, s = write(tmp_path, scene=scene)
    r = subprocess.run([driver, "--config", c, "--scene", s, "--steps", "100", "--every", "50"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines()]
    y = [x["bodies"]["falling"][1] for x in lines[:-1]]
    dt, g = np.float32(2e-4), 9.81
    for n, yy in zip((50, 100), y):
        assert yy == pytest.approx(0.1 - g * dt * dt * n * (n + 1) / 2, abs=1e-5)


CUBE_OBJ = """# a closed cube of side 0.1 centred at the origin
v -0.05 -0.05 -0.05
v 0.05 -0.05 -0.05
v 0.05 0.05 -0.05
v -0.05 0.05 -0.05
v -0.05 -0.05 0.05
v 0.05 -0.05 0.05
v 0.05 0.05 0.05
v -0.05 0.05 0.05
f 1 3 2
f 1 4 3
f 5 6 7
f 5 7 8
f 1 2 6
f 1 6 5
f 4 8 7
f 4 7 3
f 1 5 8
f 1 8 4
f 2 3 7
f 2 7 6
"""


def model_scene(tmp_path, mass):
    (tmp_path / "models").mkdir(exist_ok=True)
    (tmp_path / "models" / "box.obj").write_text(CUBE_OBJ)
    return {"container": {"width": 0.6, "height": 0.6, "depth": 0.4},
            "fluid_volumes": [{"type": "box", "name": "f", "size": [0.12, 0.12, 0.12], "center": [0.2, -0.2, 0.0]}],
            "rigid_bodies": [{"type": "model", "name": "box", "obj_filename": "models/box.obj", "mass": mass,
                              "center": [-0.15, 0.1, 0.0], "rotation": [0, 1, 0, 0.5]}]}


def test_driver_samples_wall_bodies(driver, tmp_path):
    scene = dict(SCENE)
    scene["rigid_bodies"] = [{"type": "wall", "name": "w", "mass": 0.0, "size": [0.3, 0.2],
                              "center": [0.0, 0.0, 0.1], "rotation": [0, 0, 0, 1]}]
    c, s = write(tmp_path, scene=scene)
    r = subprocess.run([driver, "--config", c, "--scene", s, "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    from fluids_gb300.scenes import Wall
    assert json.loads(r.stdout)["boundary_particles"] == len(Wall(0.3, 0.2).surface_sampling(0.015))


def test_driver_reads_model_bodies(driver, tmp_path):
    """A "model" body is read from its OBJ file (found under --data-root); its voxel
    sampling runs on the GPU, so a dry run reports it without sampling it."""
    c, s = write(tmp_path, scene=model_scene(tmp_path, 0.0))
    r = subprocess.run([driver, "--config", c, "--scene", s, "--dry-run", "--data-root", str(tmp_path)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout)
    assert out["bodies"] == 1 and out["device_sampled_bodies"] == 1 and out["boundary_particles"] == 0
    r = subprocess.run([driver, "--config", c, "--scene", s, "--dry-run", "--data-root", str(tmp_path / "none")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "models/box.obj" in r.stderr


@pytest.mark.gpu
def test_driver_runs_model_scene(gpu_lib, driver, tmp_path):
    """The voxel-sampled model with mass falls freely as a dynamic body."""
    c, s = write(tmp_path, scene=model_scene(tmp_path, 0.5))
    r = subprocess.run([driver, "--config", c, "--scene", s, "--steps", "100", "--every", "50",
                        "--data-root", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines()]
    v, ix = scenes.load_obj(str(tmp_path / "models" / "box.obj"))
    assert lines[-1]["boundary_particles"] == len(scenes.voxelize(v, ix, 0.015, 0.0015))
    y = [x["bodies"]["box"][1] for x in lines[:-1]]
    dt, g = np.float32(2e-4), 9.81
    for n, yy in zip((50, 100), y):
        assert yy == pytest.approx(0.1 - g * dt * dt * n * (n + 1) / 2, abs=1e-5)
    assert lines[-1]["flags"] == 0


@pytest.mark.gpu
def test_driver_reference_short_options_and_fps_output(gpu_lib, driver, tmp_path):
    """-c / -s / -o as the reference's main.cpp takes them; -o writes one FPS value per 6
    steps."""
    c, s = write(tmp_path)
    out = tmp_path / "fps.txt"
    r = subprocess.run([driver, "-c", c, "-s", s, "-o", str(out), "--steps", "18"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vals = [float(x) for x in out.read_text().split()]
    assert len(vals) == 3 and all(v > 0 for v in vals)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["screenspace", "particles"])
def test_driver_writes_frames(gpu_lib, driver, tmp_path, method):
    scene = dict(SCENE)
    scene["lights"] = [{"ambient_color": [100, 100, 100], "diffuse_color": [255, 255, 255],
                        "specular_color": [255, 255, 255], "direction": [-1.0, -1.0, -1.0]}]
    c, s = write(tmp_path, config=CONFIG + "render_method=%s\n" % method, scene=scene)
    frames = tmp_path / "frames"
    frames.mkdir()
    r = subprocess.run([driver, "-c", c, "-s", s, "--steps", "20", "--frames", str(frames), "--frame-every", "10",
                        "--frame-size", "160x90"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    files = sorted(frames.iterdir())
    assert [f.name for f in files] == ["frame_00000.ppm", "frame_00001.ppm"]
    raw = files[-1].read_bytes()
    assert raw.startswith(b"P6\n160 90\n255\n") and len(raw) == len(b"P6\n160 90\n255\n") + 160 * 90 * 3
    img = np.frombuffer(raw[len(b"P6\n160 90\n255\n"):], np.uint8)
    assert img.max() > 0    # the fluid is in view of the default camera
