"""The library's host scene samplers against the reference's own sampler code, and the
reference arm's scene against the benchmark scene (CPU).

sph_scene_box_volume / _fishtank / _cube (fluids_gb300/csrc/sph_scene.cpp) restate
BoxVolume::particles (fluid/simulation/boxvolume.cpp:11-40), FishTank::surface_sampling
(scene/fishtank.cpp:108-141) and Cube::surface_sampling (scene/cube.cpp:136-171); the
reference's function text is compiled by oracle/build_ref.sh (oracle/ref_shim/ref_scene.cpp)
and both must produce the same particles bit for bit.  Runs where the reference's sources
were available to build oracle/_ref."""
import numpy as np
import pytest

from oracle import refkernels as rk

pytestmark = pytest.mark.skipif(not rk.available(), reason="reference sources not available here")


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


# the benchmark containers (2 x 1 x 1 m at the three spacings, the small test tank, two
# batched aspect ratios) and a few odd sizes whose float loops end close to the far wall
TANKS = [((2.0, 1.0, 1.0), 0.005), ((2.0, 1.0, 1.0), 0.0125), ((2.0, 1.0, 1.0), 0.015),
         ((0.5, 1.0, 0.4), 0.015), ((1.37, 1.0, 1.0), 0.015), ((2.9, 1.0, 1.0), 0.015),
         ((0.3, 0.7, 0.11), 0.01), ((1.0, 1.0, 1.0), 0.1)]
CUBES = [(0.3, 0.0125), (0.06, 0.015), (1.0, 0.05), (0.33, 0.011)]
BOXES = [((0.5, 1.0, 0.7), (0.7375, 0.0125, -0.1), 0.00625), ((0.5, 1.0, 0.7), (-0.7375, 0.0125, -0.1), 0.00625),
         ((0.64, 0.64, 0.64), (0.3, -0.2, 0.0), 0.0025), ((0.1, 0.23, 0.07), (0.0, 0.0, 0.0), 0.004)]


@pytest.mark.parametrize("size,spacing", TANKS)
def test_fishtank_sampler_is_the_references(size, spacing):
    from fluids_gb300.scenes import FishTank
    assert same_bits(FishTank(*size).surface_sampling(spacing), rk.scene_fishtank(*size, spacing))


@pytest.mark.parametrize("side,spacing", CUBES)
def test_cube_sampler_is_the_references(side, spacing):
    from fluids_gb300.scenes import Cube
    assert same_bits(Cube(side).surface_sampling(spacing), rk.scene_cube(side, spacing))


@pytest.mark.parametrize("size,center,radius", BOXES)
def test_box_volume_sampler_is_the_references(size, center, radius):
    from fluids_gb300.scenes import BoxVolume
    assert same_bits(BoxVolume(size, center).particles(radius), rk.scene_box_volume(size, center, radius))


def test_reference_arm_scene_is_the_benchmark_scene():
    """bench.py --impl reference steps oracle.refscene.double_dam_4m: the same 4,194,304
    fluid particles and 321,401 wall particles as the benchmark's workload."""
    from fluids_gb300 import workloads
    from oracle import refscene
    w = workloads.double_dam_4m()
    r = refscene.double_dam_4m()
    assert r["name"] == w["name"]
    assert same_bits(r["fluid"], w["fluid"])
    assert same_bits(r["walls"], w["bodies"][0][0])
    p = w["params"]
    for k, v in r["params"].items():
        assert np.float32(v) == np.float32(getattr(p, k)), k
