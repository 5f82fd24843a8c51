"""CPU tests of the C-ABI library's host logic (no GPU): exported symbols, constant and grid
derivation against the oracle, the scene samplers and the seeded jitter."""
import os
import re

import numpy as np
import pytest

import fluids_gb300
from fluids_gb300 import capi, scenes, workloads
from oracle import Oracle, kwargs_from_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    fluids_gb300.build()


def header_functions():
    src = open(os.path.join(ROOT, "include", "sph_capi.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sph_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    names = header_functions()
    assert len(names) >= 25
    L = capi.lib()
    for n in names:
        assert hasattr(L, n), n
    assert sorted(capi.EXPORTS) == names


CASES = [
    (capi.SPH_WCSPH, capi.SPH_MODE_COMPAT, dict(particle_radius=0.0075, support_radius=0.03), (2, 1, 1)),
    (capi.SPH_WCSPH, capi.SPH_MODE_PHYSICS, dict(particle_radius=0.0075, support_radius=0.03), (2, 1, 1)),
    (capi.SPH_WCSPH, capi.SPH_MODE_PHYSICS, dict(particle_radius=0.0025, support_radius=0.01), (2, 1, 1)),
    (capi.SPH_PCISPH, capi.SPH_MODE_COMPAT, dict(particle_radius=0.00625, support_radius=0.025, time_step=5e-4),
     (2, 1, 1)),
    (capi.SPH_PCISPH, capi.SPH_MODE_PHYSICS, dict(particle_radius=0.00625, support_radius=0.025, time_step=5e-4),
     (2, 1, 1)),
    (capi.SPH_PCISPH, capi.SPH_MODE_COMPAT, {}, (1.5, 1.0, 0.8)),   # config.pci defaults
]


@pytest.mark.parametrize("method,mode,kw,container", CASES)
def test_constants_match_oracle(method, mode, kw, container):
    p = capi.make_params(method, mode=mode, **kw)
    mine = capi.describe(p, container)
    o = Oracle(**kwargs_from_params(p, container))
    ref = o.derived()
    for k in ("mass", "mass_def", "h", "h_def", "rest_density_def", "poly6_eval", "poly6_grad", "spiky_grad",
              "visc_lapl", "st_main", "st_term", "default_eval", "boundary_eval", "pci_delta", "grid_origin",
              "grid_dims", "grid_wrap", "key_bits"):
        assert mine[k] == ref[k], (k, mine[k], ref[k])


def test_compat_grid_is_the_reference_cube():
    d = capi.describe(capi.make_params(capi.SPH_WCSPH, support_radius=0.03), (2, 1, 1))
    assert d["grid_dims"] == [167, 167, 167] and d["grid_wrap"] == 1 and d["grid_origin"] == [-2.5] * 3
    d = capi.describe(capi.make_params(capi.SPH_WCSPH, mode=1, particle_radius=0.0025, support_radius=0.01),
                      (2, 1, 1))
    assert d["grid_dims"] == [204, 104, 104] and d["key_bits"] == 24


def test_pcisph_mass_rounding_and_365_constant():
    """COMPAT PCISPH: mass rho0 dx^3 / 1.15 and its 6-decimal -D rounding; 365/(64 pi h^9)."""
    d = capi.describe(capi.make_params(capi.SPH_PCISPH, particle_radius=0.00625, support_radius=0.025), (2, 1, 1))
    m = 1000.0 * 0.0125 ** 3 / 1.15
    assert abs(d["mass"] - m) / m < 1e-6
    assert d["mass_def"] == np.float32(float("%.6f" % d["mass"]))
    assert abs(d["default_eval"] / (365.0 / (64 * np.pi * 0.025 ** 9)) - 1) < 1e-6
    p = capi.describe(capi.make_params(capi.SPH_PCISPH, mode=1, particle_radius=0.00625, support_radius=0.025),
                      (2, 1, 1))
    assert abs(p["default_eval"] / (315.0 / (64 * np.pi * 0.025 ** 9)) - 1) < 1e-6
    assert p["pci_delta"] > 0


def box_volume_np(size, center, r):
    """boxvolume.cpp:11-40 with its float/double arithmetic."""
    sp = np.float32(2 * np.float32(r))
    n = [int(np.ceil(np.float32(s) / sp)) for s in size]
    d = [np.float32(np.float32(s) / np.float32(k)) for s, k in zip(size, n)]
    out = []
    for j in range(n[1]):
        for i in range(n[0]):
            for k in range(n[2]):
                xyz = []
                for a, idx in ((0, i), (1, j), (2, k)):
                    t = np.float32(np.float32(idx * d[a]) + np.float32(center[a]))
                    xyz.append(np.float32(np.float64(t) - np.float64(np.float32(size[a])) / 2.0))
                out.append(xyz + [1.0])
    return np.array(out, np.float32)


def test_box_volume_matches_restatement():
    got = scenes.BoxVolume((0.5, 0.3, 0.2), (0.74, 0.0125, -0.1)).particles(0.00625)
    exp = box_volume_np((0.5, 0.3, 0.2), (0.74, 0.0125, -0.1), 0.00625)
    assert got.shape == exp.shape == (40 * 24 * 16, 4)
    assert np.array_equal(got, exp)


def test_pcisph_scene_particle_count():
    w = workloads.pcisph_cube()
    assert len(w["fluid"]) == 2 * 40 * 80 * 56 == 358400


def test_fishtank_and_cube_sampling():
    t = scenes.FishTank(2.0, 1.0, 1.0).surface_sampling(0.015)
    assert t.shape[1] == 4 and np.all(t[:, 3] == 1)
    assert np.isclose(t[:, 1].min(), -0.5) and t[:, 1].max() <= 0.5
    assert np.all(np.abs(t[:, 0]) <= 1.0 + 1e-6) and np.all(np.abs(t[:, 2]) <= 0.5 + 1e-6)
    # base: every (x, z) of the float loops; walls on x = +-1 and z = +-0.5
    nx = len(np.arange(-1.0, 1.0 + 1e-9, 0.015))
    assert np.sum(t[:, 1] == np.float32(-0.5)) >= nx
    c = scenes.Cube(0.3).surface_sampling(0.0125)
    half = (0.3 - 0.0125) / 2
    on_face = np.isclose(np.abs(c[:, :3]), half, atol=1e-6).any(axis=1)
    assert on_face.all()
    # scene/cube.cpp:136-171 loops: 24 x-values, 24 z-values, 23 wall rows; base and top,
    # then four walls per row -- edge particles appear twice, as in the reference
    assert len(c) == 24 * 24 * 2 + 23 * (2 * 24 + 2 * 24) == 3360


def test_jitter_is_seeded_and_bounded():
    p = scenes.lattice_block(4, 5, 6, 0.01, (0, 0, 0))
    a = scenes.jitter(p, 1e-4, 7)
    b = scenes.jitter(p, 1e-4, 7)
    c = scenes.jitter(p, 1e-4, 8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    d = (a - p)[:, :3]
    assert np.abs(d).max() <= 1e-4 and np.abs(d).max() > 5e-5 and np.all(a[:, 3] == 1)


def test_workload_sizes():
    w = workloads.dam_break_65k()
    assert len(w["fluid"]) == 65536
    assert workloads.tait_stiffness(20.0) == pytest.approx(57142.857, rel=1e-6)


def test_pcisph_4m_workload_is_the_wcsph_scene_stepped_by_pcisph():
    """The 4M PCISPH line steps the WCSPH double dam break's particles and walls with the
    PCISPH settings of the 358k configuration, dt scaled by the spacing ratio."""
    pw = workloads.pcisph_double_dam_4m(n=16)
    ww = workloads.double_dam_4m(n=16)
    assert np.array_equal(pw["fluid"], ww["fluid"]) and len(pw["fluid"]) == 2 * 16 ** 3
    assert np.array_equal(pw["bodies"][0][0], ww["bodies"][0][0])
    p, q = pw["params"], workloads.pcisph_cube()["params"]
    assert p.method == capi.SPH_PCISPH and p.time_step == pytest.approx(5e-4 * 0.005 / 0.0125)
    assert p.particle_radius == pytest.approx(0.0025) and p.support_radius == pytest.approx(0.01)
    for f in ("pcisph_min_iterations", "pcisph_max_iterations", "pcisph_error_ratio", "k_viscosity",
              "surface_tension", "rest_density", "max_vel"):
        assert getattr(p, f) == pytest.approx(getattr(q, f)), f


def test_create_without_gpu_fails_cleanly():
    if capi.cuda_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(capi.SphError) as e:
        capi.Context(capi.default_params())
    assert e.value.code == 2


def test_invalid_parameters_are_rejected():
    p = capi.make_params(capi.SPH_WCSPH, support_radius=-1.0)
    with pytest.raises(capi.SphError) as e:
        capi.describe(p, (1, 1, 1))
    assert e.value.code == 1
    p = capi.make_params(capi.SPH_WCSPH, mode=1, particle_radius=0.0005, support_radius=0.001)
    with pytest.raises(capi.SphError):
        capi.describe(p, (2, 1, 1))   # 2004 cells per axis: more than 10-bit Morton coordinates
