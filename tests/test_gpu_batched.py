"""Batched scenes: S independent scenes in one context must give, scene by scene, what S
single-scene contexts give (same keys order inside a scene, same lists, same arithmetic)."""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads
from parity_util import assert_close

pytestmark = pytest.mark.gpu


def small_batch(n=4, seed=3):
    return workloads.batched_scenes(n, seed=seed, nmin=600, nmax=3000)


def test_batched_equals_single_scene_runs(gpu_lib):
    scenes = small_batch(5)
    shared = workloads.batched_params()
    batch = capi.BatchContext(shared, scenes)
    singles = [workloads.build_scene_context(shared, s) for s in scenes]
    assert batch.particle_count() == sum(len(s["fluid"]) for s in scenes)
    batch.simulate(20)
    for s in singles:
        s.simulate(20)
    pos = batch.get("POS").reshape(-1, 4)
    ids = batch.get("ID")
    dens = batch.get("DENSITY")
    for k, (sc, ctx) in enumerate(zip(scenes, singles)):
        first, count = batch.scene_range(k)
        assert count == len(sc["fluid"])
        p1 = ctx.get("POS").reshape(-1, 4)
        assert np.array_equal(ids[first:first + count] - first, ctx.get("ID"))
        assert_close("scene %d pos" % k, pos[first:first + count], p1, 4, rtol=1e-6)
        assert_close("scene %d density" % k, dens[first:first + count], ctx.get("DENSITY"), rtol=1e-5)
    st = batch.scene_stats()
    for k, ctx in enumerate(singles):
        s1 = ctx.stats()
        assert st[k, 0] == pytest.approx(s1["mean_compression"], rel=1e-4, abs=1e-7)
        assert st[k, 3] == pytest.approx(s1["kinetic"], rel=1e-4)
    assert batch.device_flags() & (capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]) == 0


def test_batched_scene_ranges_stay_contiguous(gpu_lib):
    scenes = small_batch(3, seed=9)
    batch = capi.BatchContext(workloads.batched_params(), scenes)
    batch.simulate(5)
    keys = batch.get("HASHES")
    d = capi.describe(workloads.batched_params(), (3.0, 1.0, 1.0))
    for k in range(3):
        first, count = batch.scene_range(k)
        # the sorted key's scene field equals the scene of the range
        shift = 21  # 3 x 7-bit Morton coordinates for containers up to 3 m at h = 0.03
        assert np.all((keys[first:first + count] >> shift) == k)
    assert d["grid_dims"][0] <= 128


def test_batched_rejects_single_scene_edits(gpu_lib):
    batch = capi.BatchContext(workloads.batched_params(), small_batch(2))
    with pytest.raises(capi.SphError):
        batch.set_rect_limits(1, 1, 1)
    with pytest.raises(capi.SphError):
        batch.add_volume(np.zeros((4, 4), np.float32))


def test_tile_shape_changes_no_result(gpu_lib):
    """The persistent per-scene tile launches (sph_set_tile_shape): every shape covers each
    scene's particles with tiles of 32 particles and gives the same state bit for bit (each
    particle's arithmetic does not depend on which warp takes its tile)."""
    scenes = small_batch(6, seed=5)
    shared = workloads.batched_params()
    out = []
    for bs, ctas in ((256, 0), (64, 1), (128, 4), (32, 2)):
        batch = capi.BatchContext(shared, scenes)
        batch.set_block_size(bs)
        batch.set_tile_shape(ctas)
        sh = batch.tile_shape()
        want = sum(-(-len(s["fluid"]) // 32) for s in scenes)
        assert sh["tile_particles"] == 32 and sh["ctas_per_sm"] == ctas and sh["tiles"] == want
        assert 1 <= sh["blocks"] <= -(-want // (bs // 32))
        batch.simulate(10)
        out.append((batch.get("POS"), batch.get("VEL"), batch.get("NEIGH_LEN")))
        assert batch.device_flags() & (capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]) == 0
        batch.close()
    for o in out[1:]:
        for a, b in zip(out[0], o):
            assert np.array_equal(a, b)
    single = workloads.build_scene_context(shared, scenes[0])
    assert capi.lib().sph_set_tile_shape(single.h, 2) == capi.SPH_E_INVALID   # not a batched context
    single.close()
