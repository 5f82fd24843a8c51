"""The onesweep radix sort (clsort replacement) against a stable CPU sort, bit for bit."""
import numpy as np
import pytest
import torch

from fluids_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 2, 17, 4095, 4096, 4097, 100_003, 1_000_000])
@pytest.mark.parametrize("bits", [8, 21, 32])
def test_sort_pairs_is_a_stable_sort(gpu_lib, n, bits):
    rng = np.random.default_rng(n * 31 + bits)
    hi = (1 << bits) if bits < 32 else (1 << 32)
    # odd n: keys over the whole key range; even n: few distinct keys (stability under ties)
    top = hi if n % 2 else min(hi, 1 << 10)
    keys = rng.integers(0, top, size=n, dtype=np.int64).astype(np.uint32)
    vals = np.arange(n, dtype=np.int32)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals).cuda()
    capi.sort_pairs_device(dk.data_ptr(), dv.data_ptr(), n, bits)
    torch.cuda.synchronize()
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(dk.cpu().numpy().view(np.uint32), keys[order])
    assert np.array_equal(dv.cpu().numpy(), order.astype(np.int32))


def test_sort_nearly_sorted_morton_keys(gpu_lib):
    """Keys as the step produces them: sorted last step, perturbed by motion."""
    rng = np.random.default_rng(7)
    n = 1 << 20
    keys = np.sort(rng.integers(0, 1 << 21, size=n).astype(np.uint32))
    swap = rng.integers(0, n - 1, size=n // 50)
    keys[swap], keys[swap + 1] = keys[swap + 1].copy(), keys[swap].copy()
    vals = np.arange(n, dtype=np.int32)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals).cuda()
    capi.sort_pairs_device(dk.data_ptr(), dv.data_ptr(), n, 21)
    torch.cuda.synchronize()
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(dv.cpu().numpy(), order.astype(np.int32))


# --- the step's sort: an update of the previous step's sorted order -------------------------

def _sort_ctx(n, seed=0):
    """A PHYSICS WCSPH context of n particles spread over a 1 m cube (no walls)."""
    from fluids_gb300 import workloads
    container = (1.0, 1.0, 1.0)
    rng = np.random.default_rng(seed)
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.05, 0.95, (n, 3))
    params = workloads.wcsph_params(0.01, 2e-4, capi.SPH_MODE_PHYSICS)
    ctx = capi.Context(params)
    ctx.set_rect_limits(*container)
    ctx.add_volume(pos)
    return ctx, capi.describe(params, container)["key_bits"]


def _stage_sort(ctx, keys):
    """The SORT stage over the given keys (written over the HASHES stage's output)."""
    ctx.stage("HASHES")
    ctx.set("HASHES", keys)
    ctx.stage("SORT")
    assert ctx.device_flags() & capi.FLAGS["TIMEOUT"] == 0
    return ctx.get("HASHES").astype(np.uint32), ctx.get("MASK")


def _check(ctx, keys):
    sk, perm = _stage_sort(ctx, keys)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(perm, order.astype(np.int32))
    assert np.array_equal(sk, keys[order])
    return keys[order]


@pytest.mark.parametrize("n", [1, 2, 33, 2047, 2049, 100_003])
def test_incremental_sort_is_the_stable_sort(gpu_lib, n):
    """Successive SORT stages: the first has no previous order (a full sort), each later one
    updates the last result -- unchanged keys, 1.5 % of keys moved, a moved block of equal
    keys larger than one merge tile's staged slice, heavy ties, and keys with no relation to
    the previous order.  Each is the stable sort of its keys, bit for bit."""
    ctx, bits = _sort_ctx(n, seed=n)
    rng = np.random.default_rng(n + 1)
    top = 1 << bits
    prev = _check(ctx, rng.integers(0, top, n, dtype=np.int64).astype(np.uint32))   # no previous order
    prev = _check(ctx, prev.copy())                                                 # nothing moved
    k = prev.copy()
    sel = rng.random(n) < 0.015
    k[sel] = rng.integers(0, top, int(sel.sum()), dtype=np.int64).astype(np.uint32)
    prev = _check(ctx, k)                                                          # 1.5 % moved
    k = prev.copy()
    sel = rng.random(n) < 0.05
    k[sel] = prev[n // 2]                                                          # 5 % onto one key
    prev = _check(ctx, k)
    k = prev.copy()
    sel = rng.random(n) < 0.3
    k[sel] = rng.integers(0, 8, int(sel.sum()), dtype=np.int64).astype(np.uint32)  # ties
    prev = _check(ctx, k)
    _check(ctx, rng.permutation(prev))                                              # unrelated order
    ctx.close()


def test_incremental_sort_along_a_flowing_step(gpu_lib):
    """The fused step's own sort (hash kernel with the first pass of the update) against the
    stable sort of the keys of the positions it starts from, over 40 steps of a
    65,536-particle dam break (a few per cent of the particles change cell per step)."""
    from fluids_gb300 import workloads
    w = workloads.dam_break_65k(mode=capi.SPH_MODE_PHYSICS)
    ctx = capi.Context(w["params"])
    ctx.set_rect_limits(*w["container"])
    for pts, rot, mv, mass in w["bodies"]:
        ctx.add_boundary(pts, can_move=mv, rot3x4=rot, mass=mass)
    ctx.add_volume(w["fluid"])
    moved = []
    prev = None
    for step in range(40):
        ctx.stage("HASHES")                             # the keys this step's hash kernel computes
        keys = ctx.get("HASHES").astype(np.uint32)
        if prev is not None:
            moved.append(float(np.mean(keys != prev)))
        ctx.simulate(1)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(ctx.get("MASK"), order.astype(np.int32)), "step %d" % step
        prev = ctx.get("HASHES").astype(np.uint32)      # sorted keys, in the particles' order now
        assert np.array_equal(prev, keys[order])
    assert ctx.device_flags() & capi.FLAGS["TIMEOUT"] == 0
    assert 0.0 < max(moved) < 0.5
    ctx.close()
