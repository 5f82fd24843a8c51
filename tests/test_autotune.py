"""The launch-shape autotuner: choice, persistence and reuse (CPU, with a stand-in context),
and on the GPU that the block size changes no result."""
import numpy as np
import pytest

from fluids_gb300 import autotune, capi, workloads


class FakeCtx:
    """Stands in for a context: simulate() advances a clock by a per-block-size cost."""

    def __init__(self, cost, n=5000):
        self.cost, self.n, self.bs, self.now, self.calls = cost, n, 256, 0.0, []

    def particle_count(self):
        return self.n

    def set_block_size(self, bs):
        self.bs = bs
        self.calls.append(bs)

    def simulate(self, steps):
        self.now += steps * self.cost[self.bs]

    def synchronize(self):
        pass

    def clock(self):
        return self.now


def test_tune_picks_fastest_and_caches(tmp_path):
    path = str(tmp_path / "launch.json")
    ctx = FakeCtx({64: 3.0, 128: 1.0, 256: 2.0})
    r = autotune.tune(ctx, 0, 1, False, steps=4, warmup=1, path=path, device="GB300", clock=ctx.clock)
    assert r["block_size"] == 128 and r["source"] == "timed" and ctx.bs == 128
    assert r["seconds_per_step"] == {"64": 3.0, "128": 1.0, "256": 2.0}
    ctx2 = FakeCtx({64: 0.1, 128: 9.0, 256: 9.0}, n=6000)   # same power-of-two bucket
    r2 = autotune.tune(ctx2, 0, 1, False, path=path, device="GB300", clock=ctx2.clock)
    assert r2["source"] == "cache" and r2["block_size"] == 128 and ctx2.calls == [128]
    ctx3 = FakeCtx({64: 0.1, 128: 9.0, 256: 9.0}, n=6000)
    r3 = autotune.tune(ctx3, 0, 1, True, path=path, device="GB300", clock=ctx3.clock)   # other key
    assert r3["source"] == "timed" and r3["block_size"] == 64
    assert len(autotune.load_cache(path)) == 2


def test_tie_prefers_larger_blocks(tmp_path):
    ctx = FakeCtx({64: 1.0, 128: 1.0, 256: 1.0})
    r = autotune.tune(ctx, 1, 1, False, use_cache=False, device="x", clock=ctx.clock)
    assert r["block_size"] == 256


@pytest.mark.gpu
def test_block_size_changes_no_result(gpu_lib):
    w = workloads.dam_break_65k(steps=5)
    out = []
    for bs in (64, 256):
        ctx = workloads.build_context(w)
        ctx.set_block_size(bs)
        ctx.simulate(5)
        ctx.synchronize()
        pos = ctx.get("POS").reshape(-1, 4)
        ids = ctx.get("ID")
        o = np.empty_like(pos)
        o[ids] = pos
        out.append(o)
        ctx.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
def test_tune_on_a_context_keeps_its_state(gpu_lib, tmp_path):
    w = workloads.dam_break_65k(steps=5)
    ref = workloads.build_context(w)
    ref.simulate(3)
    ctx = workloads.build_context(w)
    r = autotune.tune(ctx, capi.SPH_WCSPH, capi.SPH_MODE_PHYSICS, False, steps=3, warmup=1,
                      path=str(tmp_path / "l.json"))
    assert r["block_size"] in autotune.CANDIDATES and r["source"] == "timed"
    ctx.simulate(3)
    for f in ("POS", "VEL", "ID"):
        assert np.array_equal(ctx.get(f), ref.get(f)), f
    assert ctx.device_flags() & capi.FLAGS["NAN"] == 0


class FakeBatch(FakeCtx):
    """A batched stand-in: the cost depends on the block size and the CTAs per SM."""

    def __init__(self, cost, n=5000):
        super().__init__(cost, n)
        self.ctas = 0

    def set_tile_shape(self, k):
        self.ctas = k

    def simulate(self, steps):
        self.now += steps * self.cost[(self.bs, self.ctas)]


def test_batched_tunes_tile_shapes_and_caches(tmp_path):
    path = str(tmp_path / "launch.json")
    cost = {(bs, k): 5.0 for bs in autotune.CANDIDATES for k in autotune.TILE_CTAS}
    cost[(128, 2)] = 1.0
    ctx = FakeBatch(cost)
    r = autotune.tune(ctx, 0, 1, True, steps=2, warmup=1, path=path, device="GB300", clock=ctx.clock)
    assert (r["block_size"], r["ctas_per_sm"]) == (128, 2) and (ctx.bs, ctx.ctas) == (128, 2)
    assert len(r["seconds_per_step"]) == len(autotune.CANDIDATES) * len(autotune.TILE_CTAS)
    ctx2 = FakeBatch(cost)
    r2 = autotune.tune(ctx2, 0, 1, True, path=path, device="GB300", clock=ctx2.clock)
    assert r2["source"] == "cache" and (ctx2.bs, ctx2.ctas) == (128, 2)
