"""sph_set_field_async / sph_get_field_async: the stream-ordered copies give the same state as
the synchronous ones."""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def test_async_copies_match_sync(gpu_lib):
    import torch
    w = workloads.dam_break_65k(steps=3)
    a = workloads.build_context(w)
    b = workloads.build_context(w)
    L = capi.lib()
    n = a.particle_count()
    bufs = {f: torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy() for f in ("POS", "VEL", "VEL_HALF")}
    for _ in range(3):
        for f, h in bufs.items():
            capi.check(L.sph_get_field_async(a.h, capi.FIELDS[f], h.ctypes.data, h.nbytes), a.h)
        capi.check(L.sph_synchronize(a.h), a.h)
        for f, h in bufs.items():
            capi.check(L.sph_set_field_async(a.h, capi.FIELDS[f], h.ctypes.data, h.nbytes), a.h)
        a.simulate(1)
        for f in bufs:
            b.set(f, b.get(f))
        b.simulate(1)
    a.synchronize()
    for f in ("POS", "VEL", "VEL_HALF", "ID"):
        assert np.array_equal(a.get(f), b.get(f)), f
    with pytest.raises(capi.SphError):
        capi.check(L.sph_get_field_async(a.h, capi.FIELDS["POS"], bufs["POS"].ctypes.data, 12), a.h)


def _host_state(ctx, pinned):
    import torch
    n = ctx.particle_count()
    out = []
    for f in ("POS", "VEL", "VEL_HALF"):
        h = (torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy() if pinned
             else np.empty((n, 4), np.float32))
        h[:] = ctx.get(f).reshape(n, 4)
        out.append(h)
    return out


@pytest.mark.parametrize("method", ["wcsph", "pcisph"])
@pytest.mark.parametrize("use_graph,pinned", [(1, True), (1, False), (0, True)])
def test_simulate_host_matches_field_copies(gpu_lib, method, use_graph, pinned):
    """sph_simulate_host (state on the host, the velocity uploads beside the binning, sort and
    list pass) against the same steps through the field copies and sph_simulate: the state
    and the sort bit for bit, step after step; a graph with page-locked buffers, the
    stream-ordered path with pageable ones or without graphs."""
    if method == "wcsph":
        w = workloads.dam_break_65k(steps=5)
    else:
        w = workloads.pcisph_cube()
    w["params"].use_graph = use_graph
    a = workloads.build_context(w)
    b = workloads.build_context(w)
    pos, vel, vh = _host_state(a, pinned)
    for step in range(4):
        a.simulate_host(pos, vel, vh if method == "wcsph" else None, steps=1)
        for f in ("POS", "VEL", "VEL_HALF"):
            b.set(f, b.get(f))
        b.simulate(1)
        assert np.array_equal(pos.reshape(-1), b.get("POS")), "step %d" % step
        assert np.array_equal(vel.reshape(-1), b.get("VEL")), "step %d" % step
        if method == "wcsph":
            assert np.array_equal(vh.reshape(-1), b.get("VEL_HALF")), "step %d" % step
        assert np.array_equal(a.get("MASK"), b.get("MASK")), "step %d" % step
        assert np.array_equal(a.get("DENSITY"), b.get("DENSITY")), "step %d" % step
    assert a.device_flags() & (capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]) == 0
    # two steps in one call give the state of two single steps
    a.simulate_host(pos, vel, vh if method == "wcsph" else None, steps=2)
    b.simulate(2)
    assert np.array_equal(pos.reshape(-1), b.get("POS"))
    assert np.array_equal(vel.reshape(-1), b.get("VEL"))
    a.close()
    b.close()


def test_simulate_host_argument_checks(gpu_lib):
    w = workloads.dam_break_65k(steps=1)
    a = workloads.build_context(w)
    n = a.particle_count()
    pos = np.zeros((n, 4), np.float32)
    with pytest.raises(ValueError):
        a.simulate_host(pos, np.zeros((n, 3), np.float32), pos)
    with pytest.raises(capi.SphError):
        capi.check(capi.lib().sph_simulate_host(a.h, pos.ctypes.data, None, None, 1), a.h)
    a.close()
