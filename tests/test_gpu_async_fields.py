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
