"""sph_sort_pairs_noalloc: the sort for callers that cannot allocate device memory.

Some host programs cannot let a library call cudaMalloc (their allocator owns the device
heap, or they sort from a callback where allocating is not allowed).  This entry point uses
one fixed device array instead of allocated scratch.  These tests call it through the C ABI
and compare its output with sph_sort_pairs (the allocating entry point) bit for bit, on
consecutive calls, so that contents the shared array keeps from one call cannot leak into
the next.  This file is collected last; the tests also pass alone in a fresh process."""
import numpy as np
import pytest
import torch

from fluids_gb300 import capi

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 20


def noalloc_sort(keys, vals, bits):
    k_in = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    v_in = torch.from_numpy(vals.copy()).cuda()
    k_out = torch.full_like(k_in, -7)
    v_out = torch.full_like(v_in, -7)
    rc = capi.lib().sph_sort_pairs_noalloc(k_in.data_ptr(), v_in.data_ptr(), k_out.data_ptr(), v_out.data_ptr(),
                                           len(keys), bits, None)
    assert rc == 0, capi.STATUS.get(rc)
    torch.cuda.synchronize()
    # the input pairs are only read
    assert np.array_equal(k_in.cpu().numpy().view(np.uint32), keys)
    assert np.array_equal(v_in.cpu().numpy(), vals)
    return k_out.cpu().numpy().view(np.uint32), v_out.cpu().numpy()


def allocating_sort(keys, vals, bits):
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.copy()).cuda()
    capi.sort_pairs_device(dk.data_ptr(), dv.data_ptr(), len(keys), bits)
    torch.cuda.synchronize()
    return dk.cpu().numpy().view(np.uint32), dv.cpu().numpy()


def test_noalloc_sort_matches_allocating_sort_on_consecutive_calls(gpu_lib):
    rng = np.random.default_rng(11)
    # a large call, then a smaller one with other key widths: the second must not see the
    # first call's histograms, look-back words or ping-pong copy
    for n, bits, top in ((MAX_PAIRS, 21, 1 << 21), (300_001, 32, 1 << 32), (4_999, 8, 1 << 6)):
        keys = rng.integers(0, top, size=n, dtype=np.int64).astype(np.uint32)
        vals = rng.permutation(n).astype(np.int32)
        a_k, a_v = noalloc_sort(keys, vals, bits)
        b_k, b_v = allocating_sort(keys, vals, bits)
        assert np.array_equal(a_k, b_k), (n, bits)
        assert np.array_equal(a_v, b_v), (n, bits)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(a_v, vals[order])


def test_noalloc_sort_rejects_what_it_cannot_do(gpu_lib):
    L = capi.lib()
    k = torch.zeros(8, dtype=torch.int32, device="cuda")
    v = torch.zeros(8, dtype=torch.int32, device="cuda")
    ko = torch.zeros(8, dtype=torch.int32, device="cuda")
    vo = torch.zeros(8, dtype=torch.int32, device="cuda")
    # more pairs than the fixed array holds: refused before anything is launched
    assert L.sph_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), ko.data_ptr(), vo.data_ptr(), MAX_PAIRS + 1, 32,
                                    None) == 7
    assert L.sph_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), ko.data_ptr(), vo.data_ptr(), 8, 0, None) == 1
    # an output aliasing an input, its own or the other one (with 8-bit keys the single pass
    # would write the outputs while still reading the inputs), or the other output
    assert L.sph_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), k.data_ptr(), vo.data_ptr(), 8, 32, None) == 1
    assert L.sph_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), ko.data_ptr(), k.data_ptr(), 8, 8, None) == 1
    assert L.sph_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), v.data_ptr(), vo.data_ptr(), 8, 8, None) == 1
    assert L.sph_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), ko.data_ptr(), ko.data_ptr(), 8, 8, None) == 1
    assert L.sph_sort_pairs_noalloc(k.data_ptr(), v.data_ptr(), ko.data_ptr(), vo.data_ptr(), 0, 32, None) == 0
    torch.cuda.synchronize()
