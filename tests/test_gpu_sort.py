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
