"""Known-answer tests of the oracle (CPU only)."""
import numpy as np
import pytest

from oracle import Oracle, morton3, stable_sort_pairs
from scenes_np import jittered_block


def test_morton_known_answers():
    assert morton3(0, 0, 0) == 0
    assert morton3(1, 0, 0) == 1
    assert morton3(0, 1, 0) == 2
    assert morton3(0, 0, 1) == 4
    assert morton3(1, 1, 1) == 7
    assert morton3(2, 0, 0) == 8
    assert morton3(1023, 1023, 1023) == 2 ** 30 - 1


def test_morton_is_bit_interleaving_below_1024():
    rng = np.random.default_rng(1)
    for _ in range(200):
        x, y, z = (int(v) for v in rng.integers(0, 1024, 3))
        exp = 0
        for b in range(10):
            exp |= ((x >> b) & 1) << (3 * b) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b + 2)
        assert morton3(x, y, z) == exp


def test_stable_sort_pairs():
    rng = np.random.default_rng(2)
    k = rng.integers(0, 50, 10000).astype(np.uint32)
    v = np.arange(10000, dtype=np.int32)
    ks, vs = stable_sort_pairs(k, v)
    order = np.argsort(k, kind="stable")
    assert np.array_equal(ks, k[order]) and np.array_equal(vs, order)


def test_physics_lattice_density_near_rest():
    """PHYSICS mode (315 poly6, r^2): interior density of a 2h = 2 dx lattice is near rho0."""
    o = Oracle(method=0, mode=1, container=(1.0, 1.0, 1.0))
    o.set_fluid(jittered_block(20, 20, 20, 0.015, (-0.15, -0.15, -0.15), amp=0.0))
    for s in ("HASHES", "SORT", "SHUFFLE", "CELL_INTERVALS", "NEIGH_LIST", "SB_NEIGH_LIST", "WC_DENSITY"):
        o.stage(s)
    d = o.get("DENSITY")
    p = o.get("POS_SORTED").reshape(-1, 4)
    interior = np.all(np.abs(p[:, :3]) < 0.08, axis=1)
    m = d[interior].mean()
    assert 0.9 * 1000 < m < 1.1 * 1000, m


def test_compat_wcsph_density_is_negative():
    """The kernel text evaluates poly6 at r instead of r^2 (wcsph.cl:61-62)."""
    o = Oracle(method=0, mode=0, container=(1.0, 1.0, 1.0))
    o.set_fluid(jittered_block(8, 8, 8, 0.015, (-0.06, -0.06, -0.06)))
    for s in ("HASHES", "SORT", "SHUFFLE", "CELL_INTERVALS", "NEIGH_LIST", "SB_NEIGH_LIST", "WC_DENSITY"):
        o.stage(s)
    assert np.all(o.get("DENSITY") < 0) and np.all(o.get("PRESSURE") == 0)


def test_compat_pcisph_stops_at_min_iterations():
    o = Oracle(method=1, mode=0, container=(1.0, 1.0, 1.0), time_step=5e-4, pci_max_iter=8, surface_tension=1.0)
    o.set_fluid(jittered_block(10, 10, 10, 0.015, (-0.07, -0.2, -0.07)))
    o.step(1)
    assert o.get("PCI_ITERS")[0] == 3


def test_double_precision_oracle_runs():
    o = Oracle(method=0, mode=1, precision=1, container=(0.5, 1.0, 0.4))
    o.set_fluid(jittered_block(6, 6, 6, 0.015, (0.0, -0.45, 0.0)))
    o.step(3)
    pos = o.get("POS")
    assert pos.dtype == np.float64 and np.all(np.isfinite(pos))
    st = o.stats()
    assert st["kinetic"] > 0
