"""Parity of the CUDA path with the oracle at the benchmark configurations' full sizes.

The stage tests of test_gpu_parity.py run a ~2k-particle scene; these run the scenes the
benchmark lines are quoted on, built by fluids_gb300.workloads from the same seeds:

    dam_break_65k        65,536 fluid particles + FishTank walls (WCSPH, both modes,
                         neighbour lists and cell scan), all stages of one step
    pcisph_cube          358,400 fluid particles + walls + the rotated 0.3 m cube (PCISPH,
                         both modes): every stage, the loop's iteration count, and each pass
                         of one loop iteration alone on identical inputs
    double_dam_4m        4,194,304 fluid particles (24-bit keys, three sort passes, 2.2 M
                         cells): every WCSPH stage, then the fused CUDA-graph step the
                         benchmark times against one oracle step

Integer stages (Morton keys, mask, sort permutation, sorted positions, cell ranges,
neighbour lists and lengths) are compared bit for bit; FP32 fields within 1e-5 field-
relative (parity_util.RTOL) unless a test states otherwise, with the reason beside it.
The grid follows kernels/grid.cl:20-182, WCSPH kernels/wcsph.cl:32-224, normals
kernels/normals.cl:23-70, PCISPH kernels/pcisph.cl:33-504.
"""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads
from parity_util import RTOL, assert_close, make_pair, tait

pytestmark = pytest.mark.gpu

GRID = ["BOUNDARY_SYNC", "HASHES", "SORT", "SHUFFLE", "CELL_INTERVALS"]


def pair(w, **overrides):
    p = capi.SphParams.from_buffer_copy(w["params"])
    for k, v in overrides.items():
        setattr(p, k, v)
    return make_pair(p, w["fluid"], w["bodies"], w["container"], vel=w.get("velocities"))


def assert_lists_equal(a_list, a_len, b_list, b_len, name):
    """Column-major list[k * n + i], compared on the valid prefix k < len[i] of every
    particle, one row k at a time (the 4M lists are 800 MB each)."""
    assert np.array_equal(a_len, b_len), name + " lengths"
    n = len(a_len)
    cap = len(a_list) // max(n, 1)
    A = a_list.reshape(cap, n)
    B = b_list.reshape(cap, n)
    for k in range(cap):
        m = a_len > k
        if not m.any():
            break
        assert np.array_equal(A[k][m], B[k][m]), "%s differs in slot %d" % (name, k)


def check_grid(ctx, orc):
    for s in GRID:
        ctx.stage(s)
        orc.stage(s)
        if s == "HASHES":
            assert np.array_equal(ctx.get("HASHES"), orc.get("HASHES")), "Morton keys differ"
            assert np.array_equal(ctx.get("MASK"), orc.get("MASK"))
    assert np.array_equal(ctx.get("HASHES"), orc.get("HASHES")), "sorted keys differ"
    assert np.array_equal(ctx.get("MASK"), orc.get("MASK")), "sort permutation differs"
    assert np.array_equal(ctx.get("POS_SORTED"), orc.get("POS_SORTED"))
    assert np.array_equal(ctx.get("CELL_INTERVALS"), orc.get("CELL_INTERVALS")), "cell ranges differ"


def check_lists(ctx, orc):
    ctx.stage("NEIGH_LIST")
    orc.stage("NEIGH_LIST")
    orc.stage("SB_NEIGH_LIST")
    assert_lists_equal(ctx.get("NEIGH_LIST"), ctx.get("NEIGH_LEN"), orc.get("NEIGH_LIST"), orc.get("NEIGH_LEN"),
                       "fluid list")
    assert_lists_equal(ctx.get("SB_NEIGH_LIST"), ctx.get("SB_NEIGH_LEN"), orc.get("SB_NEIGH_LIST"),
                       orc.get("SB_NEIGH_LEN"), "boundary list")


def check_boundary(ctx, orc):
    assert np.array_equal(ctx.get("BHASHES"), orc.get("BHASHES"))
    assert np.array_equal(ctx.get("BMASK"), orc.get("BMASK"))
    assert np.array_equal(ctx.get("BPOS_SORTED"), orc.get("BPOS_SORTED"))
    assert np.array_equal(ctx.get("BCELL_INTERVALS"), orc.get("BCELL_INTERVALS"))
    assert_close("phi", ctx.get("BPHI_SORTED"), orc.get("BPHI_SORTED"))


def wcsph_stage_step(ctx, orc, params, compat):
    """One WCSPH step stage by stage (WCSPHSimulation::simulate order), each stage compared
    and the oracle continued from the GPU's output so each comparison isolates one stage."""
    n = ctx.particle_count()
    check_grid(ctx, orc)
    check_lists(ctx, orc)
    ctx.stage("WC_DENSITY")
    orc.stage("WC_DENSITY")
    d = ctx.get("DENSITY")
    assert_close("density", d, orc.get("DENSITY"))
    # the pressure is the equation of state of the density, bit for bit; compared with the
    # oracle's pressure it only inherits the density's last-place differences, amplified
    # by d p / d rho = 7 p / (rho - rho0) (hence the looser bar on that comparison)
    assert np.array_equal(ctx.get("PRESSURE"), tait(d, params)), "pressure is not the EOS of the density"
    assert_close("pressure", ctx.get("PRESSURE"), orc.get("PRESSURE"), rtol=1e-4)
    if compat:
        # COMPAT densities are negative (poly6 of r, wcsph.cl:61-62): drive the force branch
        # with physical density and pressure fields on both sides
        d = (1000.0 + 20.0 * np.sin(np.arange(n))).astype(np.float32)
        p = tait(d, params)
        for o in (ctx, orc):
            o.set("DENSITY", d)
            o.set("PRESSURE", p)
    else:
        orc.set("DENSITY", ctx.get("DENSITY"))
        orc.set("PRESSURE", ctx.get("PRESSURE"))
    ctx.stage("NORMALS")
    orc.stage("NORMALS")
    assert_close("normal", ctx.get("NORMAL"), orc.get("NORMAL"), 4)
    orc.set("NORMAL", ctx.get("NORMAL"))
    ctx.stage("WC_ACCEL")
    orc.stage("WC_ACCEL")
    assert_close("accel", ctx.get("ACCEL"), orc.get("ACCEL"), 4)
    orc.set("ACCEL", ctx.get("ACCEL"))
    ctx.stage("WC_INTEGRATE")
    orc.stage("WC_INTEGRATE")
    assert_close("pos", ctx.get("POS"), orc.get("POS"), 4, rtol=1e-6)
    assert_close("vel", ctx.get("VEL"), orc.get("VEL"), 4)
    assert_close("vel_half", ctx.get("VEL_HALF"), orc.get("VEL_HALF"), 4)
    assert np.array_equal(ctx.get("ID"), orc.get("ID"))


@pytest.mark.parametrize("mode", [capi.SPH_MODE_COMPAT, capi.SPH_MODE_PHYSICS])
@pytest.mark.parametrize("neighbor_mode", [capi.SPH_NEIGH_SCAN, capi.SPH_NEIGH_LIST])
def test_dam_break_65k_stages(gpu_lib, mode, neighbor_mode):
    w = workloads.dam_break_65k(mode=mode)
    assert len(w["fluid"]) == 65536
    ctx, orc = pair(w, neighbor_mode=neighbor_mode)
    check_boundary(ctx, orc)
    for step in range(2):
        wcsph_stage_step(ctx, orc, w["params"], mode == capi.SPH_MODE_COMPAT)
        for f in ("POS", "VEL", "VEL_HALF"):
            orc.set(f, ctx.get(f))
    ctx.close()


@pytest.mark.parametrize("mode", [capi.SPH_MODE_COMPAT, capi.SPH_MODE_PHYSICS])
def test_pcisph_cube_358k_stages(gpu_lib, mode):
    w = workloads.pcisph_cube(mode=mode)
    assert len(w["fluid"]) == 358400
    ctx, orc = pair(w)
    check_boundary(ctx, orc)
    check_grid(ctx, orc)
    check_lists(ctx, orc)
    for s in ("PCI_INIT_DENSITY", "NORMALS", "PCI_INIT_FORCES"):
        ctx.stage(s)
        orc.stage(s)
        if s == "PCI_INIT_DENSITY":
            assert_close("density", ctx.get("DENSITY"), orc.get("DENSITY"))
            orc.set("DENSITY", ctx.get("DENSITY"))
        elif s == "NORMALS":
            assert_close("normal", ctx.get("NORMAL"), orc.get("NORMAL"), 4)
            orc.set("NORMAL", ctx.get("NORMAL"))
    assert_close("f_other", ctx.get("FORCE_OTHER"), orc.get("FORCE_OTHER"), 4)
    orc.set("FORCE_OTHER", ctx.get("FORCE_OTHER"))

    # one iteration's passes alone, each on identical inputs (pressure and pressure force
    # start at zero as the loop's first iteration does)
    ctx.stage("PCI_PREDICT")
    orc.stage("PCI_PREDICT")
    assert_close("pos_pred", ctx.get("POS_PRED"), orc.get("POS_PRED"), 4, rtol=1e-6)
    orc.set("POS_PRED", ctx.get("POS_PRED"))
    ctx.stage("PCI_UPDATE_PRESSURE")
    orc.stage("PCI_UPDATE_PRESSURE")
    rho0 = w["params"].rest_density
    # rho* - rho0 is a difference of nearly equal numbers: bar of 1e-5 of rho0, the density's
    assert np.abs(ctx.get("DENS_VAR").astype(np.float64) - orc.get("DENS_VAR")).max() <= RTOL * rho0
    orc.set("DENS_VAR", ctx.get("DENS_VAR"))
    orc.set("PRESSURE", ctx.get("PRESSURE"))
    ctx.stage("PCI_PRESSURE_FORCE")
    orc.stage("PCI_PRESSURE_FORCE")
    assert_close("f_press (one pass)", ctx.get("FORCE_PRESSURE"), orc.get("FORCE_PRESSURE"), 4)

    # the whole loop from the same start: the iteration count is equal; the fields
    # accumulate the passes' last-place differences through rho* - rho0 over 3..8
    # iterations (each pass alone meets 1e-5 above)
    for o in (ctx, orc):
        o.stage("PCI_INIT_FORCES")          # F_p = 0, as at the loop's start
        o.set("PRESSURE", np.zeros(ctx.particle_count(), np.float32))   # p = 0, likewise
    orc.set("FORCE_OTHER", ctx.get("FORCE_OTHER"))
    ctx.stage("PCI_LOOP")
    orc.stage("PCI_LOOP")
    assert ctx.get("PCI_ITERS")[0] == orc.get("PCI_ITERS")[0]
    assert_close("pressure (loop)", ctx.get("PRESSURE"), orc.get("PRESSURE"), rtol=1e-4)
    assert_close("f_press (loop)", ctx.get("FORCE_PRESSURE"), orc.get("FORCE_PRESSURE"), 4, rtol=1e-4)
    orc.set("FORCE_PRESSURE", ctx.get("FORCE_PRESSURE"))
    ctx.stage("PCI_INTEGRATE")
    orc.stage("PCI_INTEGRATE")
    assert_close("pos", ctx.get("POS"), orc.get("POS"), 4, rtol=1e-6)
    assert_close("vel", ctx.get("VEL"), orc.get("VEL"), 4)
    assert np.array_equal(ctx.get("ID"), orc.get("ID"))
    ctx.close()


def test_double_dam_4m_stages(gpu_lib):
    w = workloads.double_dam_4m()
    assert len(w["fluid"]) == 4194304
    ctx, orc = pair(w)
    assert orc.derived()["key_bits"] == 24
    check_boundary(ctx, orc)
    wcsph_stage_step(ctx, orc, w["params"], False)
    ctx.close()


def test_double_dam_4m_graph_step(gpu_lib):
    """The fused step the benchmark replays (CUDA graph: fused list build + density, gather
    + cell ranges, forces with the integration as epilogue) against one oracle step."""
    w = workloads.double_dam_4m()
    ctx, orc = pair(w)
    ctx.simulate(1)
    orc.step(1)
    assert ctx.device_flags() & (capi.FLAGS["NAN"] | capi.FLAGS["TIMEOUT"]) == 0
    assert np.array_equal(ctx.get("ID"), orc.get("ID")), "particle order differs"
    assert np.array_equal(ctx.get("CELL_INTERVALS"), orc.get("CELL_INTERVALS")), "cell ranges differ"
    assert_lists_equal(ctx.get("NEIGH_LIST"), ctx.get("NEIGH_LEN"), orc.get("NEIGH_LIST"), orc.get("NEIGH_LEN"),
                       "fluid list")
    assert_lists_equal(ctx.get("SB_NEIGH_LIST"), ctx.get("SB_NEIGH_LEN"), orc.get("SB_NEIGH_LIST"),
                       orc.get("SB_NEIGH_LEN"), "boundary list")
    assert_close("density", ctx.get("DENSITY"), orc.get("DENSITY"))
    assert_close("pos", ctx.get("POS"), orc.get("POS"), 4, rtol=1e-6)
    assert_close("vel", ctx.get("VEL"), orc.get("VEL"), 4)
    assert_close("vel_half", ctx.get("VEL_HALF"), orc.get("VEL_HALF"), 4)
    ctx.close()
