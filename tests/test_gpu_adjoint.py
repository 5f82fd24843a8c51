"""Differentiable WCSPH on the GPU (sph_adj_*) against the FP64 adjoint oracle, central
finite differences of the FP64 forward, the plain solver's forward step, and itself
(checkpoint interval, determinism, linearity); plus the torch.autograd wrapper."""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _by_id(ctx, field):
    p = ctx.get(field).reshape(-1, 4)
    ids = ctx.get("ID")
    out = np.empty_like(p)
    out[ids] = p
    return out


def _seed(xT, y):
    g = np.zeros_like(xT)
    g[:, :3] = 2.0 * (xT[:, :3].astype(np.float64) - y[:, :3]) / len(xT)
    return g


@pytest.fixture(scope="module")
def block16(gpu_lib):
    w = workloads.adjoint_block(16, steps=200)
    ctx = workloads.build_context(w)
    adj = capi.Adjoint(ctx, 200, 20)
    xT, _ = adj.forward(w["fluid"], w["velocities"], w["mu"], w["kgas"])
    g = adj.backward(_seed(xT, w["target"]))
    return dict(w=w, ctx=ctx, adj=adj, xT=xT, g=g)


def test_adjoint_forward_is_the_plain_step(gpu_lib):
    w = workloads.adjoint_block(16, steps=20)
    ctx = workloads.build_context(w)
    adj = capi.Adjoint(ctx, 20, 20)
    xT, vT = adj.forward(w["fluid"], w["velocities"], w["mu"], w["kgas"])
    ctx.simulate(20)
    ctx.synchronize()
    np.testing.assert_allclose(xT[:, :3], _by_id(ctx, "POS")[:, :3], rtol=0, atol=1e-6)
    np.testing.assert_allclose(vT[:, :3], _by_id(ctx, "VEL")[:, :3], rtol=0, atol=1e-5)
    assert adj.flags() == 0


def test_gradients_match_fp64_adjoint(block16):
    from oracle import adjoint as A
    w, g = block16["w"], block16["g"]
    d = capi.describe(w["params"], w["container"])
    P = A.make_params(w["params"], d, w["container"], 200)
    xo, _, mx = A.forward(P, w["fluid"], w["velocities"])
    assert mx < 50
    assert np.abs(xo - block16["xT"][:, :3]).max() < 1e-5
    go = A.backward(P, w["fluid"], w["velocities"], 2.0 * (xo - w["target"][:, :3]) / len(xo))
    assert abs(g["g_mu"] - go["g_mu"]) <= 1e-4 * abs(go["g_mu"])
    assert abs(g["g_k"] - go["g_k"]) <= 1e-3 * abs(go["g_k"])
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)   # noqa: E731
    assert rel(g["g_v0"][:, :3], go["g_v0"]) <= 1e-3
    assert rel(g["g_x0"][:, :3], go["g_x0"]) <= 5e-3


def test_gradients_match_central_differences(block16):
    """dL/dmu, dL/dc0 and a directional dL/dv0 from the GPU adjoint within 1e-3 of central
    differences of the FP64 forward (FP32 differences are dominated by rounding noise)."""
    from oracle import adjoint as A
    w, g = block16["w"], block16["g"]
    d = capi.describe(w["params"], w["container"])
    y = w["target"][:, :3].astype(np.float64)
    x0, v0 = w["fluid"], w["velocities"]

    def loss(mu=None, k=None, v=v0):
        P = A.make_params(w["params"], d, w["container"], 200, mu=mu, k=k)
        xT, _, _ = A.forward(P, x0, v)
        return float(np.mean(np.sum((xT - y) ** 2, axis=1)))

    e = w["mu"] * 1e-3
    fd_mu = (loss(mu=w["mu"] + e) - loss(mu=w["mu"] - e)) / (2 * e)
    assert abs(g["g_mu"] - fd_mu) <= 1e-3 * abs(fd_mu)
    c0 = w["c0"]
    e = c0 * 1e-3
    fd_c0 = (loss(k=workloads.tait_stiffness(c0 + e)) - loss(k=workloads.tait_stiffness(c0 - e))) / (2 * e)
    assert abs(g["g_c0"] - fd_c0) <= 1e-3 * abs(fd_c0)
    # a smooth direction (another divergence-free Fourier field): white-noise directions
    # make the directional derivative a near-cancelling sum
    dd = workloads.fourier_velocity(x0, 8, 1.0, seed=99)[:, :3].astype(np.float64)
    e = 1e-4
    vp, vm = v0.astype(np.float64).copy(), v0.astype(np.float64).copy()
    vp[:, :3] += e * dd
    vm[:, :3] -= e * dd
    fd_v = (loss(v=vp) - loss(v=vm)) / (2 * e)
    ad_v = float(np.sum(g["g_v0"][:, :3].astype(np.float64) * dd))
    assert abs(ad_v - fd_v) <= 1e-3 * abs(fd_v)


def test_checkpoint_interval_and_determinism(block16):
    w, ctx, g = block16["w"], block16["ctx"], block16["g"]
    seed = _seed(block16["xT"], w["target"])
    again = block16["adj"].backward(seed)
    assert np.array_equal(again["g_v0"], g["g_v0"]) and again["g_mu"] == g["g_mu"] and again["g_k"] == g["g_k"]
    for every in (7, 200):
        a = capi.Adjoint(ctx, 200, every)
        xT, _ = a.forward(w["fluid"], w["velocities"], w["mu"], w["kgas"])
        assert np.array_equal(xT, block16["xT"])
        r = a.backward(seed)
        assert np.array_equal(r["g_v0"], g["g_v0"]) and np.array_equal(r["g_x0"], g["g_x0"])
        assert r["g_mu"] == g["g_mu"] and r["g_k"] == g["g_k"]


def test_backward_is_linear_in_the_seed(block16):
    adj = block16["adj"]
    n = len(block16["xT"])
    rng = np.random.default_rng(4)
    u = np.zeros((n, 4), np.float32)
    v = np.zeros((n, 4), np.float32)
    u[:, :3] = rng.normal(size=(n, 3))
    v[:, :3] = rng.normal(size=(n, 3))
    gu, gv, gs = (adj.backward(s) for s in (u, v, 2.0 * u - 3.0 * v))
    for k in ("g_x0", "g_v0"):
        ref = 2.0 * gu[k].astype(np.float64) - 3.0 * gv[k]
        assert np.linalg.norm(gs[k] - ref) <= 1e-5 * np.linalg.norm(ref)
    for k in ("g_mu", "g_k"):
        ref = 2.0 * gu[k] - 3.0 * gv[k]
        assert abs(gs[k] - ref) <= 1e-4 * (abs(gu[k]) + abs(gv[k]))


def test_torch_autograd_wrapper(block16):
    torch = pytest.importorskip("torch")
    from adjoint_torch import rollout
    w, adj, g = block16["w"], block16["adj"], block16["g"]
    dev = torch.device("cuda:0")
    x0 = torch.tensor(w["fluid"], device=dev, requires_grad=True)
    v0 = torch.tensor(w["velocities"], device=dev, requires_grad=True)
    mu = torch.tensor(float(np.float32(w["mu"])), dtype=torch.float64, requires_grad=True)
    k = torch.tensor(float(np.float32(w["kgas"])), dtype=torch.float64, requires_grad=True)
    y = torch.tensor(w["target"], device=dev)
    xT, vT = rollout(adj, x0, v0, mu, k)
    loss = ((xT[:, :3].double() - y[:, :3].double()) ** 2).sum(dim=1).mean()
    loss.backward()
    assert np.allclose(xT.detach().cpu().numpy(), block16["xT"], rtol=0, atol=0)
    np.testing.assert_allclose(v0.grad.cpu().numpy()[:, :3], g["g_v0"][:, :3], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(x0.grad.cpu().numpy()[:, :3], g["g_x0"][:, :3], rtol=1e-5, atol=1e-12)
    assert mu.grad.item() == pytest.approx(g["g_mu"], rel=1e-5)
    assert k.grad.item() == pytest.approx(g["g_k"], rel=1e-5)


def test_flags_and_rejections(gpu_lib, block16):
    assert block16["adj"].flags() == 0
    w = workloads.adjoint_block(6, steps=4)
    for change in (dict(surface_tension=0.01), dict(mode=capi.SPH_MODE_COMPAT)):
        p = capi.SphParams.from_buffer_copy(w["params"])
        for a, b in change.items():
            setattr(p, a, b)
        ctx = workloads.build_context(w, p)
        with pytest.raises(capi.SphError):
            capi.Adjoint(ctx, 4, 2)
    ctx = workloads.build_context(w)
    ctx.add_boundary(w["fluid"][:8] + np.float32([0, 0.5, 0, 0]))
    with pytest.raises(capi.SphError):
        capi.Adjoint(ctx, 4, 2)
    ctx = workloads.build_context(w)
    a = capi.Adjoint(ctx, 4, 2)
    with pytest.raises(capi.SphError):
        a.backward(np.zeros((len(w["fluid"]), 4), np.float32))
