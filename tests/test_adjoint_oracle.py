"""The FP64 adjoint oracle (oracle/sph_adjoint_oracle.cpp) against central finite
differences of its own forward step: checks the derivation the CUDA adjoint shares."""
import numpy as np
import pytest

from fluids_gb300 import capi, workloads
from oracle import adjoint as A


def _setup(n_side=8, steps=40):
    w = workloads.adjoint_block(n_side=n_side, steps=steps)
    d = capi.describe(w["params"], w["container"])
    mk = lambda: A.make_params(w["params"], d, w["container"], steps)   # noqa: E731
    y = w["target"][:, :3].astype(np.float64)
    return w, mk, y


def _loss(P, x0, v0, y):
    xT, _, mx = A.forward(P, x0, v0)
    return float(np.mean(np.sum((xT - y) ** 2, axis=1))), xT, mx


def test_adjoint_oracle_matches_central_differences():
    w, mk, y = _setup()
    P = mk()
    x0, v0 = w["fluid"], w["velocities"]
    n = len(x0)
    L0, xT, mx = _loss(P, x0, v0, y)
    assert mx < 50, "neighbour sets must stay below the list cap"
    g = A.backward(P, x0, v0, 2.0 * (xT - y) / n)
    for name, key in (("mu", "g_mu"), ("kgas", "g_k")):
        base = getattr(P, name)
        eps = base * 1e-4
        Pp, Pm = mk(), mk()
        setattr(Pp, name, base + eps)
        setattr(Pm, name, base - eps)
        fd = (_loss(Pp, x0, v0, y)[0] - _loss(Pm, x0, v0, y)[0]) / (2 * eps)
        assert abs(fd - g[key]) <= 1e-5 * abs(fd), (name, fd, g[key])
    rng = np.random.default_rng(5)
    for which, eps in (("v0", 1e-5), ("x0", 1e-7)):
        dd = rng.normal(size=(n, 3))
        base = (v0 if which == "v0" else x0).astype(np.float64)
        bp, bm = base.copy(), base.copy()
        bp[:, :3] += eps * dd
        bm[:, :3] -= eps * dd
        if which == "v0":
            fd = (_loss(P, x0, bp, y)[0] - _loss(P, x0, bm, y)[0]) / (2 * eps)
        else:
            fd = (_loss(P, bp, v0, y)[0] - _loss(P, bm, v0, y)[0]) / (2 * eps)
        ad = float(np.sum(g["g_" + which] * dd))
        assert abs(fd - ad) <= 1e-5 * abs(fd), (which, fd, ad)


def test_adjoint_oracle_linear_in_the_seed():
    """Reverse mode is linear in dL/dx_T: g(a u + b w) = a g(u) + b g(w)."""
    w, mk, y = _setup(n_side=6, steps=20)
    P = mk()
    x0, v0 = w["fluid"], w["velocities"]
    rng = np.random.default_rng(3)
    u, v = rng.normal(size=(len(x0), 3)), rng.normal(size=(len(x0), 3))
    gu, gv, gs = (A.backward(P, x0, v0, s) for s in (u, v, 2.0 * u - 3.0 * v))
    for k in ("g_x0", "g_v0"):
        np.testing.assert_allclose(gs[k], 2.0 * gu[k] - 3.0 * gv[k], rtol=1e-9, atol=1e-12)
    for k in ("g_mu", "g_k"):
        assert gs[k] == pytest.approx(2.0 * gu[k] - 3.0 * gv[k], rel=1e-9, abs=1e-18)
