"""The FP64 adjoint oracle against FP64 central finite differences (CPU only).

The oracle's reverse pass (oracle/xfem_oracle_adjoint.c) is the reference the
GPU adjoint is checked against, so it is pinned here first: d loss / d log mu
per tet, d loss / d V0 and d loss / d X0 per vertex component, each against a
central difference of the oracle's own FP64 forward loss. h = 1e-3 in log mu
(1e-5 in velocity, 1e-6 in position) keeps the O(h^2) truncation near 1e-6
of the derivative; the loss itself carries rounding noise of about 1e-13 L,
so each comparison allows FD_TOL relative error plus NOISE * L / h absolute.
"""
import types

import numpy as np
import pytest

import oracle
from xfem import workloads as W

FD_TOL = 2e-4
NOISE = 1e-12


def _case(ground, nsub=30):
    nodes, idx = W.box(6, 2, 2, 0.05)
    n = np.asarray(nodes, np.float64).reshape(-1, 3)
    if ground:
        R = W.random_rotation(W.Rng(5))
        n = (n - n.mean(0)) @ R.T
        n[:, 2] += 0.003 - n[:, 2].min()
    nodes = n.astype(np.float32).reshape(-1)
    tets, nv = oracle.parse_tets(idx)
    ep, w, fl = oracle.init_rest(nodes, tets, 1000.0, np.float64)
    order = oracle.schedule(nodes, tets, 1, 1)["tet_order"]
    nu = 0.45
    flags = W.NH_FLAGS & ~W.LOCK_LEFT if ground else W.NH_FLAGS
    s = W.default_settings(gravity=(0, 0, -9.81), compliance=W.nh_compliance(1e5, nu), poissons_ratio=nu,
                           flags=flags, ground=int(ground), friction=0.4)
    p = oracle.params_from_settings(s, 1.0 / 1200.0)
    rng = np.random.default_rng(1)
    mu = (1.0 / s["compliance"]) * np.exp(0.3 * rng.normal(size=tets.shape[0]))
    tips = np.arange(nv - 10, nv, dtype=np.uint32)
    X0 = nodes.reshape(-1, 3).astype(np.float64)
    V0 = np.zeros_like(X0)
    V0[:, 0] = 0.2
    if ground:
        V0[:, 2] = -0.5
    lock = (fl & 1).astype(np.uint8)
    targets = np.repeat(X0[tips][None], nsub, 0) + 1e-3 * rng.normal(size=(nsub, tips.size, 3))

    def loss(m=mu, v=V0, x=X0):
        return oracle.adjoint(x, v, w, tets, ep, m, order, nsub, p, tips, targets, lock, grad=False)

    def grads():
        return oracle.adjoint(X0, V0, w, tets, ep, mu, order, nsub, p, tips, targets, lock, want_dx=True)

    def forward_loss():
        X, V, ww = X0, V0, w
        total = 0.0
        for k in range(nsub):
            X, V, ww, _ = oracle.substeps(X, V, ww, tets, ep, order, 1, p, lock_mask=lock, tet_mu=mu,
                                          dtype=np.float64)
            total += float(((X[tips] - targets[k]) ** 2).sum())
        return total

    return types.SimpleNamespace(mu=mu, V0=V0, X0=X0, tips=tips, loss=loss, grads=grads, forward_loss=forward_loss)


def _central(f, a, idx, h, scale=False):
    ap, am = a.copy(), a.copy()
    if scale:
        ap[idx] *= np.exp(h)
        am[idx] *= np.exp(-h)
    else:
        ap[idx] += h
        am[idx] -= h
    return (f(ap) - f(am)) / (2 * h)


@pytest.mark.parametrize("ground", [False, True], ids=["cantilever", "ground_friction"])
def test_adjoint_vs_central_fd(ground):
    c = _case(ground)
    L, dmu, dv, dx = c.grads()
    assert L > 0 and np.isfinite(dmu).all() and np.isfinite(dv).all() and np.isfinite(dx).all()
    for t in [0, 7, 33, 50, 70]:
        h = 1e-3
        fd = _central(lambda m: c.loss(m=m), c.mu, t, h, scale=True)
        ad = dmu[t] * c.mu[t]
        assert abs(fd - ad) <= FD_TOL * abs(fd) + NOISE * L / h, (t, fd, ad)
    for (i, k) in [(int(c.tips[0]), 0), (int(c.tips[3]), 2), (5, 1), (int(c.tips[-1]), 1)]:
        h = 1e-5
        fd = _central(lambda v: c.loss(v=v), c.V0, (i, k), h)
        assert abs(fd - dv[i, k]) <= FD_TOL * abs(fd) + NOISE * L / h, (i, k, fd, dv[i, k])
    for (i, k) in [(int(c.tips[1]), 0), (int(c.tips[2]), 2), (3, 1), (40, 2)]:
        h = 1e-6
        fd = _central(lambda x: c.loss(x=x), c.X0, (i, k), h)
        assert abs(fd - dx[i, k]) <= FD_TOL * abs(fd) + NOISE * L / h, (i, k, fd, dx[i, k])


@pytest.mark.parametrize("ground", [False, True], ids=["cantilever", "ground_friction"])
def test_adjoint_loss_equals_forward(ground):
    """The adjoint's forward loss is the tip loss of the FP64 substep run."""
    c = _case(ground, nsub=12)
    L = c.loss()
    assert np.isfinite(L) and L > 0
    assert c.grads()[0] == L
    assert abs(L - c.forward_loss()) <= 1e-12 * L
