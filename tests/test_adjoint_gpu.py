"""GPU adjoint (xfem_adjoint_forward / xfem_adjoint_backward through the C ABI)
against the FP64 oracle adjoint (itself pinned to FP64 central differences in
test_oracle_adjoint.py).

What is compared: the reverse pass is a vector-Jacobian product. Both sides
get the same cotangent G = dL/d(tip trajectory), taken from the FP64 run, so
the comparison measures the adjoint itself: max |g_gpu - g_fp64| <=
ADJ_TOL * max |g_fp64| for dL/dmu, dL/dV0 and dL/dX0 (float32 forward and
reverse against the FP64 derivative of the same method). The end-to-end
gradient of a tip loss (G from the GPU's own float trajectory) is checked in
test_beam_end_to_end with the bound stated there.

Bit-exact: checkpointed and full-tape runs, the two forms of the reverse
kernel, a batched handle against its bodies run alone, the recorded
trajectory against the plain forward, and the torch.autograd binding against
the C ABI. Every run starts from a freshly
created body: a lock zeroes the vertex's inverse mass at the end of the first
substep, so a handle that has stepped does not repeat its first run.
"""
import types

import numpy as np
import pytest

import oracle
import xfem
from helpers import rel
from xfem import workloads as W

pytestmark = pytest.mark.gpu

ADJ_TOL = 1e-3
DT = 1.0 / 1200.0
NU = 0.45


def _fp64(nodes, idx, density, s, dt, nsub, mu, tips, lock, V0, order, targets):
    """FP64 tip trajectory, cotangent G = 2 (x - target) and the oracle's VJP."""
    tets, nv = oracle.parse_tets(idx)
    ep, w, _ = oracle.init_rest(nodes, tets, density, np.float64)
    p = oracle.params_from_settings(s, dt)
    X0 = np.asarray(nodes, np.float64).reshape(-1, 3)
    mu64 = np.asarray(mu, np.float32).astype(np.float64)
    X, V, ww, traj = X0, V0, w, []
    for _ in range(nsub):
        X, V, ww, _ = oracle.substeps(X, V, ww, tets, ep, order, 1, p, lock_mask=lock, tet_mu=mu64, dtype=np.float64)
        traj.append(X[tips])
    traj = np.array(traj)
    if targets is None:
        targets = traj + 1e-3 * np.random.default_rng(11).normal(size=traj.shape)
    L, dmu, dv, dx = oracle.adjoint(X0, V0, w, tets, ep, mu64, order, nsub, p, tips, targets, lock, want_dx=True)
    return traj, targets, L, dmu, dv, dx


class Case:
    """One differentiation case: mesh, settings, per-tet mu, tips, V0 and the
    FP64 reference. fresh() makes a new body in the initial state."""

    def __init__(self, nodes, idx, s, nsub, mu, tips, V0=None, lock=None, cluster_mode=0, targets=None, dt=DT):
        self.nodes, self.idx, self.s, self.nsub, self.dt = nodes, idx, s, nsub, dt
        self.mu = np.asarray(mu, np.float32)
        self.tips = np.asarray(tips, np.uint32)
        nv = nodes.size // 3
        self.V0 = np.zeros((nv, 3)) if V0 is None else np.asarray(V0, np.float32).astype(np.float64)
        tets, _ = oracle.parse_tets(idx)
        _, _, fl = oracle.init_rest(nodes, tets, 1000.0, np.float32)
        self.lock = (fl & 1).astype(np.uint8) if lock is None else np.asarray(lock, np.uint8)
        self.cluster_mode = cluster_mode
        order = self.fresh().schedule()["tet_order"]
        self.traj64, self.targets, self.L, self.dmu, self.dv, self.dx = _fp64(
            nodes, idx, 1000.0, s, dt, nsub, self.mu, self.tips, self.lock, self.V0, order, targets)
        self.G = (2.0 * (self.traj64 - self.targets)).astype(np.float32)

    def fresh(self):
        b = xfem.Body(self.nodes, self.idx, 1000.0, self.s, cluster_mode=self.cluster_mode)
        b.set_lock_mask(self.lock)
        b.set_tet_mu(self.mu)
        b.set_velocities(self.V0.astype(np.float32))
        return b

    def gpu(self, K=0, G=None, body=None):
        b = self.fresh() if body is None else body
        traj = b.adjoint_forward(self.nsub, self.dt, self.tips, K)
        dmu, dx, dv = b.adjoint_backward(self.G if G is None else G)
        return types.SimpleNamespace(traj=traj, dmu=dmu, dx=dx, dv=dv, body=b)

    def check(self, r, tol=ADJ_TOL, traj_tol=1e-5):
        assert rel(r.traj, self.traj64) <= traj_tol
        for name, a, b in (("dmu", r.dmu, self.dmu), ("dV0", r.dv, self.dv), ("dX0", r.dx, self.dx)):
            e = rel(a, b)
            assert e <= tol, (name, e)


def _nh(**kw):
    return W.default_settings(gravity=(0, 0, -9.81), compliance=W.nh_compliance(1e5, NU), poissons_ratio=NU, **kw)


def cantilever(nsub=30, cluster_mode=0):
    nodes, idx = W.box(6, 2, 2, 0.05)
    s = _nh(flags=W.NH_FLAGS)
    nt, nv = idx.size // 5, nodes.size // 3
    mu = (1.0 / s["compliance"]) * np.exp(0.3 * np.random.default_rng(3).normal(size=nt))
    V0 = np.zeros((nv, 3), np.float32)
    V0[:, 0] = 0.2
    return Case(nodes, idx, s, nsub, mu, np.arange(nv - 10, nv), V0=V0, cluster_mode=cluster_mode)


def ground_box(nsub=40):
    nodes, idx = W.box(6, 2, 2, 0.05)
    n = np.asarray(nodes, np.float64).reshape(-1, 3)
    n = (n - n.mean(0)) @ W.random_rotation(W.Rng(5)).T
    n[:, 2] += 0.003 - n[:, 2].min()
    nodes = n.astype(np.float32).reshape(-1)
    s = _nh(flags=W.NH_FLAGS & ~W.LOCK_LEFT, ground=1, friction=0.4)
    nt, nv = idx.size // 5, nodes.size // 3
    mu = (1.0 / s["compliance"]) * np.exp(0.3 * np.random.default_rng(4).normal(size=nt))
    V0 = np.zeros((nv, 3), np.float32)
    V0[:, 0] = 0.3
    V0[:, 2] = -0.5
    return Case(nodes, idx, s, nsub, mu, np.arange(0, nv, 7), V0=V0)


def test_cantilever_cube_path():
    c = cantilever()
    c.check(c.gpu())


def test_ground_friction():
    c = ground_box()
    r = c.gpu()
    assert r.body.contacts().sum() > 0
    c.check(r)


def test_one_tet_clusters():
    """cluster_mode 1 (one tet per cluster): the general chunk path."""
    c = cantilever(cluster_mode=1)
    c.check(c.gpu())


def test_checkpointed_equals_full_tape():
    """Segments re-run from checkpoints give the full tape's results bit for
    bit, and leave the handle at the end of the forward run."""
    c = cantilever()
    full = c.gpu()
    x_end = full.body.positions()
    for K in (7, 10, 1):
        ck = c.gpu(K=K)
        for k in ("traj", "dmu", "dx", "dv"):
            assert np.array_equal(getattr(full, k), getattr(ck, k)), (K, k)
        assert np.array_equal(ck.body.positions(), x_end), K


@pytest.mark.parametrize("make", [cantilever, ground_box, lambda: cantilever(cluster_mode=1)])
def test_reverse_forms_agree(make, monkeypatch):
    """The grouped reverse (8 lanes per cube cluster, the forward internals of
    its six solves recomputed side by side) and the one-lane reverse give the
    same gradients bit for bit; the small meshes here take the grouped form
    unless told otherwise."""
    c = make()
    runs = {}
    for form in ("grouped", "lane"):
        monkeypatch.setenv("XFEM_REVERSE_FORM", form)
        runs[form] = c.gpu(K=7)
    for k in ("traj", "dmu", "dx", "dv"):
        assert np.array_equal(runs["grouped"].__dict__[k], runs["lane"].__dict__[k]), k
    c.check(runs["grouped"])


def test_trajectory_is_the_plain_forward():
    """The recording forward is the plain forward, bit for bit."""
    c = cantilever(nsub=12)
    rec = c.fresh()
    traj = rec.adjoint_forward(c.nsub, c.dt, c.tips)
    plain = c.fresh()
    for k in range(c.nsub):
        plain.step_frames(1, 1, c.dt)
        assert np.array_equal(plain.positions()[c.tips], traj[k]), k
    assert np.array_equal(plain.positions(), rec.positions())
    assert np.array_equal(plain.velocities(), rec.velocities())


def test_batched_handle_matches_single_bodies():
    """Two bodies in one handle: each body's gradients as when run alone, bit for bit."""
    c1, c2 = cantilever(), ground_box()
    n = min(c1.nsub, c2.nsub)
    r1 = c1.gpu(G=c1.G[:n]) if c1.nsub == n else None
    b1, b2 = c1.fresh(), c2.fresh()
    t1 = b1.adjoint_forward(n, DT, c1.tips)
    g1 = b1.adjoint_backward(c1.G[:n])
    t2 = b2.adjoint_forward(n, DT, c2.tips)
    g2 = b2.adjoint_backward(c2.G[:n])
    B = xfem.Body(meshes=[(c1.nodes, c1.idx, 1000.0), (c2.nodes, c2.idx, 1000.0)], settings=[c1.s, c2.s])
    nv1 = c1.nodes.size // 3
    for bi, c in enumerate((c1, c2)):
        B.set_lock_mask(c.lock, bi)
        B.set_tet_mu(c.mu, bi)
        B.set_velocities(c.V0.astype(np.float32), bi)
    tb = B.adjoint_forward(n, DT, np.concatenate([c1.tips, c2.tips + nv1]))
    gb = B.adjoint_backward(np.concatenate([c1.G[:n], c2.G[:n]], axis=1))
    assert np.array_equal(tb, np.concatenate([t1, t2], axis=1))
    for k in range(3):
        assert np.array_equal(gb[k], np.concatenate([g1[k], g2[k]])), k
    if r1 is not None:
        assert np.array_equal(r1.dmu, g1[0])


def test_torch_autograd_binding():
    """loss.backward() through xfem.autograd.substeps: the C ABI's results,
    and a loss on the final state equals the same loss on the last trajectory row."""
    torch = pytest.importorskip("torch")
    from xfem import autograd as XA
    c = cantilever()
    ref = c.gpu(G=None)
    body = c.fresh()
    mu = torch.tensor(c.mu, requires_grad=True)
    x0 = torch.tensor(c.nodes.reshape(-1, 3), requires_grad=True)
    v0 = torch.tensor(c.V0.astype(np.float32), requires_grad=True)
    traj, x1, v1 = XA.substeps(body, mu, x0, v0, c.nsub, c.dt, c.tips)
    assert np.array_equal(traj.detach().numpy(), ref.traj)
    traj.backward(torch.from_numpy(c.G))
    assert np.array_equal(mu.grad.numpy(), ref.dmu)
    assert np.array_equal(x0.grad.numpy(), ref.dx)
    assert np.array_equal(v0.grad.numpy(), ref.dv)
    # final-state cotangent on the tips == the same cotangent on traj[-1]
    gl = torch.from_numpy(np.random.default_rng(2).normal(size=(c.tips.size, 3)).astype(np.float32))
    mu_a, mu_b = (torch.tensor(c.mu, requires_grad=True) for _ in range(2))
    xa = torch.tensor(c.nodes.reshape(-1, 3))
    va = torch.tensor(c.V0.astype(np.float32))
    ta, x1a, _ = XA.substeps(c.fresh(), mu_a, xa, va, c.nsub, c.dt, c.tips)
    (x1a[torch.from_numpy(c.tips.astype(np.int64))] * gl).sum().backward()
    tb_, _, _ = XA.substeps(c.fresh(), mu_b, xa, va, c.nsub, c.dt, c.tips)
    (tb_[-1] * gl).sum().backward()
    assert np.array_equal(mu_a.grad.numpy(), mu_b.grad.numpy())
    # checkpointed binding
    mu_c = torch.tensor(c.mu, requires_grad=True)
    tc, _, _ = XA.substeps(c.fresh(), mu_c, xa, va, c.nsub, c.dt, c.tips, checkpoint_every=8)
    tc.backward(torch.from_numpy(c.G))
    assert np.array_equal(mu_c.grad.numpy(), ref.dmu)


def test_unsupported_model_is_rejected():
    nodes, idx = W.box(4, 2, 2, 0.05)
    b = xfem.Body(nodes, idx, 1000.0, W.default_settings(flags=W.YEOH_FLAGS))
    with pytest.raises(xfem.XfemError):
        b.adjoint_forward(4, DT, np.array([0], np.uint32))
    with pytest.raises(xfem.XfemError):
        b.adjoint_backward(np.zeros((4, 1, 3), np.float32))


@pytest.fixture(scope="module")
def beam():
    """The 32x8x8 beam (12,288 tets), 200 substeps, 20 tips; the target is the
    FP64 tip trajectory under the second modulus field."""
    d = W.adjoint_beam()
    tets, _ = oracle.parse_tets(d["idx"])
    ep, w, _ = oracle.init_rest(d["nodes"], tets, d["density"], np.float64)
    order = xfem.Body(d["nodes"], d["idx"], d["density"], d["settings"]).schedule()["tet_order"]
    p = oracle.params_from_settings(d["settings"], d["dt"])
    X = np.asarray(d["nodes"], np.float64).reshape(-1, 3)
    V, ww, tgt = np.zeros_like(X), w, []
    for _ in range(d["substeps"]):
        X, V, ww, _ = oracle.substeps(X, V, ww, tets, ep, order, 1, p, lock_mask=d["lock"],
                                      tet_mu=d["mu_target"].astype(np.float64), dtype=np.float64)
        tgt.append(X[d["tips"]])
    c = Case(d["nodes"], d["idx"], d["settings"], d["substeps"], d["mu"], d["tips"], lock=d["lock"],
             targets=np.array(tgt), dt=d["dt"])
    c.tets, c.ep, c.w, c.order, c.p = tets, ep, w, order, p
    return c


def test_beam_vjp(beam):
    r = beam.gpu()
    beam.check(r)
    ck = beam.gpu(K=20)
    assert np.array_equal(ck.dmu, r.dmu)


def test_beam_fd(beam):
    """GPU dL/dlog(mu) of the ten most sensitive tets and dL/dV0 of the three
    largest initial-velocity entries against FP64 central differences of the
    FP64 loss (h = 1e-3 in log mu, 1e-5 m/s in V0), each within 1e-3 of the
    largest |FD| of its kind among the checked entries (1e-3 relative, on
    the scale of the gradient)."""
    c = beam
    r = c.gpu()
    X0 = np.asarray(c.nodes, np.float64).reshape(-1, 3)
    mu64 = c.mu.astype(np.float64)

    def loss(m, V0=None):
        return oracle.adjoint(X0, c.V0 if V0 is None else V0, c.w, c.tets, c.ep, m, c.order, c.nsub, c.p, c.tips,
                              c.targets, c.lock, grad=False)

    h = 1e-3
    pairs = []
    for t in np.argsort(-np.abs(c.dmu * mu64))[:10]:
        mp, mm = mu64.copy(), mu64.copy()
        mp[t] *= np.exp(h)
        mm[t] *= np.exp(-h)
        pairs.append((t, (loss(mp) - loss(mm)) / (2 * h), float(r.dmu[t]) * mu64[t]))
    scale = max(abs(fd) for _, fd, _ in pairs)
    for t, fd, ad in pairs:
        assert abs(ad - fd) <= ADJ_TOL * scale, ("dlogmu", t, fd, ad, scale)
    hv = 1e-5
    dv = np.asarray(r.dv).reshape(-1)
    vpairs = []
    for k in np.argsort(-np.abs(np.asarray(c.dv).reshape(-1)))[:3]:
        vp, vm = c.V0.copy().reshape(-1), c.V0.copy().reshape(-1)
        vp[k] += hv
        vm[k] -= hv
        fd = (loss(mu64, vp.reshape(-1, 3)) - loss(mu64, vm.reshape(-1, 3))) / (2 * hv)
        vpairs.append((k, fd, float(dv[k])))
    vscale = max(abs(fd) for _, fd, _ in vpairs)
    for k, fd, ad in vpairs:
        assert abs(ad - fd) <= ADJ_TOL * vscale, ("dV0", k, fd, ad, vscale)


def test_beam_end_to_end(beam):
    """The gradient of the tip loss with G from the GPU's own float32
    trajectory. The loss compares two nearby trajectories (tip residuals of
    ~3e-5 m against positions of ~1 m), so the float forward's rounding of
    the positions (about 6e-8 m per substep at 1 m) enters G directly, at
    ~1e-3 of it: measured 1.75e-3 of max |g| on a GB300, against the 1e-3
    that the same reverse pass meets with the FP64 cotangent
    (test_beam_vjp). Bound: 2.5e-3 of max |g| and cosine >= 0.999."""
    c = beam
    r0 = c.gpu()
    G = (2.0 * (r0.traj.astype(np.float64) - c.targets)).astype(np.float32)
    r = c.gpu(G=G)
    e = rel(r.dmu, c.dmu)
    print(f"end-to-end dL/dmu error vs FP64: {e:.3e}")
    assert e <= 2.5e-3, e
    cos = float(np.dot(r.dmu, c.dmu) / (np.linalg.norm(r.dmu) * np.linalg.norm(c.dmu)))
    assert cos >= 0.999, cos
