"""Test helpers: run the oracle on the same inputs and schedule as a GPU body."""
import numpy as np

import oracle
import xfem


def oracle_params(s, dt, lock=True, nodes=None):
    """orc_params from an xfem Settings struct or settings dict (nodes: the
    rest positions, for the Right lock's targets)."""
    return oracle.params_from_settings(s, dt, lock, nodes=nodes)


def rel(a, b):
    """max |a - b| over max |b| (the error relative to the quantity's scale)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


class OracleRun:
    """The oracle's state for one body, stepped in the body's own schedule."""

    def __init__(self, nodes, idx, density, settings, order, lock_mask=None, tet_mu=None, dtype=np.float32):
        self.tets, nv = oracle.parse_tets(idx)
        self.ep, self.w, fl = oracle.init_rest(nodes, self.tets, density, dtype)
        # bit 0: the Left lock (or the caller's mask), bit 1: the Right flag
        self.lock = ((fl & 1) if lock_mask is None else np.asarray(lock_mask, np.uint8) & 1) | (fl & 2)
        self.lock = self.lock.astype(np.uint8)
        self.nodes = np.asarray(nodes, np.float32).reshape(-1)
        self.X = np.asarray(nodes, np.float64).reshape(-1, 3).copy()
        self.V = np.zeros_like(self.X)
        self.s = settings
        self.order = order
        self.tet_mu = tet_mu
        self.dtype = dtype
        self.contact = None
        self.lam = None

    def step(self, n, dt):
        p = oracle_params(self.s, dt, nodes=self.nodes)
        self.X, self.V, self.w, self.contact, self.lam = oracle.substeps(
            self.X, self.V, self.w, self.tets, self.ep, self.order, n, p, lock_mask=self.lock,
            tet_mu=self.tet_mu, dtype=self.dtype, want_lambdas=True)
        return self


class HexOracleRun:
    """The oracle's state for one hex body, stepped in the body's hex order
    (and with vorder, a continuous-pressure model's ring order)."""

    def __init__(self, nodes, idx, density, settings, order, dtype=np.float32, vorder=None):
        self.hexes, nv = oracle.parse_hexes(idx)
        self.ep, self.w, fl = oracle.hex_init_rest(nodes, self.hexes, density, dtype)
        self.lock = (fl & 3).astype(np.uint8)
        self.nodes = np.asarray(nodes, np.float32).reshape(-1)
        self.X = np.asarray(nodes, np.float64).reshape(-1, 3).copy()
        self.V = np.zeros_like(self.X)
        self.s = settings
        self.order = order
        self.vorder = vorder
        self.dtype = dtype

    def step(self, n, dt):
        p = oracle_params(self.s, dt, nodes=self.nodes)
        if self.vorder is not None:
            self.X, self.V, self.w, _ = oracle.hex_substeps_rings(self.X, self.V, self.w, self.hexes, self.ep, self.order,
                                                                  self.vorder, n, p, lock_mask=self.lock,
                                                                  dtype=self.dtype)
            return self
        self.X, self.V, self.w, _ = oracle.hex_substeps(self.X, self.V, self.w, self.hexes, self.ep, self.order, n, p,
                                                        lock_mask=self.lock, dtype=self.dtype)
        return self


class MixedOracleRun:
    """The oracle's state for one mesh mixing tets and hexes, stepped in the
    body's tet and hex colour orders."""

    def __init__(self, nodes, idx, density, settings, torder, horder, dtype=np.float32):
        self.tets, self.hexes, nv = oracle.parse_mixed(idx)
        self.ep, self.hep, self.w, fl = oracle.mixed_init_rest(nodes, self.tets, self.hexes, density, dtype)
        self.lock = (fl & 3).astype(np.uint8)
        self.nodes = np.asarray(nodes, np.float32).reshape(-1)
        self.X = np.asarray(nodes, np.float64).reshape(-1, 3).copy()
        self.V = np.zeros_like(self.X)
        self.s = settings
        self.torder = torder
        self.horder = horder
        self.dtype = dtype
        self.contact = None

    def step(self, n, dt):
        p = oracle_params(self.s, dt, nodes=self.nodes)
        self.X, self.V, self.w, self.contact = oracle.mixed_substeps(
            self.X, self.V, self.w, self.tets, self.ep, self.torder, self.hexes, self.hep, self.horder, n, p,
            lock_mask=self.lock, dtype=self.dtype)
        return self


class QMixedOracleRun:
    """The oracle's state for one mesh mixing tets and hexes read as T10s and
    H27s (GeoQuadratic3d), stepped in the body's T10 and H27 colour orders."""

    def __init__(self, nodes, idx, density, settings, torder, horder, dtype=np.float32):
        self.q = oracle.QuadraticMixed(nodes, idx, density, dtype)
        self.lock = (self.q.flags & 3).astype(np.uint8)
        self.nodes = self.q.X0.astype(np.float32).reshape(-1)
        self.X = self.q.X0.copy()
        self.V = np.zeros_like(self.X)
        self.w = self.q.w.copy()
        self.s = settings
        self.torder = torder
        self.horder = horder

    def step(self, n, dt):
        p = oracle_params(self.s, dt, nodes=self.nodes)
        self.X, self.V, self.w, _ = self.q.substeps(self.X, self.V, self.w, self.torder, self.horder, n, p,
                                                    lock_mask=self.lock)
        return self


class T10OracleRun:
    """The oracle's state for one tet mesh read as T10s (GeoQuadratic3d),
    stepped in the body's T10 order."""

    def __init__(self, nodes, idx, density, settings, order, dtype=np.float32, vorder=None):
        self.q = oracle.Quadratic(nodes, idx, density, dtype)
        self.lock = (self.q.flags & 3).astype(np.uint8)
        self.nodes = self.q.X0.astype(np.float32).reshape(-1)
        self.X = self.q.X0.copy()
        self.V = np.zeros_like(self.X)
        self.w = self.q.w.copy()
        self.s = settings
        self.order = order
        self.vorder = vorder  # a continuous-pressure model's ring order

    def step(self, n, dt):
        p = oracle_params(self.s, dt, nodes=self.nodes)
        if self.vorder is not None:
            self.X, self.V, self.w, _ = self.q.substeps_rings(self.X, self.V, self.w, self.order, self.vorder, n, p,
                                                              lock_mask=self.lock)
            return self
        self.X, self.V, self.w, _ = self.q.substeps(self.X, self.V, self.w, self.order, n, p, lock_mask=self.lock)
        return self


def envelope(make_run, checkpoints, dt, seeds=8):
    """FP64 states at each checkpoint (substep counts) and how far FP32 runs
    of the method land from them: the largest distance over the FP32 oracle
    started from the rest positions perturbed by up to one float ulp
    (seeded). With an incompressible material or volume passes the FP32
    rounding of J grows chaotically, on T10s within the first substep, and
    single runs spread over an order of magnitude. make_run(dtype) gives a
    fresh oracle run (T10OracleRun, H27OracleRun)."""
    ref = []
    o = make_run(np.float64)
    done = 0
    for n in checkpoints:
        o.step(n - done, dt)
        o.s.tick_id = n
        done = n
        ref.append((o.X.copy(), o.V.copy()))
    env = [[0.0, 0.0] for _ in checkpoints]
    for seed in range(seeds):
        r = make_run(np.float32)
        r.X = r.X * (1.0 + np.random.default_rng(seed).uniform(-1.0, 1.0, r.X.shape) * 2.0 ** -24)
        done = 0
        for k, n in enumerate(checkpoints):
            r.step(n - done, dt)
            r.s.tick_id = n
            done = n
            env[k][0] = max(env[k][0], rel(r.X, ref[k][0]))
            env[k][1] = max(env[k][1], rel(r.V, ref[k][1]))
    return ref, env


class H27OracleRun:
    """The oracle's state for one hex mesh read as H27s (GeoQuadratic3d),
    stepped in the body's H27 order (and with vorder, a continuous-pressure
    model's ring order)."""

    def __init__(self, nodes, idx, density, settings, order, dtype=np.float32, vorder=None):
        self.q = oracle.QuadraticHex(nodes, idx, density, dtype)
        self.lock = (self.q.flags & 3).astype(np.uint8)
        self.nodes = self.q.X0.astype(np.float32).reshape(-1)
        self.X = self.q.X0.copy()
        self.V = np.zeros_like(self.X)
        self.w = self.q.w.copy()
        self.s = settings
        self.order = order
        self.vorder = vorder

    def step(self, n, dt):
        p = oracle_params(self.s, dt, nodes=self.nodes)
        if self.vorder is not None:
            self.X, self.V, self.w, _ = self.q.substeps_rings(self.X, self.V, self.w, self.order, self.vorder, n, p,
                                                              lock_mask=self.lock)
            return self
        self.X, self.V, self.w, _ = self.q.substeps(self.X, self.V, self.w, self.order, n, p, lock_mask=self.lock)
        return self
