"""GPU quadratic mixed mode: a mesh mixing tets and hexes with quadratic
elements (element type T10 or H27 in flags bits 0-3) runs as GeoQuadratic3d
(XPBDFEM/Geo.cpp:836-1008): T10s and H27s in one body (xfem_qmixed.cu,
k_qmixed), through the C ABI.

Connectivity3d numbers the edges and quads over the interleaved stream,
GeoQuadratic3d sums the masses of every T10, then every H27, and each
sweep solves every T10, then every H27 (each volume pass, the Rayleigh and
the PBD damping likewise). Against the reference's own substeps run in the
GPU body's T10 and H27 colour orders (the `qmixed_*` fixtures, whose rest
state the host reproduces bit for bit) and against the pinned oracle on a
larger jittered block. Tolerances: positions within 1e-5 of max |x_ref|,
velocities within 1e-3 or 3x the spread of FP32 runs started one ulp
apart, whichever is larger; with an incompressible material or volume passes
within 3x the spread of FP32 runs about the FP64 run of the same method and
order (J - 1 at rest is FP32 rounding noise there, as on T10 meshes).
"""
import numpy as np
import pytest

import oracle
import xfem
from conftest import golden, golden_args
from helpers import QMixedOracleRun, rel

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
QMIXED = ["qmixed_c1_nh_nu045_checker", "qmixed_c1_nh_incompressible_left", "qmixed_wonky_yeohfast_serial_nu049_checker",
          "qmixed_c1_pixar_nu045_amortized_pbd_checker", "qmixed_c1_mixed_nu045_limit_left",
          "qmixed_wonky_nh_paper_volume_checker", "qmixed_c1_yeohskin_nu045_post_pbd_left"]


def _copy(s):
    return xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_})


def qmixed_settings(name):
    """Settings of a `qmixed` fixture (refgen's `mixed` argument order),
    element type T10."""
    a = golden_args(name)["args"]
    g = golden(name)
    dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock, damping, pbd, _drag, rtype, _spacing, vp = a[10:26]
    d = g["derived"]
    flags = (xfem.ELEMENT_T10 | (energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) |
             (xfem.LOCK_LEFT if lock else 0) | (rtype << 20))
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags, damping=damping,
                              pbd_damping=pbd, time_corrected_drag=float(d[2]),
                              volume_and_time_corrected_pbd_damping=float(d[0]),
                              amortized_volume_and_time_corrected_pbd_damping=float(d[1]), volume_passes=vp)
    return g, s, dens, dt, nsub


def _fp64_and_envelope(name, s, dens, dt, nsub, seeds=6):
    """The FP64 oracle run after one and nsub substeps, and the largest
    distances from it of the reference's own run and of FP32 oracle runs
    from rest positions perturbed by up to one float ulp (seeded)."""
    g = golden(name)
    o = QMixedOracleRun(g["nodes"], g["idx"], dens, _copy(s), g["torder"], g["horder"], dtype=np.float64)
    o.step(1, dt)
    X1 = o.X.copy()
    o.s.tick_id = 1
    o.step(nsub - 1, dt)
    Xn = o.X.copy()
    e1, en = rel(g["x1"].reshape(-1, 3), X1), rel(g["xn"].reshape(-1, 3), Xn)
    for seed in range(seeds):
        f = QMixedOracleRun(g["nodes"], g["idx"], dens, _copy(s), g["torder"], g["horder"])
        f.X = f.X * (1.0 + np.random.default_rng(seed).uniform(-1.0, 1.0, f.X.shape) * 2.0 ** -24)
        f.step(1, dt)
        e1 = max(e1, rel(f.X, X1))
        f.s.tick_id = 1
        f.step(nsub - 1, dt)
        en = max(en, rel(f.X, Xn))
    return X1, Xn, e1, en


@pytest.mark.parametrize("name", QMIXED)
def test_qmixed_reference_parity(name):
    g, s, dens, dt, nsub = qmixed_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    nt, nh = g["torder"].size, g["horder"].size
    assert b.counts[0][0] == g["x0"].size // 3
    assert b.t10_count()[0] == nt and b.h27_count()[0] == nh
    # the rest state (host) and both colourings are the reference's and the fixture's
    ept, w, t10, _ = b.t10_rest_state()
    eph, w2, h27 = b.h27_rest_state()
    assert np.array_equal(t10.reshape(-1), g["t10_idx"]) and np.array_equal(h27.reshape(-1), g["h27_idx"])
    assert np.array_equal(ept.reshape(-1).view(np.uint32), g["qep"].view(np.uint32))
    assert np.array_equal(eph.reshape(-1).view(np.uint32), g["h27ep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32)) and np.array_equal(w2, w)
    assert np.array_equal(b.positions(), g["x0"].reshape(-1, 3).astype(np.float32))
    ts, hs = b.t10_schedule(), b.h27_schedule()
    assert np.array_equal(ts["t10_order"], g["torder"]) and np.array_equal(ts["colour_t10_begin"], g["colour_t10_begin"])
    assert np.array_equal(hs["h27_order"], g["horder"]) and np.array_equal(hs["colour_h27_begin"], g["colour_h27_begin"])
    b.substep(dt)
    x1, v1 = b.positions(), b.velocities()
    b.step_frames(1, nsub - 1, dt)
    xn, vn = b.positions(), b.velocities()
    # CalculateVolume: the body's double sum against the oracle's at the body's positions
    q64 = oracle.QuadraticMixed(g["nodes"], g["idx"], dens, np.float64)
    v64 = q64.volume(xn.astype(np.float64))
    assert abs(b.volume() - v64) <= 1e-6 * abs(v64)
    if s.poissons_ratio >= 0.5 or s.volume_passes:
        # the trajectories of FP32 runs spread here (see the envelope), the
        # final volume with them: held against the oracle's at the body's positions
        X1, Xn, e1, en = _fp64_and_envelope(name, s, dens, dt, nsub)
        assert rel(x1, X1) <= 3 * e1 + 1e-7, (rel(x1, X1), e1)
        assert rel(xn, Xn) <= 3 * en + 1e-7, (rel(xn, Xn), en)
        return
    assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
    assert rel(xn, g["xn"].reshape(-1, 3)) <= 1e-5
    assert abs(b.volume() - float(g["volume"][0])) <= 1e-4 * abs(v64)
    # velocities: the first substep's are a displacement of 1e-5 of the
    # coordinates over dt, and FP32 runs started one ulp apart already
    # spread by up to 4e-3 on these meshes (positions by 1e-7)
    s1, sn = _velocity_spread(name, s, dens, dt, nsub)
    assert rel(v1, g["v1"].reshape(-1, 3)) <= max(1e-3, 3 * s1), s1
    assert rel(vn, g["vn"].reshape(-1, 3)) <= max(1e-3, 3 * sn), sn


def _velocity_spread(name, s, dens, dt, nsub, seeds=4):
    """The largest distance from the reference's velocities (after one and
    after nsub substeps) of FP32 oracle runs from rest positions perturbed by
    up to one float ulp (seeded)."""
    g = golden(name)
    s1 = sn = 0.0
    for seed in range(seeds):
        f = QMixedOracleRun(g["nodes"], g["idx"], dens, _copy(s), g["torder"], g["horder"])
        f.X = f.X * (1.0 + np.random.default_rng(seed).uniform(-1.0, 1.0, f.X.shape) * 2.0 ** -24)
        f.step(1, dt)
        s1 = max(s1, rel(f.V, g["v1"].reshape(-1, 3)))
        f.s.tick_id = 1
        f.step(nsub - 1, dt)
        sn = max(sn, rel(f.V, g["vn"].reshape(-1, 3)))
    return s1, sn


def jittered_qmixed_block():
    nodes, idx = oracle.mixed_block(5, 3, 3, (0.05, 0.05, 0.05), 1, 0.2, lambda x, y, z: (x * 7 + y * 3 + z) % 3 == 0)
    nodes = (nodes + np.random.default_rng(11).normal(0, 0.002, nodes.shape)).astype(np.float32)
    return nodes, idx


@pytest.mark.parametrize("energy,simultaneous,comp,nu,vpasses,damping,rtype,pbd", [
    (xfem.ENERGY_MIXED_SEL, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_MIXED_SEL, 0, 1e-3, 0.40, 0, 0.01, 0, 0.0),
    (xfem.ENERGY_YEOH_SKIN_FAST, 1, 0.5, 0.45, 0, 0.01, 1, 0.0),
    (xfem.ENERGY_MIXED, 1, 1e-3, 0.45, 0, 0.01, 3, 0.03),
    (xfem.ENERGY_PIXAR_SEL, 1, 1e-3, 0.40, 0, 0.01, 2, 0.05),
])
def test_qmixed_oracle_parity(energy, simultaneous, comp, nu, vpasses, damping, rtype, pbd):
    """A jittered mirrored block with a third of its cells split into tets,
    as T10s and H27s, 20 substeps against the oracle in the body's orders."""
    nodes, idx = jittered_qmixed_block()
    flags = (xfem.ELEMENT_H27 | (energy << xfem.ENERGY_BIT) | (simultaneous << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT |
             (rtype << 20))
    vc, avc = xfem.pbd_damping_coefficients(pbd, DT, 0.05)
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, volume_and_time_corrected_pbd_damping=vc,
                              amortized_volume_and_time_corrected_pbd_damping=avc, volume_passes=vpasses)
    b = xfem.Body(nodes, idx, 800.0, s)
    to, ho = b.t10_schedule()["t10_order"], b.h27_schedule()["h27_order"]
    o = QMixedOracleRun(nodes, idx, 800.0, _copy(s), to, ho)
    # two FP32 runs from starts one ulp away: the velocities' noise floor
    pert = []
    for seed in range(2):
        f = QMixedOracleRun(nodes, idx, 800.0, _copy(s), to, ho)
        f.X = f.X * (1.0 + np.random.default_rng(seed).uniform(-1.0, 1.0, f.X.shape) * 2.0 ** -24)
        pert.append(f)
    for n in (1, 19):
        b.step_frames(1, n, DT)
        for r in [o] + pert:
            r.step(n, DT)
            r.s.tick_id += n
        spread = max(rel(f.V, o.V) for f in pert)
        assert rel(b.positions(), o.X) <= 1e-5, n
        assert rel(b.velocities(), o.V) <= max(1e-3, 3 * spread), (n, spread)


def test_qmixed_batch_and_repeat():
    """Two quadratic mixed bodies in one handle step as they do alone, and
    runs repeat bit for bit in one call or one call per substep."""
    g, s, dens, dt, nsub = qmixed_settings("qmixed_c1_pixar_nu045_amortized_pbd_checker")
    g2, s2, dens2, _, _ = qmixed_settings("qmixed_wonky_yeohfast_serial_nu049_checker")
    alone = []
    for gg, ss, dd in ((g, s, dens), (g2, s2, dens2)):
        b = xfem.Body(gg["nodes"], gg["idx"], dd, ss)
        b.step_frames(1, 12, dt)
        alone.append(b.positions())
    batch = xfem.Body(meshes=[(g["nodes"], g["idx"], dens), (g2["nodes"], g2["idx"], dens2)], settings=[s, s2])
    batch.step_frames(1, 12, dt)
    for k in range(2):
        assert np.array_equal(batch.positions(k), alone[k]), k
    split = xfem.Body(g["nodes"], g["idx"], dens, s)
    for _ in range(12):
        split.substep(dt)
    assert np.array_equal(split.positions(), alone[0])
