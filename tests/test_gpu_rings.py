"""GPU one-ring mode: the continuous-pressure models (energy 8-10), one
constraint (pair) per vertex over the tets around it (SolveRing,
XPBDFEM/Geo.cpp:147-193; CalculateElementEnergyAndGradients,
XPBDFEM/Fem.cpp:942-979; SolveSimplex, XPBDFEM/Geo.cpp:12-64).

Against the reference's own substeps run in the GPU body's ring order (the
`rings_*` fixtures of tests/golden, with in-solve and post-step damping) and
against the pinned oracle on a larger jittered mesh. Positions within 1e-5 of max |x_ref|; velocities within 1e-3,
or for the incompressible case within 3x the reference's own FP32 distance
from the FP64 run (as for the element models at nu = 0.5).
"""
import numpy as np
import pytest

import oracle
import xfem
from conftest import golden, golden_args
from helpers import rel
from test_gpu_models import fixture_settings

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
RINGS = ["rings_c1_cpixar_nu045_star", "rings_c1_cmixed_nu045_star", "rings_c1_cmixed_incompressible_star",
         "rings_c1_cskin_nu049_star", "rings_wonky_cmixed_paper_star", "rings_c1_cskin_limit_star",
         "rings_c1_cmixed_amortized_pbd_star", "rings_wonky_cpixar_post_star"]


def _fp64(name, s, nsub):
    g = golden(name)
    a = golden_args(name)["args"]
    tets, _ = oracle.parse_tets(g["idx"])
    ep, w, fl = oracle.init_rest(g["nodes"], tets, a[8], np.float64)
    X0 = g["nodes"].astype(np.float64)
    lm = (fl & 1).astype(np.uint8)
    p = oracle.params_from_settings(s, DT)
    X1, V1, w1, _ = oracle.substeps_rings(X0, np.zeros_like(X0), w, tets, ep, g["order"], g["vorder"], 1, p,
                                          lock_mask=lm, dtype=np.float64)
    p.tick = 1
    Xn, Vn, _, _ = oracle.substeps_rings(X1, V1, w1, tets, ep, g["order"], g["vorder"], nsub - 1, p, lock_mask=lm,
                                         dtype=np.float64)
    return X1, V1, Xn, Vn


@pytest.mark.parametrize("name", RINGS)
def test_ring_reference_parity(name):
    g, s, dens, dt, nsub, mode = fixture_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s, cluster_mode=mode)
    rs = b.ring_schedule()
    assert np.array_equal(rs["vert_order"], g["vorder"])
    assert np.array_equal(rs["colour_vert_begin"], g["colour_vert_begin"])
    b.substep(dt)
    x1, v1 = b.positions(), b.velocities()
    b.step_frames(1, nsub - 1, dt)
    xn, vn = b.positions(), b.velocities()
    if s.poissons_ratio < 0.5:
        assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
        assert rel(v1, g["v1"].reshape(-1, 3)) <= 1e-3
        assert rel(xn, g["xn"].reshape(-1, 3)) <= 1e-5
        assert rel(vn, g["vn"].reshape(-1, 3)) <= 1e-3
    else:
        X1, V1, Xn, Vn = _fp64(name, s, nsub)
        for got, ref, f64 in ((x1, g["x1"], X1), (v1, g["v1"], V1), (xn, g["xn"], Xn), (vn, g["vn"], Vn)):
            e_ref = rel(ref.reshape(-1, 3), f64)
            assert rel(got, f64) <= 3 * e_ref + 1e-7, (e_ref, rel(got, f64))


@pytest.mark.parametrize("energy,nu,comp,damping,rtype,pbd", [
    (xfem.ENERGY_CONTINUOUS_PIXAR, 0.45, 1e-3, 0.0, 2, 0.0),
    (xfem.ENERGY_CONTINUOUS_MIXED, 0.40, 1e-3, 0.01, 0, 0.0),
    (xfem.ENERGY_CONTINUOUS_SKIN, 0.45, 0.5, 0.01, 1, 0.0),
    (xfem.ENERGY_CONTINUOUS_MIXED, 0.45, 1e-3, 0.01, 3, 0.03),
    (xfem.ENERGY_CONTINUOUS_PIXAR, 0.45, 1e-3, 0.02, 2, 0.05),
])
def test_ring_oracle_parity(energy, nu, comp, damping, rtype, pbd):
    """A larger jittered block over 20 substeps against the oracle run in the
    body's ring order."""
    nodes, idx = xfem.generate_tet_block(6, 3, 2, (0.05, 0.05, 0.05), 1, 0.0)
    rng = np.random.default_rng(9)
    nodes = (nodes + rng.normal(0, 0.003, nodes.shape)).astype(np.float32)
    flags = (energy << xfem.ENERGY_BIT) | (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | (rtype << 20)
    vc, avc = xfem.pbd_damping_coefficients(pbd, DT, 0.05)
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, volume_and_time_corrected_pbd_damping=vc,
                              amortized_volume_and_time_corrected_pbd_damping=avc)
    b = xfem.Body(nodes, idx, 800.0, s)
    tets, _ = oracle.parse_tets(idx)
    ep, w, fl = oracle.init_rest(nodes, tets, 800.0)
    vorder = b.ring_schedule()["vert_order"]
    torder = b.schedule()["tet_order"]
    X, V, w_ = nodes.astype(np.float64).reshape(-1, 3), np.zeros((nodes.size // 3, 3)), w
    lm = (fl & 1).astype(np.uint8)
    tick = 0
    for n in (1, 19):
        b.step_frames(1, n, DT)
        X, V, w_, _ = oracle.substeps_rings(X, V, w_, tets, ep, torder, vorder, n,
                                            oracle.params_from_settings(s, DT, tick=tick), lock_mask=lm)
        tick += n
        assert rel(b.positions(), X) <= 1e-5, n
        assert rel(b.velocities(), V) <= 1e-3, n


def test_ring_runs_repeat_bit_for_bit():
    """The warp reductions run in a fixed order: two runs agree bit for bit,
    whether in one call or one call per substep."""
    g, s, dens, dt, nsub, mode = fixture_settings("rings_c1_cskin_limit_star")
    out = []
    for split in (False, True, False):
        b = xfem.Body(g["nodes"], g["idx"], dens, s)
        if split:
            for _ in range(nsub):
                b.substep(dt)
        else:
            b.step_frames(1, nsub, dt)
        out.append((b.positions(), b.velocities()))
    for x, v in out[1:]:
        assert np.array_equal(x, out[0][0])
        assert np.array_equal(v, out[0][1])


def test_ring_mode_limits():
    g, s, dens, dt, nsub, mode = fixture_settings("rings_c1_cmixed_nu045_star")
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    # switching to an element model needs a new handle
    s3 = xfem.default_settings()
    with pytest.raises(xfem.XfemError) as e:
        b.set_settings(s3)
    assert e.value.code == xfem.EUNSUPPORTED
    # ring and element bodies do not share a handle
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(meshes=[(g["nodes"], g["idx"], dens)] * 2, settings=[s, s3])
    assert e.value.code == xfem.EUNSUPPORTED
    # ContinuousPixar needs nu < 0.5
    s4 = xfem.default_settings(flags=(xfem.ENERGY_CONTINUOUS_PIXAR << xfem.ENERGY_BIT), poissons_ratio=0.5)
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(g["nodes"], g["idx"], dens, s4)
    assert e.value.code == xfem.EINVAL
