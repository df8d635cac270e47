"""GPU one-ring mode on hex meshes: the continuous-pressure models (energy
8-10) solving one constraint (pair) per vertex over the hexes around it
(SolveRing, XPBDFEM/Geo.cpp:147-225; the full-energy branch of
CalculateElementEnergyAndGradients, XPBDFEM/Fem.cpp:980-1036), with the
rings' Rayleigh damping and the PBD damping over the hexes
(XPBDFEM/Geo.cpp:800-811).

Against the reference's own substeps run in the GPU body's ring and hex
orders (the `hrings_*` fixtures of tests/golden) and against the pinned
oracle on a larger jittered block. Tolerances as for the tet rings:
positions within 1e-5 of max |x_ref|, velocities within 1e-3; the
incompressible case within 3x the FP32 reference's own distance from the
FP64 run of the same method and order.
"""
import numpy as np
import pytest

import xfem
from conftest import golden
from helpers import HexOracleRun, rel
from test_gpu_hexes import hex_settings

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
HRINGS = ["hrings_c1_cpixar_nu045", "hrings_c1_cmixed_nu045", "hrings_c1_cmixed_incompressible",
          "hrings_c1_cskin_nu049", "hrings_wonky_cmixed_paper", "hrings_c1_cskin_limit",
          "hrings_c1_cmixed_amortized_pbd", "hrings_wonky_cpixar_post"]


def _copy(s):
    return xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_})


def _fp64(name, s, dens, dt, nsub):
    """The oracle's FP64 instantiation in the fixture's orders: (X1, V1, Xn, Vn)."""
    g = golden(name)
    o = HexOracleRun(g["nodes"], g["idx"], dens, _copy(s), g["order"], dtype=np.float64, vorder=g["vorder"])
    o.step(1, dt)
    X1, V1 = o.X.copy(), o.V.copy()
    o.s.tick_id = 1
    o.step(nsub - 1, dt)
    return X1, V1, o.X, o.V


@pytest.mark.parametrize("name", HRINGS)
def test_hex_ring_reference_parity(name):
    g, s, dens, dt, nsub = hex_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    rs = b.ring_schedule()
    assert np.array_equal(rs["vert_order"], g["vorder"])
    assert np.array_equal(rs["colour_vert_begin"], g["colour_vert_begin"])
    assert np.array_equal(b.hex_schedule()["hex_order"], g["order"])
    b.substep(dt)
    x1, v1 = b.positions(), b.velocities()
    b.step_frames(1, nsub - 1, dt)
    xn, vn = b.positions(), b.velocities()
    if s.poissons_ratio < 0.5:
        assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
        assert rel(v1, g["v1"].reshape(-1, 3)) <= 1e-3
        assert rel(xn, g["xn"].reshape(-1, 3)) <= 1e-5
        assert rel(vn, g["vn"].reshape(-1, 3)) <= 1e-3
        return
    X1, V1, Xn, Vn = _fp64(name, s, dens, dt, nsub)
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
def test_hex_ring_oracle_parity(energy, nu, comp, damping, rtype, pbd):
    """A larger jittered mirrored hex block over 20 substeps against the
    oracle run in the body's ring and hex orders."""
    nodes, idx = xfem.generate_hex_block(6, 4, 3, (0.05, 0.05, 0.05), 1, 0.2)
    rng = np.random.default_rng(7)
    nodes = (nodes + rng.normal(0, 0.002, nodes.shape)).astype(np.float32)
    flags = (energy << xfem.ENERGY_BIT) | (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | (rtype << 20)
    vc, avc = xfem.pbd_damping_coefficients(pbd, DT, 0.05)
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, volume_and_time_corrected_pbd_damping=vc,
                              amortized_volume_and_time_corrected_pbd_damping=avc)
    b = xfem.Body(nodes, idx, 800.0, s)
    o = HexOracleRun(nodes, idx, 800.0, _copy(s), b.hex_schedule()["hex_order"],
                     vorder=b.ring_schedule()["vert_order"])
    for n in (1, 19):
        b.step_frames(1, n, DT)
        o.step(n, DT)
        o.s.tick_id += n
        assert rel(b.positions(), o.X) <= 1e-5, n
        assert rel(b.velocities(), o.V) <= 1e-3, n


def test_hex_ring_runs_repeat_bit_for_bit():
    """The warp reductions run in a fixed order: runs agree bit for bit, in
    one call or one call per substep, alone or batched with another body."""
    g, s, dens, dt, nsub = hex_settings("hrings_c1_cskin_limit")
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
    g2, s2, dens2, _, _ = hex_settings("hrings_wonky_cpixar_post")
    batch = xfem.Body(meshes=[(g["nodes"], g["idx"], dens), (g2["nodes"], g2["idx"], dens2)], settings=[s, s2])
    batch.step_frames(1, nsub, dt)
    assert np.array_equal(batch.positions(0), out[0][0])
    alone = xfem.Body(g2["nodes"], g2["idx"], dens2, s2)
    alone.step_frames(1, nsub, dt)
    assert np.array_equal(batch.positions(1), alone.positions())


def test_hex_ring_right_lock():
    """The Right lock on a hex ring body: the Right vertices sit at
    origin + T X0, and the run matches the oracle."""
    nodes, idx = xfem.generate_hex_block(5, 2, 2, (0.05, 0.05, 0.05), 0, 0.2)
    flags = (xfem.ENERGY_CONTINUOUS_MIXED << xfem.ENERGY_BIT) | (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | \
        xfem.LOCK_RIGHT | (2 << 20)
    s = xfem.default_settings(gravity=(0.0, -9.81, 0.0), compliance=1e-3, poissons_ratio=0.45, flags=flags,
                              origin=(0.003, -0.002, 0.001))
    s.locked_right_transform[:] = [0.9, 0.1, 0.0, -0.1, 0.9, 0.0, 0.0, 0.0, 1.0]
    b = xfem.Body(nodes, idx, 1000.0, s)
    o = HexOracleRun(nodes, idx, 1000.0, _copy(s), b.hex_schedule()["hex_order"],
                     vorder=b.ring_schedule()["vert_order"])
    assert (o.lock & 2).any()
    b.step_frames(1, 8, DT)
    o.step(8, DT)
    assert rel(b.positions(), o.X) <= 1e-5
    assert rel(b.velocities(), o.V) <= 1e-3


def test_hex_ring_errors():
    nodes, idx = xfem.generate_hex_block(3, 2, 2, (0.05, 0.05, 0.05))
    ring = xfem.default_settings(flags=(xfem.ENERGY_CONTINUOUS_MIXED << xfem.ENERGY_BIT), poissons_ratio=0.45)
    b = xfem.Body(nodes, idx, 1000.0, ring)
    # switching to an element model needs a new handle
    with pytest.raises(xfem.XfemError) as e:
        b.set_settings(xfem.default_settings())
    assert e.value.code == xfem.EUNSUPPORTED
    # linear and quadratic ring bodies cannot share a handle
    q = xfem.default_settings(flags=(xfem.ENERGY_CONTINUOUS_MIXED << xfem.ENERGY_BIT) | xfem.ELEMENT_H27,
                              poissons_ratio=0.45)
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(meshes=[(nodes, idx, 1000.0), (nodes, idx, 1000.0)], settings=[ring, q])
    assert e.value.code == xfem.EUNSUPPORTED
