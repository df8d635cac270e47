"""The Right lock (Settings_LockRight, XPBDFEM/Geo.cpp:323-331) on the GPU.

After every substep's constraint sweep the vertices flagged Right (x above
98% of the body's extent, XPBDFEM/Geo.cpp:725) are put at origin +
lockedRightTransform3d X0 and keep a zero inverse mass, after the Left lock.
Checked against the reference's own substeps (the `locked` fixtures, run in
this body's colour order) and against the oracle on hex, T10 and H27 meshes,
with the transform animated between substeps as the reference's demo does
(XPBDFEM/Demo.cpp:69-80). Tolerances as for compressible materials:
positions within 1e-5 of max |x|, velocities 1e-3; the locked vertices sit
exactly at their targets.
"""
import math

import numpy as np
import pytest

import xfem
from conftest import golden, golden_args
from helpers import H27OracleRun, HexOracleRun, OracleRun, T10OracleRun, rel
from xfem import workloads as W

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
LOCKED = ["locked_c1_nh_nu045_star", "locked_c1_yeoh_nu049_amortized_pbd_tet",
          "locked_wonky_nh_serial_nu045_right_only_star"]


def locked_settings(name):
    a = golden_args(name)["args"]
    g = golden(name)
    W_, H, D, sx, sy, sz, wonk, dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[1:18]
    damping, pbd, drag, rtype, spacing, vpasses = a[18:24]
    flags = ((energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) | (xfem.LOCK_LEFT if lock else 0) |
             xfem.LOCK_RIGHT | (rtype << 20))
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, time_corrected_drag=float(g["derived"][2]),
                              volume_and_time_corrected_pbd_damping=float(g["derived"][0]),
                              amortized_volume_and_time_corrected_pbd_damping=float(g["derived"][1]), tick_id=0,
                              volume_passes=vpasses, locked_right_transform=a[24:33], origin=a[33:36])
    mode = 0 if golden_args(name)["schedule_mode"] == 1 else 1
    return g, s, dens, dt, nsub, mode


@pytest.mark.parametrize("name", LOCKED)
def test_locked_right_reference_parity(name):
    g, s, dens, dt, nsub, mode = locked_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s, cluster_mode=mode)
    assert np.array_equal(b.schedule()["tet_order"], g["order"])
    _, _, fl = xfem.compute_rest_state(g["nodes"], g["idx"], dens)
    right = (fl & 2) != 0
    assert right.any()
    b.substep(dt)
    x1 = b.positions()
    assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
    assert rel(b.velocities(), g["v1"].reshape(-1, 3)) <= 1e-3
    # the Right vertices sit exactly at the reference's targets
    assert np.array_equal(x1[right], g["x1"].reshape(-1, 3)[right].astype(np.float32))
    assert np.all(b.velocities()[right] == 0.0)
    b.step_frames(1, nsub - 1, dt)
    assert rel(b.positions(), g["xn"].reshape(-1, 3)) <= 1e-5
    assert rel(b.velocities(), g["vn"].reshape(-1, 3)) <= 1e-3
    assert np.all(b.inverse_masses()[right] == 0.0)


def _rotation(theta, sep=1.0):
    """The demo's lockedRightTransform3d: rotation(theta) * scale(2 sep - 1, 1)
    in the xy plane (XPBDFEM/Demo.cpp:71-79), column-major."""
    c, s_ = math.cos(theta), math.sin(theta)
    k = 2.0 * sep - 1.0
    return [c * k, s_ * k, 0.0, -s_, c, 0.0, 0.0, 0.0, 1.0]


def _animated(body, orc, s, steps, dt):
    """Substeps with the transform turned a little each substep (the demo's
    RotateLock animation): set on the body and the oracle alike."""
    for k in range(steps):
        s.locked_right_transform[:] = _rotation(0.002 * (k + 1), 1.05)
        body.set_settings(s)
        orc.s = s
        body.substep(dt)
        orc.step(1, dt)
        s.tick_id = k + 1


def _settings(**kw):
    """nu = 0.45 with the compliance of the element-mode parity tests (1e-3),
    the Right lock on, a small origin offset."""
    s = xfem.default_settings(gravity=(0.0, -9.81, 0.0), compliance=1e-3, poissons_ratio=0.45,
                              flags=W.NH_FLAGS | xfem.LOCK_RIGHT, origin=(0.003, -0.002, 0.001))
    for k, v in kw.items():
        if k == "locked_right_transform":
            s.locked_right_transform[:] = [float(x) for x in v]
        else:
            setattr(s, k, v)
    return s


def test_locked_right_animated_tets():
    nodes, idx = xfem.generate_tet_block(6, 2, 2, (0.05, 0.05, 0.05), 0, 0.2)
    s = _settings()
    b = xfem.Body(nodes, idx, 1000.0, s)
    o = OracleRun(nodes, idx, 1000.0, s, b.schedule()["tet_order"])
    _animated(b, o, s, 12, DT)
    assert rel(b.positions(), o.X) <= 1e-5
    assert rel(b.velocities(), o.V) <= 1e-3


def test_locked_right_hexes():
    nodes, idx = xfem.generate_hex_block(5, 2, 2, (0.05, 0.05, 0.05), 0, 0.2)
    s = _settings()
    b = xfem.Body(nodes, idx, 1000.0, s)
    o = HexOracleRun(nodes, idx, 1000.0, s, b.hex_schedule()["hex_order"])
    _animated(b, o, s, 8, DT)
    assert rel(b.positions(), o.X) <= 1e-5


@pytest.mark.parametrize("element", ["t10", "h27"])
def test_locked_right_quadratic(element):
    if element == "t10":
        nodes, idx = xfem.generate_tet_block(3, 2, 2, (0.05, 0.05, 0.05), 0, 0.2)
        s = _settings(flags=W.NH_FLAGS | xfem.LOCK_RIGHT | xfem.ELEMENT_T10)
        b = xfem.Body(nodes, idx, 1000.0, s)
        o = T10OracleRun(nodes, idx, 1000.0, s, b.t10_schedule()["t10_order"])
    else:
        nodes, idx = xfem.generate_hex_block(3, 2, 2, (0.05, 0.05, 0.05), 0, 0.2)
        s = _settings(flags=W.NH_FLAGS | xfem.LOCK_RIGHT | xfem.ELEMENT_H27)
        b = xfem.Body(nodes, idx, 1000.0, s)
        o = H27OracleRun(nodes, idx, 1000.0, s, b.h27_schedule()["h27_order"])
    assert (o.lock & 2).any()
    _animated(b, o, s, 6, DT)
    assert rel(b.positions(), o.X) <= 1e-5


def test_locked_right_batch_and_launch_forms():
    """A batch with one locked and one free body, each equal to it alone; the
    persistent and CUDA-graph launches agree bit for bit."""
    nodes, idx = xfem.generate_tet_block(6, 2, 2, (0.05, 0.05, 0.05))
    locked = _settings(locked_right_transform=_rotation(0.2, 1.1))
    free = _settings(flags=W.NH_FLAGS)
    batch = xfem.Body(meshes=[(nodes, idx, 1000.0), (nodes, idx, 1000.0)], settings=[locked, free])
    batch.step_frames(1, 15, DT)
    for i, s in enumerate((locked, free)):
        out = []
        for sm in (1, 2):
            single = xfem.Body(nodes, idx, 1000.0, s, sync_mode=sm, block_size=128)
            single.step_frames(1, 15, DT)
            out.append(single.positions())
        assert np.array_equal(out[0], out[1]), i
        assert np.array_equal(batch.positions(i), out[0]), i
    assert not np.array_equal(batch.positions(0), batch.positions(1))


def test_adjoint_refuses_the_right_lock():
    nodes, idx = xfem.generate_tet_block(4, 2, 2, (0.05, 0.05, 0.05))
    b = xfem.Body(nodes, idx, 1000.0, _settings())
    with pytest.raises(xfem.XfemError) as e:
        b.adjoint_forward(4, DT, np.array([0], np.uint32))
    assert e.value.code == xfem.EUNSUPPORTED
