"""GPU damping (GeoLinear3d::Damp and the in-solve Rayleigh terms) against the
reference's own substep, run in the GPU body's colour order (the `damped`
fixtures of tests/golden, produced by the unmodified reference).

Tolerances as in test_gpu_parity.py for compressible materials: positions
1e-5 of max |x_ref| after one substep and after all of them; velocities 1e-3
relative. Launch forms, call splits and batching must agree bit for bit.
"""
import numpy as np
import pytest

import xfem
from conftest import golden, golden_args
from helpers import rel
from xfem import workloads as W

pytestmark = pytest.mark.gpu

DAMPED = ["damped_c1_nh_nu045_amortized_pbd_star", "damped_c1_nh_nu045_post_star", "damped_c1_nh_nu045_paper_star",
          "damped_c1_nh_nu045_limit_star", "damped_c1_yeoh_nu049_amortized_pbd_tet",
          "damped_wonky_nh_serial_post_pbd_star", "damped_wonky_nh_serial_limit_pbd_star"]


def damped_settings(name):
    a = golden_args(name)["args"]
    g = golden(name)
    W_, H, D, sx, sy, sz, wonk, dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[1:18]
    damping, pbd, drag, rtype, spacing = a[18:]
    flags = ((energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) | (xfem.LOCK_LEFT if lock else 0) |
             (rtype << 20))
    # the reference's own derived values (Sim::Update), as a caller fills them
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, time_corrected_drag=float(g["derived"][2]),
                              volume_and_time_corrected_pbd_damping=float(g["derived"][0]),
                              amortized_volume_and_time_corrected_pbd_damping=float(g["derived"][1]), tick_id=0)
    # the fixture's oracle schedule mode (1 edge stars, 0 one tet per cluster)
    # as the product's cluster_mode (0 edge stars, 1 one tet per cluster)
    mode = 0 if golden_args(name)["schedule_mode"] == 1 else 1
    return g, s, dens, dt, nsub, mode


def body_of(name, **opts):
    g, s, dens, dt, nsub, mode = damped_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s, cluster_mode=mode, **opts)
    return g, b, s, dt, nsub


@pytest.mark.parametrize("name", DAMPED)
def test_damped_reference_parity(name):
    g, b, s, dt, nsub = body_of(name)
    assert np.array_equal(b.schedule()["tet_order"], g["order"])
    b.substep(dt)
    assert rel(b.positions(), g["x1"].reshape(-1, 3)) <= 1e-5
    assert rel(b.velocities(), g["v1"].reshape(-1, 3)) <= 1e-3
    b.step_frames(1, nsub - 1, dt)
    assert rel(b.positions(), g["xn"].reshape(-1, 3)) <= 1e-5
    assert rel(b.velocities(), g["vn"].reshape(-1, 3)) <= 1e-3


@pytest.mark.parametrize("name", ["damped_c1_nh_nu045_amortized_pbd_star", "damped_wonky_nh_serial_limit_pbd_star",
                                  "damped_c1_nh_nu045_limit_star"])
def test_damped_launch_forms_agree(name):
    """Persistent kernel and CUDA graph, one call or one call per substep."""
    runs = []
    for mode, split in ((1, False), (2, False), (1, True)):
        g, b, s, dt, nsub = body_of(name, sync_mode=mode)
        if split:
            for _ in range(nsub):
                b.substep(dt)
        else:
            b.step_frames(1, nsub, dt)
        runs.append((b.positions(), b.velocities()))
    for x, v in runs[1:]:
        assert np.array_equal(x, runs[0][0])
        assert np.array_equal(v, runs[0][1])


def test_tick_reset_repeats():
    """xfem_set_settings sets Settings::tickId, and the amortized slices follow
    it: after a reset to the same state and tick two runs agree bit for bit,
    while the same state at another tick gives another result."""
    name = "damped_c1_nh_nu045_amortized_pbd_star"
    out = []
    for warm, tick in ((1, 0), (5, 0), (5, 5)):
        g, b, s, dt, nsub = body_of(name)
        b.step_frames(1, warm, dt)  # the lock zeroes the locked inverse masses in the first substep
        b.set_positions(g["nodes"])
        b.set_velocities(np.zeros((g["nodes"].size // 3, 3), np.float32))
        s.tick_id = tick
        b.set_settings(s)
        b.step_frames(1, 8, dt)
        out.append(b.positions())
    assert np.array_equal(out[0], out[1])
    assert not np.array_equal(out[0], out[2])


def test_batched_damped_and_undamped():
    """A damped and an undamped body in one handle: each as when run alone."""
    g1, s1, dens1, dt, nsub, mode1 = damped_settings("damped_c1_nh_nu045_amortized_pbd_star")
    nodes2, idx2 = W.box(6, 2, 2, 0.05)
    s2 = xfem.default_settings(gravity=(0, -9.81, 0), compliance=W.nh_compliance(1e5, 0.45), poissons_ratio=0.45,
                               flags=W.NH_FLAGS)
    alone = []
    for nodes, idx, s in ((g1["nodes"], g1["idx"], s1), (nodes2, idx2, s2)):
        b = xfem.Body(nodes, idx, 1000.0, s)
        b.step_frames(1, 20, dt)
        alone.append((b.positions(), b.velocities()))
    B = xfem.Body(meshes=[(g1["nodes"], g1["idx"], 1000.0), (nodes2, idx2, 1000.0)], settings=[s1, s2])
    B.step_frames(1, 20, dt)
    for k in range(2):
        assert np.array_equal(B.positions(k), alone[k][0]), k
        assert np.array_equal(B.velocities(k), alone[k][1]), k


def test_adjoint_rejects_damping():
    g, b, s, dt, nsub = body_of("damped_c1_nh_nu045_post_star")
    with pytest.raises(xfem.XfemError):
        b.adjoint_forward(4, dt, np.array([0], np.uint32))


def test_dataflow_mode_rejects_damping():
    """The dataflow kernel has no damping: asking for it with damping on is an error."""
    g, b, s, dt, nsub = body_of("damped_c1_nh_nu045_paper_star", sync_mode=3)
    with pytest.raises(xfem.XfemError) as e:
        b.step_frames(1, 2, dt)
    assert e.value.code == xfem.EUNSUPPORTED
