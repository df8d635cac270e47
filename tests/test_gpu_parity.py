"""GPU parity: libxfem.so (through its C ABI) against the reference and the oracle.

Tolerances (float32 kernel with fused multiply-add vs the reference's unfused
float arithmetic on double positions):
  - compressible material (nu < 0.5), where the coupled 2x2 solve is well
    conditioned: max |x_gpu - x_ref| <= 1e-5 * max |x_ref| after one substep
    and after 40; velocities <= 1e-3 relative; multipliers <= 1e-4 relative;
  - incompressible material (nu = 0.5): there the volumetric gradient
    2 (J - 1) adj(F) vanishes at rest and the multiplier goes as 1 / (J - 1),
    so the reference's own float path already differs from the FP64 run of
    the same method by ~1e-4 in position after one substep. Each FP32 path is
    then held to the FP64 run: err(gpu vs fp64) <= 3 err(reference vs fp64)
    + 1e-7;
  - integer results (schedule, ground-contact sets, run-to-run and
    layout-to-layout results) are bit-exact.
"""
import numpy as np
import pytest

import xfem
from conftest import golden, golden_args
from helpers import OracleRun, rel

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0


def c1_golden_body(name, cluster_mode, **opts):
    g = golden(name)
    a = golden_args(name)["args"]
    W, H, D, sx, sy, sz, wonk, dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[1:]
    flags = (energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) | (xfem.LOCK_LEFT if lock else 0)
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags)
    b = xfem.Body(g["nodes"], g["idx"], dens, s, cluster_mode=cluster_mode, **opts)
    return g, b, s, dt, nsub, dens


@pytest.mark.parametrize("name,mode", [("ordered_c1_nh_nu045_star", 0), ("ordered_c1_yeoh_nu049_tet", 1),
                                       ("ordered_wonky_nh_serial_nu045_star", 0)])
def test_reference_parity_same_order(name, mode):
    """The reference's own Geo3d::Substep, run in this GPU body's colour order
    (tests/golden), against the GPU after 1 and nsub substeps."""
    g, b, s, dt, nsub, _ = c1_golden_body(name, mode)
    assert np.array_equal(b.schedule()["tet_order"], g["order"])
    b.substep(dt)
    assert rel(b.positions(), g["x1"].reshape(-1, 3)) <= 1e-5
    assert rel(b.velocities(), g["v1"].reshape(-1, 3)) <= 1e-3
    b.step_frames(1, nsub - 1, dt)
    assert rel(b.positions(), g["xn"].reshape(-1, 3)) <= 1e-5
    assert abs(b.volume() - float(g["volume"][0])) <= 1e-5 * abs(float(g["volume"][0]))


@pytest.mark.parametrize("name,mode", [("ordered_c1_nh_star", 0), ("ordered_c1_yeoh_tet", 1)])
def test_reference_parity_incompressible_vs_fp64(name, mode):
    """nu = 0.5: GPU and reference both measured against the FP64 run."""
    g, b, s, dt, nsub, dens = c1_golden_body(name, mode)
    o64 = OracleRun(g["nodes"], g["idx"], dens, s, g["order"], dtype=np.float64)
    b.substep(dt)
    o64.step(1, dt)
    e_ref, e_gpu = rel(g["x1"].reshape(-1, 3), o64.X), rel(b.positions(), o64.X)
    assert e_gpu <= 3 * e_ref + 1e-7, (e_gpu, e_ref)
    b.step_frames(1, nsub - 1, dt)
    o64.step(nsub - 1, dt)
    e_ref, e_gpu = rel(g["xn"].reshape(-1, 3), o64.X), rel(b.positions(), o64.X)
    assert e_gpu <= 3 * e_ref + 1e-7, (e_gpu, e_ref)


@pytest.mark.parametrize("name", ["ordered_c1_nh_100frames_star", "ordered_c1_yeoh_100frames_star"])
def test_hundred_frames_stated_bound(name):
    """The small cantilever configuration over its 100 frames (2,000
    substeps), the reference run in this body's colour order. Stated bound:
    the GPU's distance from the FP64 run of the same method stays within 3x
    the reference's own FP32 distance from it (the reference itself is about
    1e-2 (Neo-Hookean) and 3e-3 (Yeoh) of max |x| from FP64 there: the
    incompressible constraint amplifies rounding)."""
    g, b, s, dt, nsub, dens = c1_golden_body(name, 0)
    assert np.array_equal(b.schedule()["tet_order"], g["order"])
    o64 = OracleRun(g["nodes"], g["idx"], dens, s, g["order"], dtype=np.float64)
    b.step_frames(100, nsub // 100, dt)
    o64.step(nsub, dt)
    e_ref, e_gpu = rel(g["xn"].reshape(-1, 3), o64.X), rel(b.positions(), o64.X)
    assert e_gpu <= 3 * e_ref, (e_gpu, e_ref)
    assert rel(b.positions(), g["xn"].reshape(-1, 3)) <= 4 * e_ref


def test_schedule_and_rest_state_of_handle():
    g, b, s, dt, _, _ = c1_golden_body("ordered_c1_nh_star", 0)
    sch = b.schedule()
    host = xfem.compute_schedule(g["nodes"], g["idx"], cluster_mode=0)
    for k in ("vert_rank", "tet_order", "colour_tet_begin"):
        assert np.array_equal(sch[k], host[k])
    ep, w = b.rest_state()
    gi = golden("init_8x2x2")
    assert np.array_equal(ep.reshape(-1).view(np.uint32), gi["ep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), gi["w"].view(np.uint32))
    assert np.array_equal(b.inverse_masses().view(np.uint32), gi["w"].view(np.uint32))


@pytest.mark.parametrize("simultaneous", [True, False])
@pytest.mark.parametrize("energy,comp,nu", [(4, 1e-3, 0.5), (4, 1e-3, 0.45), (7, 3e-3, 0.5), (7, 3e-3, 0.49)])
@pytest.mark.parametrize("mode", [0, 1])
def test_oracle_parity_energy_solve_modes(simultaneous, energy, comp, nu, mode):
    nodes, idx = xfem.generate_tet_block(6, 3, 2, (0.05, 0.05, 0.05), 1, 0.0)
    rng = np.random.default_rng(5)
    nodes = (nodes + rng.normal(0, 0.003, nodes.shape)).astype(np.float32)
    flags = (energy << xfem.ENERGY_BIT) | (int(simultaneous) << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags)
    b = xfem.Body(nodes, idx, 800.0, s, cluster_mode=mode, keep_lambdas=True)
    order = b.schedule()["tet_order"]
    o = OracleRun(nodes, idx, 800.0, s, order)
    o64 = OracleRun(nodes, idx, 800.0, s, order, dtype=np.float64)
    for n in (1, 20):
        b.step_frames(1, n, DT)
        o.step(n, DT)
        o64.step(n, DT)
        if nu < 0.5:
            assert rel(b.positions(), o.X) <= 1e-5
            if n == 1:
                assert rel(b.velocities(), o.V) <= 1e-3
                assert rel(b.lambdas(), o.lam) <= 1e-4
        else:
            e_ref, e_gpu = rel(o.X, o64.X), rel(b.positions(), o64.X)
            assert e_gpu <= 3 * e_ref + 1e-7, (n, e_gpu, e_ref)


def test_ground_friction_contacts():
    """A rotated block dropped onto z = 0 with friction: positions against the
    oracle and the contact set bit-exact after the step that lands it."""
    from xfem import workloads as W
    rng = W.Rng(11)
    nodes, idx = xfem.generate_tet_block(5, 3, 3, (0.02, 0.02, 0.02))
    n = nodes.reshape(-1, 3).astype(np.float64)
    n = (n - n.mean(0)) @ W.random_rotation(rng).T
    n[:, 2] += 0.002 - n[:, 2].min()
    nodes = n.astype(np.float32).reshape(-1)
    s = xfem.default_settings(gravity=(0, 0, -9.81), compliance=W.nh_compliance(1e5, 0.45), poissons_ratio=0.45,
                              flags=W.NH_FLAGS & ~xfem.LOCK_LEFT, ground=1, ground_normal=(0, 0, 1),
                              ground_offset=0.0, friction=0.4)
    b = xfem.Body(nodes, idx, 1000.0, s)
    o = OracleRun(nodes, idx, 1000.0, s, b.schedule()["tet_order"])
    b.set_velocities(np.tile([0.3, 0.1, -1.0], (nodes.size // 3, 1)))
    o.V[:] = [0.3, 0.1, -1.0]
    seen = 0
    for k in range(12):
        b.step_frames(1, 5, DT)
        o.step(5, DT)
        c = b.contacts()
        assert np.array_equal(c, o.contact), f"contact sets differ after {5 * (k + 1)} substeps"
        seen += int(c.sum())
        assert rel(b.positions(), o.X) <= 1e-5
    assert seen > 0
    assert b.positions()[:, 2].min() >= -1e-6


def test_per_tet_material():
    from xfem import workloads as W
    nodes, idx = xfem.generate_tet_block(8, 2, 2, (0.05, 0.05, 0.05))
    nt = idx.size // 5
    rng = W.Rng(21)
    mu = (1.0 / W.nh_compliance(1e5, 0.45) * np.exp(0.3 * rng.normal(nt))).astype(np.float32)
    s = xfem.default_settings(gravity=(0, 0, -9.81), compliance=W.nh_compliance(1e5, 0.45), poissons_ratio=0.45,
                              flags=W.NH_FLAGS)
    b = xfem.Body(nodes, idx, 1000.0, s)
    b.set_tet_mu(mu)
    o = OracleRun(nodes, idx, 1000.0, s, b.schedule()["tet_order"], tet_mu=mu)
    b.step_frames(1, 20, DT)
    o.step(20, DT)
    assert rel(b.positions(), o.X) <= 1e-5
    # back to the uniform material
    b.set_tet_mu(None)
    o.tet_mu = None
    b.step_frames(1, 5, DT)
    o.step(5, DT)
    assert rel(b.positions(), o.X) <= 1e-5


def _run(nodes, idx, s, n, **opts):
    b = xfem.Body(nodes, idx, 1000.0, s, **opts)
    b.step_frames(1, n, DT)
    return b.positions(), b.velocities()


def test_launch_modes_are_bit_identical():
    """Persistent kernel vs CUDA graph and every block size: clusters of a
    colour are independent, so the result must not depend on the launch."""
    from xfem import workloads as W
    nodes, idx = xfem.generate_tet_block(10, 6, 5, (0.05, 0.05, 0.05))
    s = xfem.default_settings(gravity=(0, 0, -9.81), compliance=W.nh_compliance(1e5), poissons_ratio=0.5,
                              flags=W.NH_FLAGS)
    ref = _run(nodes, idx, s, 30, sync_mode=1, block_size=256)
    for sm, bs in [(1, 64), (1, 128), (2, 64), (2, 256), (0, 0)]:
        x, v = _run(nodes, idx, s, 30, sync_mode=sm, block_size=bs)
        assert np.array_equal(x, ref[0]) and np.array_equal(v, ref[1]), (sm, bs)
    # repeated calls split differently give the same state too
    b = xfem.Body(nodes, idx, 1000.0, s, sync_mode=1, block_size=256)
    for _ in range(3):
        b.step_frames(1, 10, DT)
    assert np.array_equal(b.positions(), ref[0])


def test_batch_equals_single_bodies():
    from xfem import workloads as W
    w = W.batched(seed=9, nbodies=5, lo=2, hi=6)
    batch = xfem.Body(meshes=w["meshes"], settings=w["settings"])
    batch.step_frames(1, 20, DT)
    for i, (nodes, idx, dens) in enumerate(w["meshes"]):
        single = xfem.Body(nodes, idx, dens, w["settings"][i])
        single.step_frames(1, 20, DT)
        assert np.array_equal(batch.positions(i), single.positions()), i
        assert np.array_equal(batch.contacts(i), single.contacts()), i


def test_state_transfer_round_trip():
    nodes, idx = xfem.generate_tet_block(4, 3, 2, (0.1, 0.1, 0.1))
    b = xfem.Body(nodes, idx, 1000.0, xfem.default_settings(flags=(4 << 6) | (1 << 11)))
    x = nodes.reshape(-1, 3) + 0.01
    v = np.random.default_rng(1).normal(size=x.shape).astype(np.float32)
    b.set_positions(x)
    b.set_velocities(v)
    assert np.array_equal(b.positions(), x.astype(np.float32))
    assert np.array_equal(b.velocities(), v)


def test_throughput_mesh_one_substep_vs_fp64():
    """Full-size 1,572,864-tet incompressible mesh: one substep against the FP64
    oracle next to the reference-semantics oracle (run with all host threads
    in the same colour order), plus size-independent properties: volume kept
    by the incompressible constraint, the fixed face stays put."""
    import os

    import oracle
    from helpers import oracle_params
    from xfem import workloads as W
    w = W.throughput()
    b = xfem.Body(w["nodes"], w["idx"], w["density"], w["settings"])
    b.set_lock_mask(w["lock"])
    sch = b.schedule()
    sdt = w["dt"] / w["substeps"]
    b.substep(sdt)
    x = b.positions()
    o = OracleRun(w["nodes"], w["idx"], w["density"], w["settings"], sch["tet_order"], lock_mask=w["lock"])
    p = oracle_params(w["settings"], sdt)
    X32, _v32, _w32, _ = oracle.substeps(o.X, o.V, o.w, o.tets, o.ep, sch["tet_order"], 1, p, lock_mask=o.lock,
                                         threads=os.cpu_count(), colour_begin=sch["colour_tet_begin"])
    ep64, w64, _ = oracle.init_rest(w["nodes"], o.tets, w["density"], np.float64)
    X64, _, _, _ = oracle.substeps(o.X, o.V, w64, o.tets, ep64, sch["tet_order"], 1, p, lock_mask=o.lock,
                                   dtype=np.float64)
    e_ref, e_gpu = rel(X32, X64), rel(x, X64)
    assert e_gpu <= 3 * e_ref + 1e-7, (e_gpu, e_ref)
    # one frame more: volume against the oracle's (one Gauss-Seidel iteration
    # per substep keeps volume only approximately; both must drift alike)
    b.step_frames(1, w["substeps"], sdt)
    x = b.positions()
    X32, _, _, _ = oracle.substeps(X32, _v32, _w32, o.tets, o.ep, sch["tet_order"], w["substeps"], p,
                                   lock_mask=o.lock, threads=os.cpu_count(), colour_begin=sch["colour_tet_begin"])
    v_orc = oracle.volume(X32, o.tets, np.float64)
    assert abs(b.volume() - v_orc) <= 1e-5 * v_orc
    fixed = w["lock"].astype(bool)
    assert np.array_equal(x[fixed], w["nodes"].reshape(-1, 3)[fixed])


@pytest.mark.parametrize("pinned", [False, True])
def test_state_transfer_forms_agree(pinned):
    """xfem_set_state equals xfem_set_positions then xfem_set_velocities, and
    page-locked buffers (read and written by the kernels themselves) equal
    pageable ones, bit for bit, on a batch's second body."""
    import ctypes
    meshes = [xfem.generate_tet_block(4, 3, 2, (0.05, 0.05, 0.05)) + (1000.0,),
              xfem.generate_tet_block(6, 3, 3, (0.04, 0.05, 0.06), 1, 0.2) + (900.0,)]
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=1e-3, poissons_ratio=0.45)
    a = xfem.Body(meshes=meshes, settings=[s, s])
    b = xfem.Body(meshes=meshes, settings=[s, s])
    nv = meshes[1][0].size // 3
    rng = np.random.default_rng(5)
    x = (meshes[1][0].reshape(-1, 3) + rng.normal(0, 1e-3, (nv, 3))).astype(np.float32)
    v = rng.normal(0, 0.1, (nv, 3)).astype(np.float32)
    bufs = []
    if pinned:
        for arr in (x, v):
            p = xfem.lib().xfem_alloc_host(arr.nbytes)
            buf = np.frombuffer((ctypes.c_float * arr.size).from_address(p), np.float32)
            buf[:] = arr.reshape(-1)
            bufs.append((p, buf))
        xin, vin = bufs[0][1], bufs[1][1]
    else:
        xin, vin = x, v
    a.set_positions(xin, body=1)
    a.set_velocities(vin, body=1)
    b.set_state(xin, vin, body=1)
    for h in (a, b):
        h.step_frames(1, 5, DT)
    out = np.zeros(3 * nv, np.float32) if not pinned else bufs[0][1]
    xa = a.positions(1, out=out).copy()
    assert np.array_equal(xa, b.positions(1))
    assert np.array_equal(a.velocities(1), b.velocities(1))
    assert np.array_equal(a.positions(0), b.positions(0))
    for p, _ in bufs:
        xfem.lib().xfem_free_host(p)
