"""GPU brick launch form (sync_mode 4, k_bricks) through the C ABI.

The brick kernel runs the same colours, clusters and arithmetic as the
persistent kernel (GeoLinear3d::Constrain's loop, XPBDFEM/Geo.cpp:774-788,
in the colour order), with each brick's own vertices in shared memory and
waits on neighbouring bricks instead of a grid barrier. Tets of one colour
are independent, so every result must equal the persistent kernel's bit for
bit; the persistent kernel itself is held to the reference and the oracle in
test_gpu_parity.py. One case is also checked against a reference fixture
directly.
"""
import numpy as np
import pytest

import xfem
from conftest import golden, golden_args
from helpers import rel
from xfem import workloads as W

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0


def _settings(nu=0.45, ground=False, flags=W.NH_FLAGS, **kw):
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=W.nh_compliance(1e5, nu), poissons_ratio=nu,
                              flags=flags, **kw)
    if ground:
        s.ground, s.friction = 1, 0.4
        s.ground_normal[0], s.ground_normal[1], s.ground_normal[2] = 0.0, 1.0, 0.0
        s.ground_offset = -0.01
    return s


def _pair(nodes, idx, s, block=256, density=1000.0):
    a = xfem.Body(nodes, idx, density, s, sync_mode=1, block_size=256)
    b = xfem.Body(nodes, idx, density, s, sync_mode=4, block_size=block)
    assert b.info()["sync_mode"] == 4
    return a, b


def _same(a, b, k=0):
    assert np.array_equal(a.positions(k), b.positions(k))
    assert np.array_equal(a.velocities(k), b.velocities(k))
    assert np.array_equal(a.contacts(k), b.contacts(k))


@pytest.mark.parametrize("dims,block", [((8, 2, 2), 256), ((16, 8, 8), 256), ((24, 16, 12), 224), ((48, 32, 16), 256),
                                        ((48, 32, 16), 128)])
def test_bricks_equal_persistent(dims, block):
    """One brick (the small cantilever), a few, and many with neighbours all
    round; one call of 20 substeps, then calls split differently."""
    nodes, idx = xfem.generate_tet_block(*dims, (0.05, 0.05, 0.05), 0, 0.2)
    a, b = _pair(nodes, idx, _settings(), block)
    for n in (20, 1, 7):
        a.step_frames(1, n, DT)
        b.step_frames(1, n, DT)
        _same(a, b)


def test_bricks_incompressible_ground_and_locks():
    """nu = 0.5, ground contact with friction, Left lock and a caller lock
    mask: still bit-identical."""
    nodes, idx = xfem.generate_tet_block(32, 16, 8, (0.05, 0.05, 0.05), 0, 0.3)
    nodes = nodes.reshape(-1, 3).copy()
    nodes[:, 1] -= nodes[:, 1].min()
    s = _settings(nu=0.5, ground=True)
    a, b = _pair(nodes.reshape(-1), idx, s)
    mask = (np.arange(nodes.shape[0]) % 17 == 0).astype(np.uint8)
    for h in (a, b):
        h.set_lock_mask(mask)
        h.set_velocities(np.tile(np.array([0.0, -2.0, 0.0], np.float32), (nodes.shape[0], 1)))
    for n in (15, 15):
        a.step_frames(1, n, DT)
        b.step_frames(1, n, DT)
        _same(a, b)
    assert a.contacts().any()


def test_bricks_yeoh_and_batch():
    """A batch of bodies with different materials split into bricks across
    bodies, Neo-Hookean and Yeoh with custom coefficients."""
    meshes, settings = [], []
    for k, dims in enumerate([(12, 8, 8), (20, 6, 6), (10, 10, 10)]):
        nodes, idx = xfem.generate_tet_block(*dims, (0.04, 0.05, 0.06), 0, 0.1 * k)
        meshes.append((nodes, idx, 900.0 + 100 * k))
        flags = W.YEOH_FLAGS if k == 1 else W.NH_FLAGS
        s = _settings(nu=0.45 + 0.02 * k, flags=flags)
        if k == 1:
            s.yeoh[0], s.yeoh[1], s.yeoh[2] = 1.0, 1e3 / 3e4, 1e2 / 3e4  # C10, C20, C30 = 3e4, 1e3, 1e2 over C10
        settings.append(s)
    a = xfem.Body(meshes=meshes, settings=settings, sync_mode=1, block_size=256)
    b = xfem.Body(meshes=meshes, settings=settings, sync_mode=4, block_size=256)
    a.step_frames(1, 20, DT)
    b.step_frames(1, 20, DT)
    for k in range(3):
        _same(a, b, k)


def test_bricks_reference_fixture():
    """The small cantilever against the reference's own substeps in the same
    colour order, through the brick kernel."""
    name = "ordered_c1_nh_nu045_star"
    g = golden(name)
    a = golden_args(name)["args"]
    W_, H, D, sx, sy, sz, wonk, dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[1:]
    flags = (energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) | (xfem.LOCK_LEFT if lock else 0)
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags)
    b = xfem.Body(g["nodes"], g["idx"], dens, s, sync_mode=4)
    assert np.array_equal(b.schedule()["tet_order"], g["order"])
    b.substep(dt)
    assert rel(b.positions(), g["x1"].reshape(-1, 3)) <= 1e-5
    b.step_frames(1, nsub - 1, dt)
    assert rel(b.positions(), g["xn"].reshape(-1, 3)) <= 1e-5


def test_bricks_wait_times_out_and_recovers():
    """A neighbour wait that expects one pass more than the bricks publish
    runs out after the short limit: XFEM_EDEVICE_TIMEOUT, and the handle
    steps normally afterwards."""
    nodes, idx = xfem.generate_tet_block(24, 16, 8, (0.05, 0.05, 0.05))
    s = _settings()
    ref = xfem.Body(nodes, idx, 1000.0, s, sync_mode=4, block_size=256)
    b = xfem.Body(nodes, idx, 1000.0, s, sync_mode=4, block_size=256, wait_timeout_ms=100)
    x0 = nodes.reshape(-1, 3)
    v0 = np.zeros_like(x0)
    for h in (ref, b):  # the locks take hold in the first substep
        h.step_frames(1, 1, DT)
        h.set_positions(x0)
        h.set_velocities(v0)
    ref.step_frames(1, 6, DT)
    xfem.test_hook(b, xfem.HOOK_MISSING_ARRIVAL, 1)
    b.step_frames(1, 6, DT)
    with pytest.raises(xfem.XfemError) as e:
        b.synchronize()
    assert e.value.code == xfem.EDEVICE_TIMEOUT
    b.set_positions(x0)
    b.set_velocities(v0)
    b.step_frames(1, 6, DT)
    assert np.array_equal(b.positions(), ref.positions())


def test_bricks_refuse_what_they_do_not_run():
    nodes, idx = xfem.generate_tet_block(16, 8, 8, (0.05, 0.05, 0.05))
    # damping, or the multiplier output, with the brick form forced
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(nodes, idx, 1000.0, _settings(damping=0.01), sync_mode=4)
    assert e.value.code == xfem.EUNSUPPORTED
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(nodes, idx, 1000.0, _settings(), sync_mode=4, keep_lambdas=True)
    assert e.value.code == xfem.EUNSUPPORTED
    # one tet per cluster, or the mirrored split: no cube chunks
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(nodes, idx, 1000.0, _settings(), sync_mode=4, cluster_mode=1)
    assert e.value.code == xfem.EUNSUPPORTED
    mn, mi = xfem.generate_tet_block(16, 8, 8, (0.05, 0.05, 0.05), 1)
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(mn, mi, 1000.0, _settings(), sync_mode=4)
    assert e.value.code == xfem.EUNSUPPORTED
    # an automatic handle that picked bricks falls back when damping starts
    b = xfem.Body(nodes, idx, 1000.0, _settings())
    b.step_frames(1, 4, DT)
    b.set_settings(_settings(damping=0.01, flags=W.NH_FLAGS | (2 << 20)))
    b.step_frames(1, 4, DT)
    assert b.info()["sync_mode"] != 4 and np.isfinite(b.positions()).all()


def test_bricks_follow_material_changes():
    """Per-tet shear moduli set after creation, then a new body compliance,
    then back to the uniform material: the brick chunks hold their own copy
    of each tet's record and must follow every change."""
    nodes, idx = xfem.generate_tet_block(24, 16, 8, (0.05, 0.05, 0.05), 0, 0.2)
    nt = idx.size // 5
    s = _settings()
    a, b = _pair(nodes, idx, s)
    mu = (1.0 / s.compliance * np.exp(0.3 * np.random.default_rng(4).normal(size=nt))).astype(np.float32)
    for h in (a, b):
        h.set_tet_mu(mu)
    for n in (10, 10):
        a.step_frames(1, n, DT)
        b.step_frames(1, n, DT)
        _same(a, b)
    s2 = _settings(nu=0.45)
    s2.compliance = s.compliance * 0.5
    for h in (a, b):
        h.set_tet_mu(None)
        h.set_settings(s2)
    a.step_frames(1, 10, DT)
    b.step_frames(1, 10, DT)
    _same(a, b)


def test_two_bricks_per_sm_on_the_throughput_mesh():
    """A mesh with three chunks or more per brick and colour at two bricks
    per SM (the 1,572,864-tet throughput mesh) is split that way, runs blocks
    of 192 threads, and stays bit-identical to the persistent kernel."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    w = W.throughput()
    sdt = w["dt"] / w["substeps"]
    a = xfem.Body(w["nodes"], w["idx"], w["density"], w["settings"], sync_mode=1, block_size=256)
    b = xfem.Body(w["nodes"], w["idx"], w["density"], w["settings"], sync_mode=4)
    info = b.info()
    assert info["bricks"] == 2 * sms and info["block_size"] == 192 and info["sync_mode"] == 4
    for h in (a, b):
        h.set_lock_mask(w["lock"])
        h.step_frames(1, w["substeps"], sdt)
    _same(a, b)
