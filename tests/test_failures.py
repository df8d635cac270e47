"""Failure detection, exercised on purpose without faulting the GPU.

The reference checks nothing at run time beyond asserts
(XPBDFEM/Allocator.cpp:5-10, XPBDFEM/Connectivity.cpp:261-263). This library
reports failures as status codes instead, and these tests make each one
happen:
  - bad input (unknown tags, truncated streams, vertex-count mismatches,
    invalid settings) is refused before any device is touched (CPU tests);
  - a device buffer allocation that fails (test hook) gives XFEM_ENOMEM and
    leaves the process able to create the next handle;
  - a bounded device wait that runs out (test hook: a grid barrier or a
    neighbour-chunk wait that expects one arrival more than the blocks make)
    gives XFEM_EDEVICE_TIMEOUT after the handle's short wait limit, and the
    handle steps normally afterwards;
  - a NaN position makes the device's non-finite sentinel report
    XFEM_ENONFINITE at the next synchronising call;
  - the grid barrier's 32-bit arrival counter may wrap within a launch (test
    hook: it starts at 2^32 - 1): the results stay bit-identical.
"""
import numpy as np
import pytest

import xfem
from xfem import workloads as W

DT = 1.0 / 1200.0


def _block():
    nodes, idx = xfem.generate_tet_block(4, 3, 2, (0.05, 0.05, 0.05))
    s = xfem.default_settings(gravity=(0.0, 0.0, -9.81), compliance=W.nh_compliance(1e5, 0.45), poissons_ratio=0.45,
                              flags=W.NH_FLAGS)
    return nodes, idx, s


# ---- bad input: refused with or without a GPU -----------------------------------
@pytest.mark.parametrize("case", ["tag", "truncated", "count", "density", "mixed", "empty", "empty_body"])
def test_bad_mesh_is_refused_before_the_device(case):
    nodes, idx, s = _block()
    code = xfem.EINVAL
    if case == "empty":
        nodes, idx = np.zeros(0, np.float32), np.zeros(0, np.uint32)
    elif case == "empty_body":
        # one body of a batch without elements: named
        with pytest.raises(xfem.XfemError) as e:
            xfem.Body(meshes=[(nodes, idx, 1000.0), (np.zeros(0, np.float32), np.zeros(0, np.uint32), 1000.0)],
                      settings=[s, s])
        assert e.value.code == code and "body 1" in str(e.value)
        return
    if case == "tag":
        idx = idx.copy()
        idx[5] = 6  # the second record's tag
    elif case == "truncated":
        idx = idx[:-2]
    elif case == "count":
        nodes = np.concatenate([nodes, np.zeros(3, np.float32)])
    elif case == "density":
        pass
    elif case == "mixed":
        # a mesh mixing tets and hexes with a continuous-pressure model
        idx = np.concatenate([idx, np.array([8, 0, 1, 2, 3, 4, 5, 6, 7], np.uint32)])
        s.flags = (s.flags & ~(31 << xfem.ENERGY_BIT)) | (9 << xfem.ENERGY_BIT)
        code = xfem.EUNSUPPORTED
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(nodes, idx, -1.0 if case == "density" else 1000.0, s)
    assert e.value.code == code, str(e.value)


@pytest.mark.parametrize("field,value", [("compliance", 0.0), ("poissons_ratio", 0.7), ("damping", -1.0),
                                         ("volume_passes", 65), ("friction", -0.1)])
def test_bad_settings_are_refused_before_the_device(field, value):
    nodes, idx, s = _block()
    if field == "friction":
        s.ground = 1
    setattr(s, field, value)
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(nodes, idx, 1000.0, s)
    assert e.value.code == xfem.EINVAL, str(e.value)


def test_bad_body_of_a_batch_is_named():
    nodes, idx, s = _block()
    bad = idx.copy()
    bad[0] = 3
    with pytest.raises(xfem.XfemError) as e:
        xfem.Body(meshes=[(nodes, idx, 1000.0), (nodes, bad, 1000.0)], settings=[s, s])
    assert e.value.code == xfem.EINVAL and "body 1" in str(e.value)


def test_handle_hooks_need_a_handle():
    with pytest.raises(xfem.XfemError) as e:
        xfem.test_hook(None, xfem.HOOK_MISSING_ARRIVAL, 1)
    assert e.value.code == xfem.EINVAL
    xfem.test_hook(None, xfem.HOOK_FAIL_ALLOC, 0)  # process-wide; off


# ---- on the GPU --------------------------------------------------------------------
def _fresh(**opts):
    nodes, idx, s = _block()
    return xfem.Body(nodes, idx, 1000.0, s, **opts)


@pytest.mark.gpu
@pytest.mark.parametrize("nth", [1, 4])
def test_allocation_failure_reports_enomem_and_recovers(nth):
    nodes, idx, s = _block()
    xfem.test_hook(None, xfem.HOOK_FAIL_ALLOC, nth)
    try:
        with pytest.raises(xfem.XfemError) as e:
            xfem.Body(nodes, idx, 1000.0, s)
        assert e.value.code == xfem.ENOMEM, str(e.value)
    finally:
        xfem.test_hook(None, xfem.HOOK_FAIL_ALLOC, 0)
    b = xfem.Body(nodes, idx, 1000.0, s)
    b.step_frames(1, 4, DT)
    assert np.isfinite(b.positions()).all()


@pytest.mark.gpu
@pytest.mark.parametrize("sync_mode", [1, 3])
def test_device_wait_times_out_and_the_handle_recovers(sync_mode):
    """A 100 ms wait limit; one stepping call whose waits expect an arrival
    that never comes. The call's status (reported by the next synchronising
    call) is XFEM_EDEVICE_TIMEOUT; after the state is set again the handle
    steps exactly like a fresh one."""
    ref = _fresh(sync_mode=sync_mode, block_size=128)
    b = _fresh(sync_mode=sync_mode, block_size=128, wait_timeout_ms=100)
    x0, v0 = b.positions(), b.velocities()
    # one substep first, on both: it sets the locked vertices' inverse mass to
    # zero (from the first substep on, as the reference), which a reset of
    # positions and velocities keeps
    for h in (ref, b):
        h.step_frames(1, 1, DT)
        h.set_positions(x0)
        h.set_velocities(v0)
    ref.step_frames(1, 10, DT)
    xfem.test_hook(b, xfem.HOOK_MISSING_ARRIVAL, 1)
    b.step_frames(1, 10, DT)
    with pytest.raises(xfem.XfemError) as e:
        b.synchronize()
    assert e.value.code == xfem.EDEVICE_TIMEOUT, str(e.value)
    b.synchronize()  # the error was reported once and cleared
    b.set_positions(x0)
    b.set_velocities(v0)
    b.step_frames(1, 10, DT)
    assert np.array_equal(b.positions(), ref.positions())
    assert np.array_equal(b.velocities(), ref.velocities())


@pytest.mark.gpu
def test_hex_mode_wait_times_out_and_recovers():
    nodes, idx = xfem.generate_hex_block(4, 3, 2, (0.05, 0.05, 0.05))
    s = xfem.default_settings(gravity=(0.0, 0.0, -9.81), compliance=W.nh_compliance(1e5, 0.45), poissons_ratio=0.45,
                              flags=W.NH_FLAGS)
    ref = xfem.Body(nodes, idx, 1000.0, s)
    b = xfem.Body(nodes, idx, 1000.0, s, wait_timeout_ms=100)
    x0, v0 = nodes.reshape(-1, 3), np.zeros((nodes.size // 3, 3), np.float32)
    for h in (ref, b):  # as above: the locks take hold in the first substep
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


@pytest.mark.gpu
def test_nonfinite_state_is_reported():
    b = _fresh(sync_mode=1, block_size=128)
    x = b.positions()
    bad = x.copy()
    bad[7, 1] = np.nan
    b.set_positions(bad)
    b.step_frames(1, 3, DT)
    with pytest.raises(xfem.XfemError) as e:
        b.positions()
    assert e.value.code == xfem.ENONFINITE, str(e.value)
    b.set_positions(x)
    b.set_velocities(np.zeros_like(x))
    b.step_frames(1, 3, DT)
    assert np.isfinite(b.positions()).all()


@pytest.mark.gpu
@pytest.mark.parametrize("sync_mode", [1, 3])
def test_barrier_counter_wrap_keeps_results(sync_mode):
    """The grid barrier compares arrival and target through their signed
    difference: starting the counter at 2^32 - 1 (so that the first barrier
    wraps it) changes nothing, bit for bit."""
    a = _fresh(sync_mode=sync_mode, block_size=128)
    b = _fresh(sync_mode=sync_mode, block_size=128)
    xfem.test_hook(b, xfem.HOOK_BARRIER_BASE, 1)
    for _ in range(2):
        a.step_frames(1, 25, DT)
        b.step_frames(1, 25, DT)
        assert np.array_equal(a.positions(), b.positions())
        assert np.array_equal(a.velocities(), b.velocities())


def _mode_mesh(mode):
    """A small body of each element and one-ring mode: (nodes, idx, settings)."""
    ring = (xfem.ENERGY_CONTINUOUS_MIXED << xfem.ENERGY_BIT) | (1 << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT
    if mode in ("t10", "t10_rings", "tet_rings"):
        nodes, idx = xfem.generate_tet_block(4, 3, 2, (0.05, 0.05, 0.05))
    elif mode in ("qmixed", "mixed"):
        import oracle
        nodes, idx = oracle.mixed_block(4, 2, 2, (0.05, 0.05, 0.05), 0, 0.0, lambda x, y, z: (x + y + z) % 2 == 0)
    else:
        nodes, idx = xfem.generate_hex_block(4, 3, 2, (0.05, 0.05, 0.05))
    el = {"t10": xfem.ELEMENT_T10, "t10_rings": xfem.ELEMENT_T10, "h27": xfem.ELEMENT_H27,
          "h27_rings": xfem.ELEMENT_H27, "qmixed": xfem.ELEMENT_T10}.get(mode, 0)
    flags = (ring if mode.endswith("rings") else W.NH_FLAGS) | el
    s = xfem.default_settings(gravity=(0.0, 0.0, -9.81), compliance=1e-3 if mode.endswith("rings") else
                              W.nh_compliance(1e5, 0.45), poissons_ratio=0.45, flags=flags)
    return nodes, idx, s


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["tet_rings", "hex_rings", "t10", "t10_rings", "h27", "h27_rings", "mixed", "qmixed"])
def test_element_and_ring_waits_time_out_and_recover(mode):
    """The same bounded-wait check for the element and one-ring kernels
    (k_rings, k_hex_rings, k_elements on T10s and H27s, k_t10_rings,
    k_h27_rings, k_mixed, k_qmixed)."""
    nodes, idx, s = _mode_mesh(mode)
    ref = xfem.Body(nodes, idx, 1000.0, s)
    b = xfem.Body(nodes, idx, 1000.0, s, wait_timeout_ms=100)
    x0 = b.positions()
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
    assert e.value.code == xfem.EDEVICE_TIMEOUT, str(e.value)
    b.set_positions(x0)
    b.set_velocities(v0)
    b.step_frames(1, 6, DT)
    assert np.array_equal(b.positions(), ref.positions())
