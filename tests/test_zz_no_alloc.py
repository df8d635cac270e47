"""GPU test of xfem_step_frames_noalloc, the stepping entry point for callers
that cannot allocate device memory when they step (their device memory is
held by another allocator, they must avoid cudaMalloc's device-wide
synchronisation, or they step while a stream is being captured).

It runs through the C ABI and is checked against xfem_step_frames, the
regular entry point, on two calls in a row, within the position tolerance of
the parity tests (1e-5 relative; the two share the solve kernel, so the
results are expected to be identical). The file is named to be collected
last, so a run that stops at the first failure has run every other test
before it.
"""
import numpy as np
import pytest

import xfem
from helpers import rel

pytestmark = pytest.mark.gpu


def _bodies():
    from xfem import workloads as W
    rng = W.Rng(31)
    nodes, idx = W.box(6, 4, 3, 0.03)
    n = nodes.reshape(-1, 3).astype(np.float64)
    n = (n - n.mean(0)) @ W.random_rotation(rng).T
    n[:, 2] += 0.01 - n[:, 2].min()
    nodes = n.astype(np.float32).reshape(-1)
    s = W.default_settings(gravity=(0.0, 0.0, -9.81), compliance=W.nh_compliance(2e5), poissons_ratio=0.5,
                           flags=W.NH_FLAGS, ground=1, ground_normal=(0.0, 0.0, 1.0), friction=0.4)
    lock = W.lock_mask_axis(nodes, 0)
    regular = xfem.Body(nodes, idx, 1000.0, s)
    noalloc = xfem.Body(nodes, idx, 1000.0, s)
    for b in (regular, noalloc):
        b.set_lock_mask(lock)
    return regular, noalloc


def test_noalloc_matches_regular_entry_point_on_two_calls():
    regular, noalloc = _bodies()
    dt = 1.0 / 1200.0
    for call in range(2):
        regular.step_frames(1, 20, dt)
        noalloc.step_frames_noalloc(1, 20, dt)
        xr, xn = regular.positions(), noalloc.positions()
        vr, vn = regular.velocities(), noalloc.velocities()
        assert rel(xn, xr) <= 1e-5, f"call {call}: positions differ"
        assert rel(vn, vr) <= 1e-5, f"call {call}: velocities differ"
        assert np.array_equal(noalloc.contacts(), regular.contacts()), f"call {call}: contact sets differ"
    assert not np.allclose(xn, regular.positions() * 0)  # the bodies did move and stay finite
    assert np.isfinite(xn).all()


def test_noalloc_rejects_oversized_calls():
    _, noalloc = _bodies()
    with pytest.raises(xfem.XfemError) as e:
        noalloc.step_frames_noalloc(1 << 16, 1 << 15, 1.0 / 1200.0)
    assert e.value.code == xfem.ELIMIT
