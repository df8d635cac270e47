"""GPU tests of xfem_step_frames_noalloc, the stepping entry point for
callers that cannot allocate device memory when they step: their device
memory is held by another allocator (a framework's caching pool), or they
run a real-time loop that must not take cudaMalloc's device-wide
synchronisation.

Each case runs through the C ABI and is checked against xfem_step_frames, the
regular entry point, on two calls in a row. Both launch the same persistent
kernel on the same schedule, so positions, velocities and contact sets must
be identical bit for bit (np.array_equal). Covered: a plain tet body with
ground contact; a body with post-step damping sweeps and one with volume
passes (the extended kernel, whose substeps run several passes per colour);
a hex body (element mode, which steps with the handle's own scratch); the
arrival counter started at 2^32 - 1 so that it wraps inside the call; and
the per-call limit on grid-barrier arrivals, which counts every pass kind.
The file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import numpy as np
import pytest

import xfem
from xfem import workloads as W

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0


def _dropped_block():
    rng = W.Rng(31)
    nodes, idx = W.box(6, 4, 3, 0.03)
    n = nodes.reshape(-1, 3).astype(np.float64)
    n = (n - n.mean(0)) @ W.random_rotation(rng).T
    n[:, 2] += 0.01 - n[:, 2].min()
    return n.astype(np.float32).reshape(-1), idx


def _pair(nodes, idx, s, lock=None, **opts):
    regular = xfem.Body(nodes, idx, 1000.0, s, **opts)
    noalloc = xfem.Body(nodes, idx, 1000.0, s, **opts)
    if lock is not None:
        for b in (regular, noalloc):
            b.set_lock_mask(lock)
    return regular, noalloc


def _plain():
    nodes, idx = _dropped_block()
    s = W.default_settings(gravity=(0.0, 0.0, -9.81), compliance=W.nh_compliance(2e5), poissons_ratio=0.5,
                           flags=W.NH_FLAGS, ground=1, ground_normal=(0.0, 0.0, 1.0), friction=0.4)
    return _pair(nodes, idx, s, lock=W.lock_mask_axis(nodes, 0))


def _damped():
    # post-step element Rayleigh damping and PBD damping: two damping sweeps
    # per substep after the solve sweep
    nodes, idx = _dropped_block()
    flags = W.NH_FLAGS | (2 << 20)  # Rayleigh_Post (flags bits 20-21)
    c = xfem.pbd_damping_coefficients(0.02, DT, 0.03)
    s = W.default_settings(gravity=(0.0, 0.0, -9.81), compliance=W.nh_compliance(2e5, 0.45), poissons_ratio=0.45,
                           flags=flags, damping=0.05, pbd_damping=0.02, volume_and_time_corrected_pbd_damping=c[0],
                           amortized_volume_and_time_corrected_pbd_damping=c[1], ground=1,
                           ground_normal=(0.0, 0.0, 1.0), friction=0.4)
    return _pair(nodes, idx, s, lock=W.lock_mask_axis(nodes, 0))


def _volume_passes():
    nodes, idx = _dropped_block()
    s = W.default_settings(gravity=(0.0, 0.0, -9.81), compliance=W.nh_compliance(2e5, 0.45), poissons_ratio=0.45,
                           flags=W.NH_FLAGS, volume_passes=2, ground=1, ground_normal=(0.0, 0.0, 1.0), friction=0.4)
    return _pair(nodes, idx, s, lock=W.lock_mask_axis(nodes, 0))


def _hexes():
    nodes, idx = xfem.generate_hex_block(5, 3, 3, (0.03, 0.03, 0.03))
    n = nodes.reshape(-1, 3)
    n[:, 2] += 0.005 - n[:, 2].min()
    s = W.default_settings(gravity=(0.0, 0.0, -9.81), compliance=W.nh_compliance(2e5, 0.45), poissons_ratio=0.45,
                           flags=W.NH_FLAGS, ground=1, ground_normal=(0.0, 0.0, 1.0), friction=0.4)
    return _pair(nodes, idx, s, lock=W.lock_mask_axis(nodes, 0))


def _check_two_calls(regular, noalloc, substeps=20):
    for call in range(2):
        regular.step_frames(1, substeps, DT)
        noalloc.step_frames_noalloc(1, substeps, DT)
        xr, xn = regular.positions(), noalloc.positions()
        assert np.array_equal(xn, xr), f"call {call}: positions differ"
        assert np.array_equal(noalloc.velocities(), regular.velocities()), f"call {call}: velocities differ"
        assert np.array_equal(noalloc.contacts(), regular.contacts()), f"call {call}: contact sets differ"
    assert np.isfinite(xn).all()
    return xn


@pytest.mark.parametrize("make", [_plain, _damped, _volume_passes, _hexes])
def test_noalloc_matches_regular_entry_point_on_two_calls(make):
    regular, noalloc = make()
    x0 = noalloc.positions()
    xn = _check_two_calls(regular, noalloc)
    assert np.abs(xn - x0).max() > 0.0  # the bodies moved


def test_noalloc_with_wrapping_arrival_counter():
    regular, noalloc = _damped()
    xfem.test_hook(noalloc, xfem.HOOK_BARRIER_BASE, 1)
    _check_two_calls(regular, noalloc)


def test_noalloc_rejects_oversized_calls():
    _, noalloc = _plain()
    with pytest.raises(xfem.XfemError) as e:
        noalloc.step_frames_noalloc(1 << 16, 1 << 15, DT)
    assert e.value.code == xfem.ELIMIT


def test_noalloc_limit_counts_every_pass_kind():
    """A damped body runs three passes per colour per substep (solve, element
    damping, PBD damping). A call sized so that one pass per colour would stay
    under the limit but three do not is refused before any launch."""
    _, noalloc = _damped()
    noalloc.step_frames_noalloc(1, 1, DT)
    info = noalloc.info()
    per_substep_one_kind = info["colours"] * info["blocks"]
    assert per_substep_one_kind > 0
    nsub = (1 << 31) // (2 * per_substep_one_kind)  # 1 kind: below 2^31; 3 kinds: above
    with pytest.raises(xfem.XfemError) as e:
        noalloc.step_frames_noalloc(1, nsub, DT)
    assert e.value.code == xfem.ELIMIT
