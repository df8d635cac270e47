"""The launch-configuration autotuner through the C ABI.

The tuner times block size x launch form at a handle's first step
(`autotune` in xfem_api.cpp); cluster_mode 3 adds the tets-per-lane axis at
create: edge-star clusters (up to 6 tets per lane) against one tet per lane,
each layout tuned and timed, the faster kept. Every configuration runs the
colours of its layout in order, so a tuned handle must step exactly like a
handle created with the configuration it picked.
"""
import numpy as np
import pytest

import xfem
from xfem import workloads as W

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0


def _settings(flags=W.NH_FLAGS, **kw):
    return xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=W.nh_compliance(1e5, 0.45),
                                 poissons_ratio=0.45, flags=flags, **kw)


def _same(a, b):
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())


@pytest.mark.parametrize("dims,sync", [((48, 32, 16), 0), ((8, 4, 4), 0), ((24, 16, 8), 1)])
def test_layout_trial_steps_like_its_pick(dims, sync):
    nodes, idx = xfem.generate_tet_block(*dims, (0.05, 0.05, 0.05), 0, 0.2)
    s = _settings()
    t = xfem.Body(nodes, idx, 1000.0, s, cluster_mode=3, sync_mode=sync)
    info = t.info()
    assert info["cluster_mode"] in (1, 2)
    if sync:
        assert info["sync_mode"] == sync
    # the trial left the state as created
    assert np.array_equal(t.positions(), nodes.reshape(-1, 3))
    assert not t.velocities().any()
    f = xfem.Body(nodes, idx, 1000.0, s, cluster_mode=info["cluster_mode"], sync_mode=info["sync_mode"],
                  block_size=info["block_size"])
    for n in (20, 7):
        t.step_frames(1, n, DT)
        f.step_frames(1, n, DT)
        _same(t, f)
    assert t.info()["sync_mode"] == info["sync_mode"] and t.info()["block_size"] == info["block_size"]


def test_layout_trial_with_the_brick_form_forced():
    """One tet per lane has no cube chunks for the brick form: the trial keeps
    the edge-star layout."""
    nodes, idx = xfem.generate_tet_block(24, 16, 8, (0.05, 0.05, 0.05))
    t = xfem.Body(nodes, idx, 1000.0, _settings(), cluster_mode=3, sync_mode=4, block_size=256)
    assert t.info()["cluster_mode"] == 2 and t.info()["sync_mode"] == 4
    f = xfem.Body(nodes, idx, 1000.0, _settings(), sync_mode=4, block_size=256)
    t.step_frames(1, 20, DT)
    f.step_frames(1, 20, DT)
    _same(t, f)


def test_layout_trial_batch_and_damping():
    meshes = [xfem.generate_tet_block(12, 8, 8, (0.04, 0.05, 0.06), 0, 0.1) + (900.0,),
              xfem.generate_tet_block(10, 6, 6, (0.05, 0.05, 0.05), 1, 0.2) + (1100.0,)]
    settings = [_settings(damping=0.01, flags=W.NH_FLAGS | (2 << 20)), _settings()]
    t = xfem.Body(meshes=meshes, settings=settings, cluster_mode=3)
    info = t.info()
    f = xfem.Body(meshes=meshes, settings=settings, cluster_mode=info["cluster_mode"], sync_mode=info["sync_mode"],
                  block_size=info["block_size"])
    t.step_frames(1, 20, DT)
    f.step_frames(1, 20, DT)
    for k in range(2):
        assert np.array_equal(t.positions(k), f.positions(k))


def test_layout_trial_on_meshes_without_tet_clusters():
    """Rings and hexes have no cluster layout to choose: the first handle is
    kept and steps as usual."""
    nodes, idx = xfem.generate_tet_block(6, 4, 4, (0.05, 0.05, 0.05))
    s = _settings(flags=(xfem.ENERGY_CONTINUOUS_MIXED << xfem.ENERGY_BIT) | (1 << xfem.XPBD_SOLVE_BIT) | W.LOCK_LEFT)
    s.compliance = 1e-3
    r = xfem.Body(nodes, idx, 1000.0, s, cluster_mode=3)
    ref = xfem.Body(nodes, idx, 1000.0, s)
    r.step_frames(1, 10, DT)
    ref.step_frames(1, 10, DT)
    _same(r, ref)
    hn, hi = xfem.generate_hex_block(6, 4, 4, (0.05, 0.05, 0.05))
    h = xfem.Body(hn, hi, 1000.0, _settings(), cluster_mode=3)
    h.step_frames(1, 10, DT)
    assert np.isfinite(h.positions()).all()
