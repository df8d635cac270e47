"""GPU set-up path (xfem_setup.cu) against the host set-up, bit for bit.

A handle's rest state (InitTriTetFiniteElement, XPBDFEM/Fem.cpp:196-224),
inverse masses and Left / Right flags (XPBDFEM/Geo.cpp:697-745), vertex ranks
and colour schedule must not depend on where they were computed: the GPU
phases (rest state, incidence, Morton ranks, cluster order) run the same
arithmetic as the host's, and the greedy clustering and colouring run on the
host either way. Also checked against the reference's own rest state (the
`init_*` golden fixtures) and by stepping both handles.
"""
import numpy as np
import pytest

import xfem
from conftest import golden, golden_args
from xfem import workloads as W

pytestmark = pytest.mark.gpu


def _meshes():
    out = {"box": W.box(7, 4, 3, 0.05)}
    rng = np.random.default_rng(11)
    nodes, idx = xfem.generate_tet_block(6, 5, 4, (0.1, 0.07, 0.05), 1, 0.3)
    nodes = (nodes + rng.normal(0, 0.004, nodes.shape)).astype(np.float32)
    # shuffled vertex ids and tet order, so nothing relies on generator order
    nv = nodes.size // 3
    perm = rng.permutation(nv).astype(np.uint32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(nv, dtype=np.uint32)
    tets = inv[idx.reshape(-1, 5)[:, 1:]][rng.permutation(idx.size // 5)]
    nodes = nodes.reshape(-1, 3)[perm].reshape(-1)
    out["shuffled"] = (nodes.astype(np.float32),
                       np.concatenate([np.full((tets.shape[0], 1), 4, np.uint32), tets], 1).reshape(-1))
    # one tet and one vertex (2) in no tet
    out["single_isolated"] = (np.array([0, 0, 0, 1, 0, 0, 2, 2, 2, 0, 1, 0, 0, 0, 1], np.float32),
                              np.array([4, 0, 1, 3, 4], np.uint32))
    return out


MESHES = _meshes()


def _both(nodes, idx, **opts):
    return [xfem.Body(nodes, idx, 900.0, host_setup=h, **opts) for h in (True, False)]


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    if a.dtype.kind == "f":
        assert np.array_equal(a.view(np.uint32 if a.itemsize == 4 else np.uint64),
                              b.view(np.uint32 if b.itemsize == 4 else np.uint64))
    else:
        assert np.array_equal(a, b)


@pytest.mark.parametrize("mesh", sorted(MESHES))
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("morton", [True, False])
def test_gpu_setup_equals_host_setup(mesh, mode, morton):
    nodes, idx = MESHES[mesh]
    host, gpu = _both(nodes, idx, cluster_mode=mode, morton=morton)
    for x, y in zip(host.rest_state(), gpu.rest_state()):
        _same(x, y)
    _same(host.inverse_masses(), gpu.inverse_masses())
    sh, sg = host.schedule(), gpu.schedule()
    for k in ("vert_rank", "tet_order", "colour_tet_begin"):
        _same(sh[k], sg[k])
    assert host.info()["colours"] == gpu.info()["colours"]
    assert host.info()["clusters"] == gpu.info()["clusters"]


@pytest.mark.parametrize("name", ["init_8x2x2", "init_3x2x2_mirror_wonky", "init_5x3x2_aniso_wonky"])
def test_gpu_setup_rest_state_is_the_reference(name):
    g = golden(name)
    dens = golden_args(name)["args"][9]
    b = xfem.Body(g["nodes"], g["idx"], dens)
    ep, w = b.rest_state()
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["ep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))


def test_gpu_setup_steps_like_host_setup():
    """Same rest state, Left flags (the lock, XPBDFEM/Geo.cpp:318-322) and
    schedule, so the same trajectory bit for bit."""
    w = W.cantilever_small()
    runs = []
    for host in (True, False):
        b = xfem.Body(w["nodes"], w["idx"], w["density"], w["settings"], host_setup=host, sync_mode=1)
        b.step_frames(3, w["substeps"], w["dt"] / w["substeps"])
        runs.append((b.positions(), b.velocities()))
    _same(runs[0][0], runs[1][0])
    _same(runs[0][1], runs[1][1])


def test_gpu_setup_batch():
    """A batch set up with its large body on the GPU and the others on host
    threads equals the same batch set up on the host."""
    meshes = [(n, i, 1000.0) for n, i in MESHES.values()] + [(*W.box(48, 24, 12, 0.02), 1000.0)]
    host = xfem.Body(meshes=meshes, host_setup=True)
    gpu = xfem.Body(meshes=meshes)
    for k in range(len(meshes)):
        for x, y in zip(host.rest_state(k), gpu.rest_state(k)):
            _same(x, y)
        for key in ("vert_rank", "tet_order", "colour_tet_begin"):
            _same(host.schedule(k)[key], gpu.schedule(k)[key])
