"""CPU tests of libxfem.so's host side (no GPU needed).

- the library loads and exports every function include/xfem.h declares;
- rest state and masses equal the reference's (golden vectors) bit for bit
  (XPBDFEM/Fem.cpp:131-224, XPBDFEM/Geo.cpp:697-745);
- GenerateTetBlock (XPBDFEM/MeshGen.cpp:156-244) is reproduced bit for bit;
- the colour schedule equals the oracle's independent restatement bit for
  bit, and is a valid Gauss-Seidel colouring (every tet once, no two tets of
  one colour share a vertex);
- without a CUDA device the solver refuses to run (no CPU fallback).
"""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden, golden_args

import xfem


def header_functions():
    src = open(os.path.join(ROOT, "include", "xfem.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|float|void\*?|const char\*)\s+\*?(xfem_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    L = xfem.lib()
    names = header_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(L, n), n
    assert sorted(names) == sorted(xfem.EXPORTS)


@pytest.mark.parametrize("name", ["meshgen_8x2x2", "meshgen_3x2x2_mirror_wonky", "meshgen_4x3x2_aniso_wonky"])
def test_generate_tet_block_bit_exact(name):
    g = golden(name)
    a = golden_args(name)["args"]
    nodes, idx = xfem.generate_tet_block(a[1], a[2], a[3], tuple(a[4:7]), a[7], a[8])
    assert np.array_equal(idx, g["idx"])
    assert np.array_equal(nodes.view(np.uint32), g["nodes"].view(np.uint32))


@pytest.mark.parametrize("name", ["init_8x2x2", "init_3x2x2_mirror_wonky", "init_5x3x2_aniso_wonky"])
def test_rest_state_bit_exact_vs_reference(name):
    g = golden(name)
    a = golden_args(name)["args"]
    ep, w, fl = xfem.compute_rest_state(g["nodes"], g["idx"], a[9])
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["ep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])


def _random_mesh(seed, W, H, D):
    rng = np.random.default_rng(seed)
    nodes, idx = xfem.generate_tet_block(W, H, D, (0.1, 0.07, 0.05), seed % 2, 0.0)
    nodes = nodes + rng.normal(0, 0.004, nodes.shape).astype(np.float32)
    # shuffle vertex ids and tet order so nothing relies on generator order
    nv = nodes.size // 3
    perm = rng.permutation(nv).astype(np.uint32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(nv, dtype=np.uint32)
    tets = idx.reshape(-1, 5)[:, 1:]
    tets = inv[tets][rng.permutation(tets.shape[0])]
    nodes = nodes.reshape(-1, 3)[perm].reshape(-1)
    idx = np.concatenate([np.full((tets.shape[0], 1), 4, np.uint32), tets], 1).reshape(-1)
    return nodes.astype(np.float32), idx.astype(np.uint32)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_rest_state_matches_oracle_on_jittered_meshes(orc, seed):
    nodes, idx = _random_mesh(seed, 5, 4, 3)
    ep, w, fl = xfem.compute_rest_state(nodes, idx, 1000.0)
    tets, _ = orc.parse_tets(idx)
    e2, w2, f2 = orc.init_rest(nodes, tets, 1000.0)
    assert np.array_equal(ep.view(np.uint32), e2.view(np.uint32))
    assert np.array_equal(w.view(np.uint32), w2.view(np.uint32))
    assert np.array_equal(fl, f2)


def check_colouring(tets, order, cb, cluster_of):
    """Every tet once; clusters of one colour share no vertex (tets inside a
    cluster run in sequence on one thread and may share vertices)."""
    nt = tets.shape[0]
    assert np.array_equal(np.sort(order), np.arange(nt))
    for c in range(cb.size - 1):
        ts = order[cb[c]:cb[c + 1]]
        owner = {}
        for t in ts:
            for v in tets[t]:
                k = owner.setdefault(int(v), int(cluster_of[t]))
                assert k == cluster_of[t], f"colour {c}: clusters {k} and {cluster_of[t]} share vertex {v}"


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("morton", [True, False])
@pytest.mark.parametrize("mesh", ["box", "jitter"])
def test_schedule_bit_exact_vs_oracle(orc, mode, morton, mesh):
    if mesh == "box":
        nodes, idx = xfem.generate_tet_block(9, 5, 4, (0.1, 0.1, 0.1))
    else:
        nodes, idx = _random_mesh(7, 6, 5, 4)
    s = xfem.compute_schedule(nodes, idx, cluster_mode=mode, morton=morton)
    tets, _ = orc.parse_tets(idx)
    # product cluster_mode: 0 default (edge stars), 1 one tet each, 2 edge stars
    o = orc.schedule(nodes, tets, mode=0 if mode == 1 else 1, morton=int(morton))
    assert s["colours"] == o["colours"]
    assert s["clusters"] == o["clusters"]
    assert np.array_equal(s["vert_rank"], o["vert_rank"])
    assert np.array_equal(s["tet_order"], o["tet_order"])
    assert np.array_equal(s["colour_tet_begin"], o["colour_tet_begin"])
    check_colouring(tets, s["tet_order"], s["colour_tet_begin"], o["cluster_of"])


def test_schedule_colour_counts_on_cube_grid():
    # 6-tet cubes: an interior vertex touches 24 tets and 8 cubes, so one tet
    # per cluster needs >= 24 colours and edge-star (cube) clusters >= 8.
    nodes, idx = xfem.generate_tet_block(12, 8, 6, (0.1, 0.1, 0.1))
    s_tet = xfem.compute_schedule(nodes, idx, cluster_mode=1)
    s_star = xfem.compute_schedule(nodes, idx, cluster_mode=0)
    assert s_star["clusters"] == 12 * 8 * 6
    assert s_star["colours"] == 8
    assert 24 <= s_tet["colours"] <= 40


def test_errors_without_gpu_or_bad_input():
    nodes, idx = xfem.generate_tet_block(2, 1, 1, (0.1, 0.1, 0.1))
    hexes = np.array([8, 0, 1, 2, 3, 4, 5, 6, 7], np.uint32)
    with pytest.raises(xfem.XfemError) as e:
        xfem.compute_rest_state(np.zeros(24, np.float32), hexes, 1000.0)
    assert e.value.code == xfem.EUNSUPPORTED
    with pytest.raises(xfem.XfemError) as e:
        xfem.compute_rest_state(nodes[:-3], idx, 1000.0)
    assert e.value.code == xfem.EINVAL
    import torch
    if not torch.cuda.is_available():
        # no silent CPU path: creating a solver needs the GPU
        with pytest.raises(xfem.XfemError) as e:
            xfem.Body(nodes, idx, 1000.0)
        assert e.value.code == xfem.ECUDA


def test_time_corrected_drag():
    assert xfem.time_corrected_drag(0.0, 1 / 1200) == 0.0
    v = xfem.time_corrected_drag(0.002, 1 / 3000)
    assert abs(v - (1 - (1 - 0.002) ** (1000 / 3000))) < 1e-7


@pytest.mark.parametrize("name", ["damped_c1_nh_nu045_amortized_pbd_star", "damped_c1_yeoh_nu049_amortized_pbd_tet",
                                  "damped_wonky_nh_serial_post_pbd_star"])
def test_pbd_damping_coefficients_match_reference(name):
    """xfem_pbd_damping_coefficients and xfem_time_corrected_drag against the
    values Sim::Update computed in the reference (XPBDFEM/Demo.cpp:53-63),
    within 2 ulp (powf may round differently between C libraries)."""
    g = golden(name)
    a = golden_args(name)["args"]
    dt, pbd, drag, spacing = a[15], a[19], a[20], a[22]
    vc, avc = xfem.pbd_damping_coefficients(pbd, dt, spacing)
    for got, want in ((vc, g["derived"][0]), (avc, g["derived"][1]), (xfem.time_corrected_drag(drag, dt), g["derived"][2])):
        assert abs(np.float32(got) - want) <= 2 * np.spacing(np.float32(want)), (got, want)


@pytest.mark.parametrize("morton", [True, False])
@pytest.mark.parametrize("mesh", ["box", "jitter"])
def test_ring_schedule_bit_exact_vs_oracle(orc, morton, mesh):
    """The ring schedule of the continuous-pressure models (one-rings of one
    colour share no vertex) equals the oracle's independent restatement."""
    if mesh == "box":
        nodes, idx = xfem.generate_tet_block(9, 5, 4, (0.1, 0.1, 0.1))
    else:
        nodes, idx = _random_mesh(7, 6, 5, 4)
    s = xfem.compute_ring_schedule(nodes, idx, morton=morton)
    tets, _ = orc.parse_tets(idx)
    o = orc.ring_schedule(nodes, tets, morton=int(morton))
    assert s["colours"] == o["colours"]
    assert np.array_equal(s["vert_order"], o["vert_order"])
    assert np.array_equal(s["colour_vert_begin"], o["colour_vert_begin"])


@pytest.mark.parametrize("morton", [True, False])
def test_hex_ring_schedule_bit_exact_vs_oracle(orc, morton):
    """The continuous-pressure models on a hex mesh: one-rings over the hexes
    around each vertex, the same colouring rule; equal to the oracle's
    restatement and, with Morton order, to the vertex order the reference's
    own `hrings` fixtures ran in."""
    nodes, idx = xfem.generate_hex_block(7, 5, 4, (0.1, 0.1, 0.1), 1, 0.3)
    s = xfem.compute_ring_schedule(nodes, idx, morton=morton)
    hexes, _ = orc.parse_hexes(idx)
    o = orc.ring_schedule(nodes, hexes, morton=int(morton))
    assert s["colours"] == o["colours"]
    assert np.array_equal(s["vert_order"], o["vert_order"])
    assert np.array_equal(s["colour_vert_begin"], o["colour_vert_begin"])
    if morton:
        for name in ("hrings_c1_cpixar_nu045", "hrings_wonky_cmixed_paper"):
            g = golden(name)
            f = xfem.compute_ring_schedule(g["nodes"], g["idx"])
            assert np.array_equal(f["vert_order"], g["vorder"]), name
            assert np.array_equal(f["colour_vert_begin"], g["colour_vert_begin"]), name


@pytest.mark.parametrize("morton", [True, False])
@pytest.mark.parametrize("pattern", [0, 1])
def test_t10_ring_schedule_is_the_linear_one(orc, morton, pattern):
    """A T10 body rings its mesh vertices over the T10s around them. Two such
    rings that share an edge node share that edge's two vertices, so the
    colouring (and the order) is the linear tet mesh's: the oracle's T10 ring
    schedule equals compute_ring_schedule of the linear mesh, and the
    reference's own `qrings` fixtures ran in that order."""
    nodes, idx = xfem.generate_tet_block(6, 4, 5, (0.05, 0.05, 0.05), pattern, 0.2)
    s = xfem.compute_ring_schedule(nodes, idx, morton=morton)
    o = orc.Quadratic(nodes, idx, 1000.0).ring_schedule(morton=int(morton))
    assert s["colours"] == o["colours"]
    assert np.array_equal(s["vert_order"], o["vert_order"])
    assert np.array_equal(s["colour_vert_begin"], o["colour_vert_begin"])
    if morton and pattern == 0:
        for name in ("qrings_c1_cpixar_nu045", "qrings_wonky_cmixed_paper"):
            g = golden(name)
            f = xfem.compute_ring_schedule(g["nodes"], g["idx"])
            assert np.array_equal(f["vert_order"], g["vorder"]), name
            assert np.array_equal(f["colour_vert_begin"], g["colour_vert_begin"]), name


@pytest.mark.parametrize("morton", [True, False])
@pytest.mark.parametrize("pattern", [0, 1])
def test_h27_ring_schedule_is_the_linear_one(orc, morton, pattern):
    """The same for H27 bodies: a ring shares an added edge, face or centre
    node with another only through an H27 holding both centres' corners, so
    the order is the linear hex mesh's, as the `h27rings` fixtures ran."""
    nodes, idx = xfem.generate_hex_block(6, 4, 5, (0.05, 0.05, 0.05), pattern, 0.2)
    s = xfem.compute_ring_schedule(nodes, idx, morton=morton)
    o = orc.QuadraticHex(nodes, idx, 1000.0).ring_schedule(morton=int(morton))
    assert s["colours"] == o["colours"]
    assert np.array_equal(s["vert_order"], o["vert_order"])
    assert np.array_equal(s["colour_vert_begin"], o["colour_vert_begin"])
    if morton and pattern == 0:
        for name in ("h27rings_c1_cpixar_nu045", "h27rings_wonky_cmixed_paper"):
            g = golden(name)
            f = xfem.compute_ring_schedule(g["nodes"], g["idx"])
            assert np.array_equal(f["vert_order"], g["vorder"]), name
            assert np.array_equal(f["colour_vert_begin"], g["colour_vert_begin"]), name


# ---- linear hexahedra: the host side of hex mode ----
def test_generate_hex_block_bit_exact():
    g = golden("hmeshgen_3x2x2_mirror_wonky")
    a = golden_args("hmeshgen_3x2x2_mirror_wonky")["args"]
    nodes, idx = xfem.generate_hex_block(a[1], a[2], a[3], tuple(a[4:7]), a[7], a[8])
    assert np.array_equal(idx, g["idx"])
    assert np.array_equal(nodes.view(np.uint32), g["nodes"].view(np.uint32))
    # the tet block is the same grid split six ways
    tn, _ = xfem.generate_tet_block(a[1], a[2], a[3], tuple(a[4:7]), a[7], a[8])
    assert np.array_equal(tn.view(np.uint32), nodes.view(np.uint32))


@pytest.mark.parametrize("name", ["hinit_4x2x2", "hinit_3x2x2_mirror_wonky", "hinit_4x3x2_aniso_wonky"])
def test_hex_rest_state_bit_exact_vs_reference(name):
    """InitQuadHexFiniteElement (XPBDFEM/Fem.cpp:225-265) through
    GeoLinear3d::Init: records, inverse masses and flags."""
    g = golden(name)
    a = golden_args(name)["args"]
    ep, w, fl = xfem.compute_hex_rest_state(g["nodes"], g["idx"], a[9])
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["hep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])


@pytest.mark.parametrize("seed", [1, 2])
def test_hex_rest_state_matches_oracle_on_jittered_meshes(orc, seed):
    rng = np.random.default_rng(seed)
    nodes, idx = xfem.generate_hex_block(5, 4, 3, (0.03, 0.05, 0.04), seed % 2, 0.4)
    nodes = (nodes + rng.normal(0, 0.002, nodes.shape)).astype(np.float32)
    ep, w, fl = xfem.compute_hex_rest_state(nodes, idx, 700.0)
    hexes, _ = orc.parse_hexes(idx)
    e2, w2, f2 = orc.hex_init_rest(nodes, hexes, 700.0)
    assert np.array_equal(ep.view(np.uint32), e2.view(np.uint32))
    assert np.array_equal(w.view(np.uint32), w2.view(np.uint32))
    assert np.array_equal(fl, f2)


@pytest.mark.parametrize("morton", [True, False])
@pytest.mark.parametrize("pattern", [0, 1])
def test_hex_schedule_bit_exact_vs_oracle(orc, morton, pattern):
    nodes, idx = xfem.generate_hex_block(6, 5, 3, (0.1, 0.1, 0.1), pattern, 0.3)
    s = xfem.compute_hex_schedule(nodes, idx, morton=morton)
    hexes, _ = orc.parse_hexes(idx)
    o = orc.hex_schedule(nodes, hexes, morton=1 if morton else 0)
    for k in ("vert_rank", "hex_order", "colour_hex_begin"):
        assert np.array_equal(s[k], o[k]), k
    cb, order = s["colour_hex_begin"], s["hex_order"]
    for c in range(s["colours"]):
        verts = hexes[order[cb[c]:cb[c + 1]]].reshape(-1)
        assert np.unique(verts).size == verts.size


def test_hex_mesh_errors():
    nodes, idx = xfem.generate_hex_block(2, 2, 2, (0.1, 0.1, 0.1))
    tn, ti = xfem.generate_tet_block(2, 2, 2, (0.1, 0.1, 0.1))
    # a tet-only helper refuses a hex mesh and the other way round
    with pytest.raises(xfem.XfemError) as e:
        xfem.compute_rest_state(nodes, idx, 1000.0)
    assert e.value.code == xfem.EUNSUPPORTED
    with pytest.raises(xfem.XfemError):
        xfem.compute_hex_rest_state(tn, ti, 1000.0)
    # a stream mixing tets and hexes is not a hex mesh (its own helpers below)
    mixed = np.concatenate([idx[:9], ti[:5]])
    with pytest.raises(xfem.XfemError) as e:
        xfem.compute_hex_rest_state(nodes, mixed, 1000.0)
    assert e.value.code == xfem.EINVAL
    with pytest.raises(xfem.XfemError) as e:
        xfem.compute_mixed_rest_state(nodes, idx, 1000.0)
    assert e.value.code == xfem.EINVAL
    # a truncated hex record
    with pytest.raises(xfem.XfemError) as e:
        xfem.compute_hex_rest_state(nodes, idx[:-1], 1000.0)
    assert e.value.code == xfem.EINVAL


# ---- meshes mixing tets and hexes (GeoLinear3d on one tagged stream) ----
MIXED_FIX = ["mixed_c1_nh_nu045_checker", "mixed_c1_nh_incompressible_left", "mixed_wonky_yeohfast_serial_nu049_checker",
             "mixed_wonky_nh_paper_volume_checker"]


@pytest.mark.parametrize("name", MIXED_FIX)
def test_mixed_host_setup_bit_exact_vs_reference(name):
    """The library's host set-up of a mixed mesh against the reference's
    own GeoLinear3d::Init (XPBDFEM/Geo.cpp:697-745): tet and hex records,
    inverse masses of both kinds summed tets first, vertex flags; and the
    tet and hex colourings in the fixture's orders."""
    g = golden(name)
    dens = golden_args(name)["args"][10]
    ep, hep, w, fl = xfem.compute_mixed_rest_state(g["nodes"], g["idx"], dens)
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["ep"].view(np.uint32))
    assert np.array_equal(hep.reshape(-1).view(np.uint32), g["hep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])
    s = xfem.compute_mixed_schedule(g["nodes"], g["idx"])
    assert np.array_equal(s["tet_order"], g["torder"])
    assert np.array_equal(s["colour_tet_begin"], g["colour_tet_begin"])
    assert np.array_equal(s["hex_order"], g["horder"])
    assert np.array_equal(s["colour_hex_begin"], g["colour_hex_begin"])


@pytest.mark.parametrize("morton", [True, False])
def test_mixed_host_matches_oracle_on_a_jittered_block(orc, morton):
    import oracle
    nodes, idx = oracle.mixed_block(5, 4, 3, (0.05, 0.06, 0.04), 1, 0.25, lambda x, y, z: (x * 7 + y * 3 + z) % 3 == 0)
    nodes = (nodes + np.random.default_rng(3).normal(0, 0.002, nodes.shape)).astype(np.float32)
    tets, hexes, _ = orc.parse_mixed(idx)
    ep, hep, w, fl = xfem.compute_mixed_rest_state(nodes, idx, 950.0)
    e2, h2, w2, f2 = orc.mixed_init_rest(nodes, tets, hexes, 950.0)
    assert np.array_equal(ep.view(np.uint32), e2.view(np.uint32))
    assert np.array_equal(hep.view(np.uint32), h2.view(np.uint32))
    assert np.array_equal(w.view(np.uint32), w2.view(np.uint32))
    assert np.array_equal(fl, f2)
    s = xfem.compute_mixed_schedule(nodes, idx, morton=morton)
    ts = orc.tet_element_schedule(nodes, tets, morton=1 if morton else 0)
    hs = orc.hex_schedule(nodes, hexes, morton=1 if morton else 0)
    assert np.array_equal(s["vert_rank"], hs["vert_rank"])
    assert np.array_equal(s["tet_order"], ts["tet_order"])
    assert np.array_equal(s["colour_tet_begin"], ts["colour_tet_begin"])
    assert np.array_equal(s["hex_order"], hs["hex_order"])
    for order, els, cb in ((s["tet_order"], tets, s["colour_tet_begin"]), (s["hex_order"], hexes, s["colour_hex_begin"])):
        for c in range(cb.size - 1):
            verts = els[order[cb[c]:cb[c + 1]]].reshape(-1)
            assert np.unique(verts).size == verts.size


# ---- quadratic tets (GeoQuadratic3d on a tet mesh) ----
@pytest.mark.parametrize("name", ["qinit_3x2x2", "qinit_3x2x2_mirror_wonky"])
def test_t10_rest_state_bit_exact_vs_reference(name):
    """GeoQuadratic3d::Init (XPBDFEM/Geo.cpp:836-941): Connectivity3d's edge
    numbering (the T10 indices), the double midpoint positions, the T10
    records (InitTriTetFiniteElement on ElementParamsQuadraticTet), the
    inverse masses (LumpsTet10) and the flags of every vertex."""
    g = golden(name)
    a = golden_args(name)["args"]
    edges, t10 = xfem.compute_t10_edges(g["idx"])
    assert np.array_equal(t10.reshape(-1), g["t10_idx"])
    x, ep, w, fl = xfem.compute_t10_rest_state(g["nodes"], g["idx"], a[9])
    assert np.array_equal(x.reshape(-1).view(np.uint64), g["x0"].view(np.uint64))
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["qep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])


@pytest.mark.parametrize("seed", [1, 2])
def test_t10_host_matches_oracle_on_jittered_meshes(orc, seed):
    """Edges, rest state and schedule against the oracle on jittered blocks."""
    rng = np.random.default_rng(seed)
    nodes, idx = xfem.generate_tet_block(5, 3, 3, (0.03, 0.05, 0.04), seed % 2, 0.3)
    nodes = (nodes + rng.normal(0, 0.002, nodes.shape)).astype(np.float32)
    q = orc.Quadratic(nodes, idx, 700.0)
    edges, t10 = xfem.compute_t10_edges(idx)
    assert np.array_equal(edges, q.edges) and np.array_equal(t10, q.t10)
    x, ep, w, fl = xfem.compute_t10_rest_state(nodes, idx, 700.0)
    assert np.array_equal(x.view(np.uint64), q.X0.view(np.uint64))
    assert np.array_equal(ep.view(np.uint32), q.ep.view(np.uint32))
    assert np.array_equal(w.view(np.uint32), q.w.view(np.uint32))
    assert np.array_equal(fl, q.flags)
    for morton in (True, False):
        s = xfem.compute_t10_schedule(nodes, idx, morton=morton)
        o = q.schedule(morton=1 if morton else 0)
        assert np.array_equal(s["vert_rank"], o["vert_rank"])
        assert np.array_equal(s["t10_order"], o["tet_order"])
        assert np.array_equal(s["colour_t10_begin"], o["colour_tet_begin"])


@pytest.mark.parametrize("name", ["qordered_c1_nh_nu045", "qvolume_wonky_nh_serial_1_post"])
def test_t10_schedule_is_the_fixture_order(name):
    """The product's T10 colouring is the order the reference fixtures ran in."""
    g = golden(name)
    s = xfem.compute_t10_schedule(g["nodes"], g["idx"])
    assert np.array_equal(s["t10_order"], g["order"])
    assert np.array_equal(s["colour_t10_begin"], g["colour_tet_begin"])



# ---- quadratic hexes (GeoQuadratic3d on a hex mesh) ----
@pytest.mark.parametrize("name", ["h27init_2x2x1", "h27init_3x2x2_mirror_wonky"])
def test_h27_rest_state_bit_exact_vs_reference(name):
    """GeoQuadratic3d::Init on hexes (XPBDFEM/Geo.cpp:836-933): the H27
    indices (Connectivity3d's edge and quad numbering), the double positions
    of the edge, face and centre nodes, the 703-value records, the inverse
    masses and the flags of every vertex."""
    g = golden(name)
    a = golden_args(name)["args"]
    _, _, h27 = xfem.compute_h27_mesh(g["idx"])
    assert np.array_equal(h27.reshape(-1), g["h27_idx"])
    x, ep, w, fl = xfem.compute_h27_rest_state(g["nodes"], g["idx"], a[9])
    assert np.array_equal(x.reshape(-1).view(np.uint64), g["x0"].view(np.uint64))
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["h27ep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])


@pytest.mark.parametrize("seed", [1, 2])
def test_h27_host_matches_oracle_on_jittered_meshes(orc, seed):
    rng = np.random.default_rng(seed)
    nodes, idx = xfem.generate_hex_block(4, 3, 3, (0.03, 0.05, 0.04), seed % 2, 0.3)
    nodes = (nodes + rng.normal(0, 0.002, nodes.shape)).astype(np.float32)
    q = orc.QuadraticHex(nodes, idx, 700.0)
    edges, quads, h27 = xfem.compute_h27_mesh(idx)
    assert np.array_equal(edges, q.edges) and np.array_equal(quads, q.quads) and np.array_equal(h27, q.h27)
    x, ep, w, fl = xfem.compute_h27_rest_state(nodes, idx, 700.0)
    assert np.array_equal(x.view(np.uint64), q.X0.view(np.uint64))
    assert np.array_equal(ep.view(np.uint32), q.ep.view(np.uint32))
    assert np.array_equal(w.view(np.uint32), q.w.view(np.uint32))
    assert np.array_equal(fl, q.flags)
    for morton in (True, False):
        s = xfem.compute_h27_schedule(nodes, idx, morton=morton)
        o = q.schedule(morton=1 if morton else 0)
        assert np.array_equal(s["vert_rank"], o["vert_rank"])
        assert np.array_equal(s["h27_order"], o["hex_order"])
        assert np.array_equal(s["colour_h27_begin"], o["colour_hex_begin"])


@pytest.mark.parametrize("name", ["h27ordered_c1_nh_nu045", "h27volume_wonky_nh_serial_1_post"])
def test_h27_schedule_is_the_fixture_order(name):
    g = golden(name)
    s = xfem.compute_h27_schedule(g["nodes"], g["idx"])
    assert np.array_equal(s["h27_order"], g["order"])
    assert np.array_equal(s["colour_h27_begin"], g["colour_hex_begin"])
