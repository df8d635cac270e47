"""Pins the oracle restatement (oracle/xfem_oracle.c) to the reference.

Every fixture in tests/golden/ was produced by the unmodified reference code
(tests/golden/make_golden.py). The float restatement must reproduce each one
bit for bit: mesh generation (XPBDFEM/MeshGen.cpp:156-244), rest state and
masses (XPBDFEM/Fem.cpp:196-224, XPBDFEM/Geo.cpp:697-745), the MINSTD order
(XPBDFEM/Geo.cpp:759-771), single-element solves (XPBDFEM/Fem.cpp:437-564,
XPBDFEM/Xpbd.h:87-215), whole substeps (XPBDFEM/Geo.cpp:305-356), and
substeps with damping: the in-solve Rayleigh terms (XPBDFEM/Xpbd.h:87-205),
GeoLinear3d::Damp with DampElement and PbdDamp (XPBDFEM/Geo.cpp:346-355,
790-811; XPBDFEM/Fem.cpp:908-931; XPBDFEM/Xpbd.h:217-346), amortized or not;
every energy model SolveElement dispatches on a linear tet
(XPBDFEM/Fem.cpp:872-888), and volume passes (XPBDFEM/Fem.cpp:840-867).
Linear hexahedra the same way: GenerateHexBlock, InitQuadHexFiniteElement
(XPBDFEM/Fem.cpp:225-265), SolveElement on H8 for every energy model but the
continuous-pressure ones (the cube models' SolveElementCube included), and
whole substeps with the hex loops of GeoLinear3d::Constrain and Damp
(XPBDFEM/Geo.cpp:774-811).
"""
import numpy as np
import pytest

from conftest import golden, golden_args

MESH = ["meshgen_8x2x2", "meshgen_3x2x2_mirror_wonky", "meshgen_4x3x2_aniso_wonky"]
INIT = ["init_8x2x2", "init_3x2x2_mirror_wonky", "init_5x3x2_aniso_wonky"]
SOLVE = ["solve_nh_sim_incompressible", "solve_nh_sim_nu045", "solve_yeoh_sim_incompressible",
         "solve_nh_serial_nu045", "solve_yeoh_serial_nu049",
         # the other energy models (XPBDFEM/Fem.cpp:361-433, 459-522, 872-888)
         "solve_pixar_nu045", "solve_pixar_reduced_nu040", "solve_pixarsel_nu049", "solve_mixed_sim_nu045",
         "solve_mixed_sim_incompressible", "solve_mixed_serial_nu049", "solve_yeohskin_sim_nu045",
         "solve_yeohskin_sim_incompressible", "solve_yeohskinsel_serial_nu049", "solve_cube_neo_noop",
         "solve_id20_mixedsel"]
SUBSTEP = ["substep_c1_nh_native", "substep_c1_yeoh_native", "substep_wonky_nh_serial_native",
           "ordered_c1_nh_star", "ordered_c1_yeoh_tet", "ordered_c1_nh_nu045_star", "ordered_c1_yeoh_nu049_tet",
           "ordered_wonky_nh_serial_nu045_star", "ordered_c1_nh_100frames_star", "ordered_c1_yeoh_100frames_star"]
DAMPED = ["damped_c1_nh_nu045_amortized_pbd_star", "damped_c1_nh_nu045_post_star", "damped_c1_nh_nu045_paper_star",
          "damped_c1_nh_nu045_limit_star", "damped_c1_yeoh_nu049_amortized_pbd_tet",
          "damped_wonky_nh_serial_post_pbd_star", "damped_wonky_nh_serial_limit_pbd_star"]
# energy models other than MixedSel / YeohSkinFast, and volume passes
# (SolveElementVolume, XPBDFEM/Fem.cpp:840-867; XPBDFEM/Geo.cpp:780-783), in
# the `damped` form (damping 0 where none is wanted)
MODELS = ["model_c1_pixar_nu045_star", "model_c1_pixarsel_nu045_tet", "model_c1_mixed_nu045_star",
          "model_wonky_mixed_serial_nu045_star", "model_c1_yeohskin_nu049_tet",
          "model_wonky_yeohskinsel_serial_nu049_star", "model_c1_cube_pbd_star", "model_c1_pixar_amortized_pbd_star",
          "model_c1_pixar_paper_tet", "model_c1_mixed_limit_star", "model_wonky_yeohskin_serial_post_star",
          "volume_c1_nh_nu045_2_star", "volume_c1_yeoh_nu049_3_tet", "volume_wonky_pixar_1_post_pbd_star"]


@pytest.mark.parametrize("name", MESH)
def test_meshgen_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    nodes, idx = orc.gen_tet_block(a[1], a[2], a[3], tuple(a[4:7]), a[7], a[8])
    assert np.array_equal(idx, g["idx"])
    assert np.array_equal(nodes.view(np.uint32), g["nodes"].view(np.uint32))


@pytest.mark.parametrize("name", INIT)
def test_rest_state_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    tets, nv = orc.parse_tets(g["idx"])
    assert np.array_equal(tets.reshape(-1), g["tet_idx"])
    ep, w, fl = orc.init_rest(g["nodes"], tets, a[9])
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["ep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])
    assert np.array_equal(orc.minstd_order(tets.shape[0]), g["torder"])
    X = g["nodes"].astype(np.float64)
    assert np.float32(orc.volume(X, tets)).view(np.uint32) == g["volume"].view(np.uint32)[0]


@pytest.mark.parametrize("name", SOLVE)
def test_element_solve_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    p = orc.make_params(dt=a[7], compliance=a[5], poisson=a[6], energy=a[3], simultaneous=bool(a[4]))
    n = a[2]
    xin, xout = g["xin"].reshape(n, 4, 3), g["xout"].reshape(n, 4, 3)
    ep, w, rest = g["ep"].reshape(n, 17), g["w"].reshape(n, 4), g["rest"].reshape(n, 4, 3)
    for t in range(n):
        # rest state of the random tet (InitFiniteElement on float-rounded nodes)
        e, _, _ = orc.init_rest(rest[t].astype(np.float32).reshape(-1), np.array([[0, 1, 2, 3]], np.uint32), 1000.0)
        assert np.array_equal(e[0].view(np.uint32), ep[t].view(np.uint32)), t
        x, _ = orc.solve_tet(xin[t], w[t], ep[t], p)
        assert np.array_equal(x.view(np.uint64), xout[t].view(np.uint64)), t


@pytest.mark.parametrize("name", SUBSTEP)
def test_substeps_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    W, H, D, sx, sy, sz, wonk, dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[1:]
    tets, nv = orc.parse_tets(g["idx"])
    ep, w, fl = orc.init_rest(g["nodes"], tets, dens)
    order = g["order"] if "order" in g else orc.minstd_order(tets.shape[0])
    p = orc.make_params(dt=dt, compliance=comp, poisson=nu, energy=energy, simultaneous=bool(simul),
                        gravity=(gx, gy, 0.0), lock=bool(lock))
    X0 = g["nodes"].astype(np.float64)
    V0 = np.zeros_like(X0)
    lock_mask = (fl & 1).astype(np.uint8)
    X1, V1, w1, _ = orc.substeps(X0, V0, w, tets, ep, order, 1, p, lock_mask=lock_mask)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = orc.substeps(X1, V1, w1, tets, ep, order, nsub - 1, p, lock_mask=lock_mask)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(orc.volume(Xn, tets)).view(np.uint32) == g["volume"].view(np.uint32)[0]


def damped_params(orc, a, derived, tick):
    """orc_params of a `damped` fixture (refgen's argument order)."""
    W, H, D, sx, sy, sz, wonk, dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[1:18]
    damping, pbd, drag, rtype, spacing = a[18:23]
    vpasses = a[23] if len(a) > 23 else 0
    return orc.make_params(dt=dt, compliance=comp, poisson=nu, energy=energy, simultaneous=bool(simul),
                           gravity=(gx, gy, 0.0), lock=bool(lock), drag=float(derived[2]), damping=damping,
                           rayleigh_type=rtype, pbd_damping=pbd, pbd_coeff=float(derived[0]),
                           pbd_coeff_amortized=float(derived[1]), tick=tick, volume_passes=vpasses)


@pytest.mark.parametrize("name", DAMPED + MODELS)
def test_damped_substeps_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    dens, nsub = a[8], a[16]
    tets, nv = orc.parse_tets(g["idx"])
    ep, w, fl = orc.init_rest(g["nodes"], tets, dens)
    order = g["order"]
    X0 = g["nodes"].astype(np.float64)
    V0 = np.zeros_like(X0)
    lock_mask = (fl & 1).astype(np.uint8)
    X1, V1, w1, _ = orc.substeps(X0, V0, w, tets, ep, order, 1, damped_params(orc, a, g["derived"], 0),
                                 lock_mask=lock_mask)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = orc.substeps(X1, V1, w1, tets, ep, order, nsub - 1, damped_params(orc, a, g["derived"], 1),
                                lock_mask=lock_mask)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    # the damping, the model and the volume passes each did something: the
    # run without them differs
    p0 = damped_params(orc, a, g["derived"], 0)
    if p0.damping > 0 or p0.pbd_damping > 0:
        p0.damping, p0.pbd_damping = 0.0, 0.0
    elif p0.volume_passes:
        p0.volume_passes = 0
    else:
        p0.energy = orc.ENERGY_MIXED_SEL
    Xu, _, _, _ = orc.substeps(X0, V0, w, tets, ep, order, nsub, p0, lock_mask=lock_mask)
    assert not np.array_equal(Xu.reshape(-1), g["xn"])


LOCKED = ["locked_c1_nh_nu045_star", "locked_c1_yeoh_nu049_amortized_pbd_tet",
          "locked_wonky_nh_serial_nu045_right_only_star"]


def locked_params(orc, a, derived, tick, nodes):
    """orc_params of a `locked` fixture: the `damped` ones plus the Right
    lock's targets from lockedRightTransform3d and Geo3d::origin."""
    p = damped_params(orc, a[:24], derived, tick)
    targets = orc.right_targets(nodes, a[24:33], a[33:36])
    return orc.make_params(dt=p.dt, compliance=p.compliance, poisson=p.poisson, energy=p.energy,
                           simultaneous=bool(p.simultaneous), gravity=tuple(p.gravity), lock=bool(p.lock_active),
                           drag=p.time_corrected_drag, damping=p.damping, rayleigh_type=p.rayleigh_type,
                           pbd_damping=p.pbd_damping, pbd_coeff=p.pbd_coeff, pbd_coeff_amortized=p.pbd_coeff_amortized,
                           tick=tick, volume_passes=p.volume_passes, right_target=targets)


@pytest.mark.parametrize("name", LOCKED)
def test_locked_right_substeps_bit_exact(orc, name):
    """Settings_LockRight (XPBDFEM/Geo.cpp:323-331): the Right vertices (x
    above 98% of the extent) end every substep at origin +
    lockedRightTransform3d X0 with a zero inverse mass, after the Left lock;
    the oracle in the fixture's order equals the reference bit for bit."""
    g = golden(name)
    a = golden_args(name)["args"]
    dens, nsub = a[8], a[16]
    tets, nv = orc.parse_tets(g["idx"])
    ep, w, fl = orc.init_rest(g["nodes"], tets, dens)
    assert (fl & 2).any()
    order = g["order"]
    X0 = g["nodes"].astype(np.float64)
    V0 = np.zeros_like(X0)
    lock_mask = (fl & 3).astype(np.uint8)
    X1, V1, w1, _ = orc.substeps(X0, V0, w, tets, ep, order, 1, locked_params(orc, a, g["derived"], 0, g["nodes"]),
                                 lock_mask=lock_mask)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, wn, _ = orc.substeps(X1, V1, w1, tets, ep, order, nsub - 1,
                                 locked_params(orc, a, g["derived"], 1, g["nodes"]), lock_mask=lock_mask)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.all(wn[(fl & 2) != 0] == 0)
    # the lock moved them: without it the run differs
    Xu, _, _, _ = orc.substeps(X0, V0, w, tets, ep, order, nsub, damped_params(orc, a[:24], g["derived"], 0),
                               lock_mask=lock_mask)
    assert not np.array_equal(Xu.reshape(-1), g["xn"])


RINGS = ["rings_c1_cpixar_nu045_star", "rings_c1_cmixed_nu045_star", "rings_c1_cmixed_incompressible_star",
         "rings_c1_cskin_nu049_star", "rings_wonky_cmixed_paper_star", "rings_c1_cskin_limit_star",
         "rings_c1_cmixed_amortized_pbd_star", "rings_wonky_cpixar_post_star"]


@pytest.mark.parametrize("name", RINGS)
def test_ring_substeps_bit_exact(orc, name):
    """The continuous-pressure models: every vertex's one-ring solved in the
    fixture's vertex order (XPBDFEM/Geo.cpp:147-193, 774-811;
    XPBDFEM/Fem.cpp:942-979; XPBDFEM/Geo.cpp:12-64), with damping where the
    fixture has it; and the ring schedule restatement reproduces the order."""
    g = golden(name)
    a = golden_args(name)["args"]
    dens, nsub = a[8], a[16]
    tets, nv = orc.parse_tets(g["idx"])
    rs = orc.ring_schedule(g["nodes"], tets, morton=1)
    assert np.array_equal(rs["vert_order"], g["vorder"])
    assert np.array_equal(rs["colour_vert_begin"], g["colour_vert_begin"])
    ep, w, fl = orc.init_rest(g["nodes"], tets, dens)
    X0 = g["nodes"].astype(np.float64)
    V0 = np.zeros_like(X0)
    lock_mask = (fl & 1).astype(np.uint8)
    X1, V1, w1, _ = orc.substeps_rings(X0, V0, w, tets, ep, g["order"], g["vorder"], 1,
                                       damped_params(orc, a, g["derived"], 0), lock_mask=lock_mask)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = orc.substeps_rings(X1, V1, w1, tets, ep, g["order"], g["vorder"], nsub - 1,
                                      damped_params(orc, a, g["derived"], 1), lock_mask=lock_mask)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))


def test_ring_schedule_is_a_valid_colouring(orc):
    """Rings of one colour share no node, on a jittered shuffled mesh."""
    rng = np.random.default_rng(4)
    nodes, idx = orc.gen_tet_block(5, 4, 3, (0.1, 0.1, 0.1), 1, 0.3)
    tets, nv = orc.parse_tets(idx)
    perm = rng.permutation(tets.shape[0])
    tets = tets[perm]
    rs = orc.ring_schedule(nodes, tets, morton=1)
    assert np.array_equal(np.sort(rs["vert_order"]), np.arange(nv))
    ring = [set() for _ in range(nv)]
    for t in tets:
        for v in t:
            ring[v].update(int(x) for x in t)
    for v in range(nv):
        ring[v].add(v)
    cb = rs["colour_vert_begin"]
    for c in range(cb.size - 1):
        seen = set()
        for v in rs["vert_order"][cb[c]:cb[c + 1]]:
            assert not (ring[v] & seen), c
            seen |= ring[v]


def test_cube_models_leave_tets_untouched(orc):
    """SolveElementCube acts on quads and hexes only: on a tet mesh the
    substep is free fall (XPBDFEM/Fem.cpp:568-838)."""
    g = golden("solve_cube_neo_noop")
    assert np.array_equal(g["xin"], g["xout"])


def test_continuous_models_refused(orc):
    """The continuous-pressure models (8-10) run a per-vertex ring solve,
    not an element solve: the element restatement refuses them (and the ring
    restatement refuses element models)."""
    g = golden("solve_pixar_nu045")
    for e in (8, 9, 10):
        p = orc.make_params(dt=1 / 1200, compliance=0.01, poisson=0.45, energy=e)
        with pytest.raises(ValueError):
            orc.solve_tet(g["xin"][:12], g["w"][:4], g["ep"][:17], p)


# ---- linear hexahedra (GeoLinear3d's hex loops; oracle/xfem_oracle_hex.inc) ----
HINIT = ["hinit_4x2x2", "hinit_3x2x2_mirror_wonky", "hinit_4x3x2_aniso_wonky"]
HSOLVE = ["hsolve_nh_sim_nu045", "hsolve_nh_sim_incompressible", "hsolve_nh_serial_nu045",
          "hsolve_yeohfast_sim_nu049", "hsolve_yeohfast_serial_incompressible", "hsolve_mixed_sim_nu045",
          "hsolve_mixed_serial_nu049", "hsolve_yeohskin_sim_nu045", "hsolve_yeohskinsel_sim_nu049",
          "hsolve_yeohskinsel_serial_nu045", "hsolve_pixar_nu045", "hsolve_pixar_reduced_nu040",
          "hsolve_pixarsel_nu049", "hsolve_id20_mixedsel",
          # SolveElementCube (XPBDFEM/Fem.cpp:566-838): the short path (CubeNeo,
          # nu = 0.5, no damping) and the general one
          "hsolve_cube_neo_fast", "hsolve_cube_neo_nu045", "hsolve_cube_skin_nu049", "hsolve_cube_skin_incompressible"]
HSUBSTEP = ["hordered_c1_nh_nu045", "hordered_c1_nh_incompressible", "hordered_c1_yeohfast_nu049",
            "hordered_wonky_nh_serial_nu045", "hordered_c1_mixed_nu045", "hordered_wonky_yeohskinsel_serial_nu049",
            "hordered_c1_pixar_nu045", "hdamped_c1_nh_nu045_post_pbd", "hdamped_c1_nh_nu045_amortized_pbd",
            "hdamped_c1_nh_nu045_paper", "hdamped_c1_nh_nu045_limit", "hdamped_wonky_yeohskin_serial_post",
            "hvolume_c1_nh_nu045_2", "hvolume_wonky_pixar_1_post_pbd", "hordered_c1_cube_neo_fast",
            "hordered_wonky_cube_neo_nu045", "hordered_c1_cube_skin_nu049", "hdamped_c1_cube_neo_nu045_paper",
            "hdamped_c1_cube_skin_nu045_limit", "hdamped_c1_cube_neo_incompressible_amortized_pbd"]


def test_hex_meshgen_bit_exact(orc):
    g = golden("hmeshgen_3x2x2_mirror_wonky")
    a = golden_args("hmeshgen_3x2x2_mirror_wonky")["args"]
    nodes, idx = orc.gen_hex_block(a[1], a[2], a[3], tuple(a[4:7]), a[7], a[8])
    assert np.array_equal(idx, g["idx"])
    assert np.array_equal(nodes.view(np.uint32), g["nodes"].view(np.uint32))


def test_hex_tables_structure(orc):
    """The hex tables built from the reference's printed magnitudes: shape
    functions sum to ~1 at every point, gradients to ~0, and the centre
    gradients are the means of the Gauss-point ones up to the printing."""
    n8, g8, g1 = orc.hex_tables()
    assert np.allclose(n8.sum(1), 1.0, atol=1e-5)
    assert np.allclose(g8.sum(1), 0.0, atol=1e-6)
    assert np.allclose(g8.mean(0), g1, atol=1e-6)
    assert np.array_equal(n8, n8.T)  # the point and node numberings agree


@pytest.mark.parametrize("name", HINIT)
def test_hex_rest_state_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    hexes, nv = orc.parse_hexes(g["idx"])
    assert np.array_equal(hexes.reshape(-1), g["hex_idx"])
    ep, w, fl = orc.hex_init_rest(g["nodes"], hexes, a[9])
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["hep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])
    assert np.array_equal(orc.minstd_order(hexes.shape[0]), g["horder"])
    X = g["nodes"].astype(np.float64)
    assert np.float32(orc.hex_volume(X, hexes, ep)).view(np.uint32) == g["volume"].view(np.uint32)[0]


@pytest.mark.parametrize("name", HSOLVE)
def test_hex_element_solve_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    p = orc.make_params(dt=a[7], compliance=a[5], poisson=a[6], energy=a[3], simultaneous=bool(a[4]))
    n = a[2]
    xin, xout = g["xin"].reshape(n, 8, 3), g["xout"].reshape(n, 8, 3)
    ep, w, rest = g["hep"].reshape(n, orc.HEX_EP), g["w"].reshape(n, 8), g["rest"].reshape(n, 8, 3)
    one = np.arange(8, dtype=np.uint32)[None]
    for t in range(n):
        e, _, _ = orc.hex_init_rest(rest[t].astype(np.float32).reshape(-1), one, 1000.0)
        assert np.array_equal(e[0].view(np.uint32), ep[t].view(np.uint32)), t
        x = orc.solve_hex(xin[t], w[t], ep[t], p, O=rest[t])
        assert np.array_equal(x.view(np.uint64), xout[t].view(np.uint64)), t


def hex_params(orc, a, g, tick):
    """orc_params of an `hordered` / `hdamped` fixture (refgen's argument order)."""
    energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[10:19]
    kw = dict(rayleigh_type=2)
    if a[0] in ("hdamped", "hrings"):
        damping, pbd, drag, rtype, spacing = a[19:24]
        d = g["derived"]
        kw = dict(damping=damping, rayleigh_type=rtype, pbd_damping=pbd, pbd_coeff=float(d[0]),
                  pbd_coeff_amortized=float(d[1]), drag=float(d[2]), volume_passes=a[24] if len(a) > 24 else 0)
    return orc.make_params(dt=dt, compliance=comp, poisson=nu, energy=energy, simultaneous=bool(simul),
                           gravity=(gx, gy, 0.0), lock=bool(lock), tick=tick, **kw)


@pytest.mark.parametrize("name", HSUBSTEP)
def test_hex_substeps_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    dens, nsub = a[9], a[17]
    hexes, nv = orc.parse_hexes(g["idx"])
    ep, w, fl = orc.hex_init_rest(g["nodes"], hexes, dens)
    # the fixture ran in the hex schedule's colour order
    sch = orc.hex_schedule(g["nodes"], hexes)
    assert np.array_equal(sch["hex_order"], g["order"])
    assert np.array_equal(sch["colour_hex_begin"], g["colour_hex_begin"])
    X0 = g["nodes"].astype(np.float64)
    V0 = np.zeros_like(X0)
    lm = (fl & 1).astype(np.uint8)
    X1, V1, w1, _ = orc.hex_substeps(X0, V0, w, hexes, ep, g["order"], 1, hex_params(orc, a, g, 0), lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = orc.hex_substeps(X1, V1, w1, hexes, ep, g["order"], nsub - 1, hex_params(orc, a, g, 1),
                                    lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(orc.hex_volume(Xn, hexes, ep)).view(np.uint32) == g["volume"].view(np.uint32)[0]


HRINGS = ["hrings_c1_cpixar_nu045", "hrings_c1_cmixed_nu045", "hrings_c1_cmixed_incompressible",
          "hrings_c1_cskin_nu049", "hrings_wonky_cmixed_paper", "hrings_c1_cskin_limit",
          "hrings_c1_cmixed_amortized_pbd", "hrings_wonky_cpixar_post"]


@pytest.mark.parametrize("name", HRINGS)
def test_hex_ring_substeps_bit_exact(orc, name):
    """The continuous-pressure models on a hex mesh: every vertex's one-ring
    (its hexes) solved in the fixture's vertex order through the full-energy
    branch (XPBDFEM/Geo.cpp:147-225, 774-811; XPBDFEM/Fem.cpp:983-1036), the
    PBD damping over the hexes in the fixture's hex order; and the ring
    schedule restatement reproduces the vertex order."""
    g = golden(name)
    a = golden_args(name)["args"]
    dens, nsub = a[9], a[17]
    hexes, nv = orc.parse_hexes(g["idx"])
    rs = orc.ring_schedule(g["nodes"], hexes, morton=1)
    assert np.array_equal(rs["vert_order"], g["vorder"])
    assert np.array_equal(rs["colour_vert_begin"], g["colour_vert_begin"])
    ep, w, fl = orc.hex_init_rest(g["nodes"], hexes, dens)
    X0 = g["nodes"].astype(np.float64)
    V0 = np.zeros_like(X0)
    lm = (fl & 1).astype(np.uint8)
    X1, V1, w1, _ = orc.hex_substeps_rings(X0, V0, w, hexes, ep, g["order"], g["vorder"], 1, hex_params(orc, a, g, 0),
                                           lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = orc.hex_substeps_rings(X1, V1, w1, hexes, ep, g["order"], g["vorder"], nsub - 1,
                                          hex_params(orc, a, g, 1), lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))


MIXED = ["mixed_c1_nh_nu045_checker", "mixed_c1_nh_incompressible_left", "mixed_wonky_yeohfast_serial_nu049_checker",
         "mixed_c1_pixar_nu045_amortized_pbd_checker", "mixed_c1_mixed_nu045_limit_left",
         "mixed_wonky_nh_paper_volume_checker", "mixed_c1_cube_neo_nu045_post_checker",
         "mixed_c1_yeohskin_nu045_post_pbd_left"]


def mixed_params(orc, a, g, tick):
    """orc_params of a `mixed` fixture (its arguments after the mesh ones)."""
    dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock, damping, pbd, drag, rtype, spacing, vpasses = a[10:26]
    d = g["derived"]
    return orc.make_params(dt=dt, compliance=comp, poisson=nu, energy=energy, simultaneous=bool(simul),
                           gravity=(gx, gy, 0.0), lock=bool(lock), tick=tick, damping=damping, rayleigh_type=rtype,
                           pbd_damping=pbd, pbd_coeff=float(d[0]), pbd_coeff_amortized=float(d[1]), drag=float(d[2]),
                           volume_passes=vpasses)


@pytest.mark.parametrize("name", MIXED)
def test_mixed_mesh_substeps_bit_exact(orc, name):
    """A mesh mixing tets and hexes (GeoLinear3d on one tagged stream): rest
    state with the masses of both kinds summed tets first, then substeps
    that solve every tet, then every hex, and damp likewise
    (XPBDFEM/Geo.cpp:697-745, 777-811), in the fixture's tet and hex colour
    orders, which the element schedule restatement reproduces."""
    g = golden(name)
    a = golden_args(name)["args"]
    dens, nsub = a[10], a[18]
    tets, hexes, nv = orc.parse_mixed(g["idx"])
    assert tets.shape[0] and hexes.shape[0] and nv == g["nodes"].size // 3
    ep, hep, w, fl = orc.mixed_init_rest(g["nodes"], tets, hexes, dens)
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["ep"].view(np.uint32))
    assert np.array_equal(hep.reshape(-1).view(np.uint32), g["hep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(fl, g["vflags"])
    ts = orc.tet_element_schedule(g["nodes"], tets, morton=1)
    hs = orc.hex_schedule(g["nodes"], hexes, morton=1)
    assert np.array_equal(ts["tet_order"], g["torder"]) and np.array_equal(hs["hex_order"], g["horder"])
    X0 = g["nodes"].astype(np.float64)
    lm = (fl & 1).astype(np.uint8)
    X1, V1, w1, _ = orc.mixed_substeps(X0, np.zeros_like(X0), w, tets, ep, g["torder"], hexes, hep, g["horder"], 1,
                                       mixed_params(orc, a, g, 0), lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = orc.mixed_substeps(X1, V1, w1, tets, ep, g["torder"], hexes, hep, g["horder"], nsub - 1,
                                      mixed_params(orc, a, g, 1), lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(orc.mixed_volume(Xn, tets, hexes, hep)).view(np.uint32) == g["volume"].view(np.uint32)[0]


def test_hex_schedule_is_a_valid_colouring(orc):
    """Hexes of one colour share no vertex; greedy first fit in id order
    (each hex takes the smallest colour free among earlier neighbours)."""
    nodes, idx = orc.gen_hex_block(5, 4, 3, (0.1, 0.1, 0.1), 1, 0.3)
    hexes, nv = orc.parse_hexes(idx)
    s = orc.hex_schedule(nodes, hexes)
    cb, order = s["colour_hex_begin"], s["hex_order"]
    assert sorted(order.tolist()) == list(range(hexes.shape[0]))
    colour = np.empty(hexes.shape[0], np.int64)
    for c in range(s["colours"]):
        hs = order[cb[c]:cb[c + 1]]
        colour[hs] = c
        verts = hexes[hs].reshape(-1)
        assert np.unique(verts).size == verts.size
    for h in range(hexes.shape[0]):
        nb = [k for k in range(h) if np.intersect1d(hexes[k], hexes[h]).size]
        taken = {int(colour[k]) for k in nb}
        assert colour[h] == min(set(range(65)) - taken)
    assert s["colours"] == 8  # a structured block needs exactly 8


def test_hex_continuous_models_refused(orc):
    nodes, idx = orc.gen_hex_block(2, 1, 1, (0.1, 0.1, 0.1))
    hexes, nv = orc.parse_hexes(idx)
    ep, w, fl = orc.hex_init_rest(nodes, hexes, 1000.0)
    X = nodes.astype(np.float64).reshape(-1, 3)
    for e in (8, 9, 10):
        p = orc.make_params(dt=1e-3, compliance=1e-3, poisson=0.45, energy=e)
        with pytest.raises(ValueError):
            orc.hex_substeps(X, np.zeros_like(X), w, hexes, ep, np.arange(2, dtype=np.uint32), 1, p)


# ---- quadratic tetrahedra (GeoQuadratic3d; oracle/xfem_oracle_t10.inc) ----
QINIT = ["qinit_3x2x2", "qinit_3x2x2_mirror_wonky"]
QSOLVE = ["qsolve_nh_sim_nu045", "qsolve_nh_sim_incompressible", "qsolve_nh_serial_nu045",
          "qsolve_yeohfast_sim_nu049", "qsolve_mixed_sim_nu045", "qsolve_yeohskinsel_serial_nu045",
          "qsolve_pixar_nu045", "qsolve_pixarsel_nu049"]
QSUBSTEP = ["qordered_c1_nh_nu045", "qordered_c1_nh_incompressible", "qordered_wonky_yeohfast_serial_nu049",
            "qordered_c1_mixed_nu045", "qdamped_c1_nh_nu045_amortized_pbd", "qdamped_c1_pixar_nu045_limit",
            "qvolume_wonky_nh_serial_1_post"]


def test_t10_tables_structure(orc):
    """The quadratic-tet tables built from the reference's printed
    magnitudes: gradients sum to ~0 at every point (the shape functions are a
    partition of unity) and the weights to 1."""
    g4, g10, w10 = orc.t10_tables()
    assert np.allclose(g4.sum(1), 0.0, atol=5e-6)
    assert np.allclose(g10.sum(1), 0.0, atol=5e-6)
    assert abs(float(w10.sum()) - 1.0) < 1e-5


@pytest.mark.parametrize("name", QINIT)
def test_t10_rest_state_bit_exact(orc, name):
    """GeoQuadratic3d::Init: Connectivity3d's edge numbering (the midpoint
    vertex ids), midpoint positions, flags of all vertices, T10 records,
    masses, the MINSTD order and CalculateVolume."""
    g = golden(name)
    a = golden_args(name)["args"]
    q = orc.Quadratic(g["nodes"], g["idx"], a[9])
    assert np.array_equal(q.t10.reshape(-1), g["t10_idx"])
    assert np.array_equal(q.X0.reshape(-1).view(np.uint64), g["x0"].view(np.uint64))
    assert np.array_equal(q.ep.reshape(-1).view(np.uint32), g["qep"].view(np.uint32))
    assert np.array_equal(q.w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(q.flags, g["vflags"])
    assert np.array_equal(orc.minstd_order(q.t10.shape[0]), g["torder"])
    assert np.float32(q.volume(q.X0)).view(np.uint32) == g["volume"].view(np.uint32)[0]


@pytest.mark.parametrize("name", QSOLVE)
def test_t10_element_solve_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    p = orc.make_params(dt=a[7], compliance=a[5], poisson=a[6], energy=a[3], simultaneous=bool(a[4]))
    n = a[2]
    xin, xout = g["xin"].reshape(n, 10, 3), g["xout"].reshape(n, 10, 3)
    ep, w, rest = g["qep"].reshape(n, orc.T10_EP), g["w"].reshape(n, 10), g["rest"].reshape(n, 10, 3)
    for t in range(n):
        x = orc.solve_t10(xin[t], w[t], ep[t], p, O=rest[t])
        assert np.array_equal(x.view(np.uint64), xout[t].view(np.uint64)), t


def q_params(orc, a, g, tick):
    """orc_params of a `qordered` / `qdamped` (T10) or `Qordered` / `Qdamped` (H27) fixture."""
    energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[10:19]
    kw = dict(rayleigh_type=2)
    if a[0] in ("qdamped", "Qdamped", "qrings", "Qrings"):
        damping, pbd, drag, rtype, spacing = a[19:24]
        d = g["derived"]
        kw = dict(damping=damping, rayleigh_type=rtype, pbd_damping=pbd, pbd_coeff=float(d[0]),
                  pbd_coeff_amortized=float(d[1]), drag=float(d[2]), volume_passes=a[24] if len(a) > 24 else 0)
    return orc.make_params(dt=dt, compliance=comp, poisson=nu, energy=energy, simultaneous=bool(simul),
                           gravity=(gx, gy, 0.0), lock=bool(lock), tick=tick, **kw)


@pytest.mark.parametrize("name", QSUBSTEP)
def test_t10_substeps_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    q = orc.Quadratic(g["nodes"], g["idx"], a[9])
    sch = q.schedule()
    assert np.array_equal(sch["tet_order"], g["order"])
    assert np.array_equal(sch["colour_tet_begin"], g["colour_tet_begin"])
    lm = (q.flags & 1).astype(np.uint8)
    X1, V1, w1, _ = q.substeps(q.X0, np.zeros_like(q.X0), q.w, g["order"], 1, q_params(orc, a, g, 0), lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = q.substeps(X1, V1, w1, g["order"], a[17] - 1, q_params(orc, a, g, 1), lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(q.volume(Xn)).view(np.uint32) == g["volume"].view(np.uint32)[0]


QRINGS = ["qrings_c1_cpixar_nu045", "qrings_c1_cmixed_nu045", "qrings_c1_cmixed_incompressible",
          "qrings_c1_cskin_nu049", "qrings_wonky_cmixed_paper", "qrings_c1_cskin_limit",
          "qrings_c1_cmixed_amortized_pbd", "qrings_wonky_cpixar_post"]


@pytest.mark.parametrize("name", QRINGS)
def test_t10_rings_bit_exact(orc, name):
    """The continuous-pressure models on quadratic tets: GeoQuadratic3d's
    rings of the mesh's own vertices over the T10s around them (SolveRing,
    XPBDFEM/Geo.cpp:147-225, 944-953, 971-1008) in the fixture's ring order,
    which the centres-only ring schedule reproduces; PBD damping over the
    T10s in the fixture's T10 order."""
    g = golden(name)
    a = golden_args(name)["args"]
    q = orc.Quadratic(g["nodes"], g["idx"], a[9])
    assert np.array_equal(q.schedule()["tet_order"], g["order"])
    rs = q.ring_schedule()
    assert np.array_equal(rs["vert_order"], g["vorder"])
    assert np.array_equal(rs["colour_vert_begin"], g["colour_vert_begin"])
    lm = (q.flags & 1).astype(np.uint8)
    X1, V1, w1, _ = q.substeps_rings(q.X0, np.zeros_like(q.X0), q.w, g["order"], g["vorder"], 1,
                                     q_params(orc, a, g, 0), lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = q.substeps_rings(X1, V1, w1, g["order"], g["vorder"], a[17] - 1, q_params(orc, a, g, 1),
                                    lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(q.volume(Xn)).view(np.uint32) == g["volume"].view(np.uint32)[0]


def test_t10_schedule_is_a_valid_colouring(orc):
    nodes, idx = orc.gen_tet_block(4, 3, 2, (0.1, 0.1, 0.1), 1, 0.3)
    q = orc.Quadratic(nodes, idx, 1000.0)
    s = q.schedule()
    cb, order = s["colour_tet_begin"], s["tet_order"]
    assert sorted(order.tolist()) == list(range(q.t10.shape[0]))
    for c in range(s["colours"]):
        verts = q.t10[order[cb[c]:cb[c + 1]]].reshape(-1)
        assert np.unique(verts).size == verts.size


# ---- quadratic hexahedra (GeoQuadratic3d on hexes; oracle/xfem_oracle_h27.inc) ----
H27INIT = ["h27init_2x2x1", "h27init_3x2x2_mirror_wonky"]
H27SOLVE = ["h27solve_nh_sim_nu045", "h27solve_nh_sim_incompressible", "h27solve_nh_serial_nu045",
            "h27solve_yeohfast_sim_nu049", "h27solve_mixed_sim_nu045", "h27solve_yeohskinsel_serial_nu045",
            "h27solve_pixar_nu045", "h27solve_pixarsel_nu049"]
H27SUBSTEP = ["h27ordered_c1_nh_nu045", "h27ordered_c1_nh_incompressible", "h27ordered_wonky_yeohfast_serial_nu049",
              "h27ordered_c1_mixed_nu045", "h27damped_c1_nh_nu045_amortized_pbd", "h27damped_c1_pixar_nu045_limit",
              "h27volume_wonky_nh_serial_1_post"]


def test_h27_tables_structure(orc):
    """The 27-node tables from the printed 1-D Gauss points and weights: the
    gradients sum to ~0 at every point, the shape functions to ~1, the
    weights to 8 (the cube [-1, 1]^3), and the corner map's gradients are
    those of the trilinear map."""
    g8, g27, n27, map27, w27 = orc.h27_tables()
    assert np.allclose(g8.sum(1), 0.0, atol=5e-6) and np.allclose(g27.sum(1), 0.0, atol=5e-6)
    assert np.allclose(n27.sum(1), 1.0, atol=5e-6)
    assert abs(float(w27.sum()) - 8.0) < 1e-4
    assert np.allclose(map27.sum(1), 0.0, atol=5e-6)


@pytest.mark.parametrize("name", H27INIT)
def test_h27_rest_state_bit_exact(orc, name):
    """GeoQuadratic3d::Init on hexes: Connectivity3d's edge and quad
    numbering (the H27 indices), edge, face and hex-centre positions, flags
    of all vertices, the 703-value records, masses and CalculateVolume."""
    g = golden(name)
    a = golden_args(name)["args"]
    q = orc.QuadraticHex(g["nodes"], g["idx"], a[9])
    assert np.array_equal(q.h27.reshape(-1), g["h27_idx"])
    assert np.array_equal(q.X0.reshape(-1).view(np.uint64), g["x0"].view(np.uint64))
    assert np.array_equal(q.ep.reshape(-1).view(np.uint32), g["h27ep"].view(np.uint32))
    assert np.array_equal(q.w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(q.flags, g["vflags"])
    assert np.array_equal(orc.minstd_order(q.h27.shape[0]), g["horder"])
    assert np.float32(q.volume(q.X0)).view(np.uint32) == g["volume"].view(np.uint32)[0]


@pytest.mark.parametrize("name", H27SOLVE)
def test_h27_element_solve_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    p = orc.make_params(dt=a[7], compliance=a[5], poisson=a[6], energy=a[3], simultaneous=bool(a[4]))
    n = a[2]
    xin, xout = g["xin"].reshape(n, 27, 3), g["xout"].reshape(n, 27, 3)
    ep, w, rest = g["h27ep"].reshape(n, orc.H27_EP), g["w"].reshape(n, 27), g["rest"].reshape(n, 27, 3)
    for t in range(n):
        x = orc.solve_h27(xin[t], w[t], ep[t], p, O=rest[t])
        assert np.array_equal(x.view(np.uint64), xout[t].view(np.uint64)), t


@pytest.mark.parametrize("name", H27SUBSTEP)
def test_h27_substeps_bit_exact(orc, name):
    g = golden(name)
    a = golden_args(name)["args"]
    q = orc.QuadraticHex(g["nodes"], g["idx"], a[9])
    sch = q.schedule()
    assert np.array_equal(sch["hex_order"], g["order"])
    assert np.array_equal(sch["colour_hex_begin"], g["colour_hex_begin"])
    lm = (q.flags & 1).astype(np.uint8)
    X1, V1, w1, _ = q.substeps(q.X0, np.zeros_like(q.X0), q.w, g["order"], 1, q_params(orc, a, g, 0), lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = q.substeps(X1, V1, w1, g["order"], a[17] - 1, q_params(orc, a, g, 1), lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(q.volume(Xn)).view(np.uint32) == g["volume"].view(np.uint32)[0]


def test_h27_schedule_is_a_valid_colouring(orc):
    nodes, idx = orc.gen_hex_block(4, 3, 2, (0.1, 0.1, 0.1), 1, 0.3)
    q = orc.QuadraticHex(nodes, idx, 1000.0)
    s = q.schedule()
    cb, order = s["colour_hex_begin"], s["hex_order"]
    assert sorted(order.tolist()) == list(range(q.h27.shape[0]))
    for c in range(s["colours"]):
        verts = q.h27[order[cb[c]:cb[c + 1]]].reshape(-1)
        assert np.unique(verts).size == verts.size


H27RINGS = ["h27rings_c1_cpixar_nu045", "h27rings_c1_cmixed_nu045", "h27rings_c1_cmixed_incompressible",
            "h27rings_c1_cskin_nu049", "h27rings_wonky_cmixed_paper", "h27rings_c1_cskin_limit",
            "h27rings_c1_cmixed_amortized_pbd", "h27rings_wonky_cpixar_post"]


@pytest.mark.parametrize("name", H27RINGS)
def test_h27_rings_bit_exact(orc, name):
    """The continuous-pressure models on quadratic hexes: GeoQuadratic3d's
    rings of the mesh's own vertices over the H27s around them (SolveRing,
    XPBDFEM/Geo.cpp:147-225, 944-953, 971-1008; the full-energy branch on
    the 8- and 27-point rules, XPBDFEM/Fem.cpp:983-1036) in the fixture's
    ring order, which the centres-only ring schedule reproduces; PBD damping
    over the H27s in the fixture's H27 order."""
    g = golden(name)
    a = golden_args(name)["args"]
    q = orc.QuadraticHex(g["nodes"], g["idx"], a[9])
    assert np.array_equal(q.schedule()["hex_order"], g["order"])
    rs = q.ring_schedule()
    assert np.array_equal(rs["vert_order"], g["vorder"])
    assert np.array_equal(rs["colour_vert_begin"], g["colour_vert_begin"])
    lm = (q.flags & 1).astype(np.uint8)
    X1, V1, w1, _ = q.substeps_rings(q.X0, np.zeros_like(q.X0), q.w, g["order"], g["vorder"], 1,
                                     q_params(orc, a, g, 0), lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = q.substeps_rings(X1, V1, w1, g["order"], g["vorder"], a[17] - 1, q_params(orc, a, g, 1),
                                    lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(q.volume(Xn)).view(np.uint32) == g["volume"].view(np.uint32)[0]


QMIXED = ["qmixed_c1_nh_nu045_checker", "qmixed_c1_nh_incompressible_left", "qmixed_wonky_yeohfast_serial_nu049_checker",
          "qmixed_c1_pixar_nu045_amortized_pbd_checker", "qmixed_c1_mixed_nu045_limit_left",
          "qmixed_wonky_nh_paper_volume_checker", "qmixed_c1_yeohskin_nu045_post_pbd_left"]


@pytest.mark.parametrize("name", QMIXED)
def test_quadratic_mixed_mesh_bit_exact(orc, name):
    """GeoQuadratic3d on a mesh mixing tets and hexes (XPBDFEM/Geo.cpp:836-1008):
    Connectivity3d's edge and quad numbering over the interleaved stream, every
    vertex position, the T10 and H27 indices and records, the masses of all
    T10s then all H27s in one sum; then substeps that solve every T10, then
    every H27, and damp likewise, in the fixture's T10 and H27 colour orders,
    which the element schedule restatement reproduces."""
    g = golden(name)
    a = golden_args(name)["args"]
    dens, nsub = a[10], a[18]
    q = orc.QuadraticMixed(g["nodes"], g["idx"], dens)
    assert q.tets.shape[0] and q.hexes.shape[0]
    assert np.array_equal(q.X0.reshape(-1).view(np.uint64), g["x0"].view(np.uint64))
    assert np.array_equal(q.t10.reshape(-1), g["t10_idx"]) and np.array_equal(q.h27.reshape(-1), g["h27_idx"])
    assert np.array_equal(q.ept.reshape(-1).view(np.uint32), g["qep"].view(np.uint32))
    assert np.array_equal(q.eph.reshape(-1).view(np.uint32), g["h27ep"].view(np.uint32))
    assert np.array_equal(q.w.view(np.uint32), g["w"].view(np.uint32))
    assert np.array_equal(q.flags, g["vflags"])
    s = q.schedules()
    assert np.array_equal(s["t10_order"], g["torder"]) and np.array_equal(s["h27_order"], g["horder"])
    lm = (q.flags & 1).astype(np.uint8)
    X1, V1, w1, _ = q.substeps(q.X0, np.zeros_like(q.X0), q.w, g["torder"], g["horder"], 1,
                               mixed_params(orc, a, g, 0), lock_mask=lm)
    assert np.array_equal(X1.reshape(-1).view(np.uint64), g["x1"].view(np.uint64))
    assert np.array_equal(V1.reshape(-1).view(np.uint64), g["v1"].view(np.uint64))
    Xn, Vn, _, _ = q.substeps(X1, V1, w1, g["torder"], g["horder"], nsub - 1, mixed_params(orc, a, g, 1), lock_mask=lm)
    assert np.array_equal(Xn.reshape(-1).view(np.uint64), g["xn"].view(np.uint64))
    assert np.array_equal(Vn.reshape(-1).view(np.uint64), g["vn"].view(np.uint64))
    assert np.float32(q.volume(Xn)).view(np.uint32) == g["volume"].view(np.uint32)[0]


@pytest.mark.parametrize("pattern", [0, 1])
def test_quad_mesh_numbering_on_pure_streams(orc, pattern):
    """The stream-order numbering of a mixed stream reduces to the tet and
    hex numberings on streams of one kind."""
    nodes, idx = orc.gen_tet_block(4, 3, 2, (0.1, 0.1, 0.1), pattern, 0.3)
    tets, nv = orc.parse_tets(idx)
    e1, t1 = orc.tet_edges(tets, nv)
    e2, q2, t2, _ = orc.quad_mesh(idx, nv)
    assert np.array_equal(e1, e2) and np.array_equal(t1, t2) and q2.shape[0] == 0
    nodes, idx = orc.gen_hex_block(4, 3, 2, (0.1, 0.1, 0.1), pattern, 0.3)
    hexes, nv = orc.parse_hexes(idx)
    e1, q1, h1 = orc.h27_mesh(hexes, nv)
    e2, q2, _, h2 = orc.quad_mesh(idx, nv)
    assert np.array_equal(e1, e2) and np.array_equal(q1, q2) and np.array_equal(h1, h2)
