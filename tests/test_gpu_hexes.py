"""GPU hex mode: linear hexahedra (xfem_hexes.cu) through the C ABI.

GeoLinear3d's hex loops (XPBDFEM/Geo.cpp:777-811) with SolveElement on
ElementParamsLinearHex (XPBDFEM/Fem.cpp:871-896): the Pixar models, Mixed,
MixedSel, the Yeoh models, the cube models and ids above 12, coupled or
serial, in-solve and post-step damping, PBD damping and volume passes.

Against the reference's own substeps run in the GPU body's hex colour order
(the `hordered_*`, `hdamped_*` and `hvolume_*` fixtures) and against the
pinned oracle on larger jittered blocks. Tolerances as for the tets:
compressible materials, positions within 1e-5 of max |x_ref| and velocities
1e-3 relative; with an incompressible material or volume passes, within 3x
the FP32 reference's own distance from the FP64 run of the same method after
one substep, and within 3x the spread of FP32 runs (the reference and the
FP32 oracle from 1-ulp perturbed starts) after the whole run.
Launch forms, call splits and batching agree bit for bit.
"""
import numpy as np
import pytest

import oracle
import xfem
from conftest import golden, golden_args
from helpers import HexOracleRun, rel

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
HFIX = ["hordered_c1_nh_nu045", "hordered_c1_nh_incompressible", "hordered_c1_yeohfast_nu049",
        "hordered_wonky_nh_serial_nu045", "hordered_c1_mixed_nu045", "hordered_wonky_yeohskinsel_serial_nu049",
        "hordered_c1_pixar_nu045", "hdamped_c1_nh_nu045_post_pbd", "hdamped_c1_nh_nu045_amortized_pbd",
        "hdamped_c1_nh_nu045_paper", "hdamped_c1_nh_nu045_limit", "hdamped_wonky_yeohskin_serial_post",
        "hvolume_c1_nh_nu045_2", "hvolume_wonky_pixar_1_post_pbd",
        # the cube models (SolveElementCube, XPBDFEM/Fem.cpp:566-838)
        "hordered_c1_cube_neo_fast", "hordered_wonky_cube_neo_nu045", "hordered_c1_cube_skin_nu049",
        "hdamped_c1_cube_neo_nu045_paper", "hdamped_c1_cube_skin_nu045_limit",
        "hdamped_c1_cube_neo_incompressible_amortized_pbd"]


def hex_settings(name):
    """Settings of an `hordered` / `hdamped` / `hrings` fixture (refgen's argument order)."""
    a = golden_args(name)["args"]
    g = golden(name)
    dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[9:19]
    kw = dict(rtype=2, damping=0.0, pbd=0.0, drag=0.0, vc=0.0, avc=0.0, vp=0)
    if a[0] in ("hdamped", "hrings"):
        d = g["derived"]
        kw = dict(damping=a[19], pbd=a[20], rtype=a[22], drag=float(d[2]), vc=float(d[0]), avc=float(d[1]),
                  vp=a[24] if len(a) > 24 else 0)
    flags = ((energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) | (xfem.LOCK_LEFT if lock else 0) |
             (kw["rtype"] << 20))
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=kw["damping"], pbd_damping=kw["pbd"], time_corrected_drag=kw["drag"],
                              volume_and_time_corrected_pbd_damping=kw["vc"],
                              amortized_volume_and_time_corrected_pbd_damping=kw["avc"], volume_passes=kw["vp"])
    return g, s, dens, dt, nsub


def fp64_run(name, s, dt, nsub):
    g = golden(name)
    dens = golden_args(name)["args"][9]
    o = HexOracleRun(g["nodes"], g["idx"], dens, s, g["order"], dtype=np.float64)
    o.step(1, dt)
    V1 = o.V.copy()
    o.s = xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_})
    o.s.tick_id = 1
    o.step(nsub - 1, dt)
    return V1, o.X


def fp32_envelope(name, s, dt, nsub, Xn_64, seeds=8):
    """How far FP32 runs of the method land from the FP64 run after nsub
    substeps: the largest distance over the reference's own run and the FP32
    oracle started from the rest positions perturbed by up to one float ulp
    (seeded). With an incompressible material the FP32 rounding of J grows
    chaotically, and single runs spread over an order of magnitude."""
    g = golden(name)
    dens = golden_args(name)["args"][9]
    e = rel(g["xn"].reshape(-1, 3), Xn_64)
    for seed in range(seeds):
        o = HexOracleRun(g["nodes"], g["idx"], dens, xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_}),
                         g["order"])
        o.X = o.X * (1.0 + np.random.default_rng(seed).uniform(-1.0, 1.0, o.X.shape) * 2.0 ** -24)
        o.step(1, dt)
        o.s.tick_id = 1
        o.step(nsub - 1, dt)
        e = max(e, rel(o.X, Xn_64))
    return e


@pytest.mark.parametrize("name", HFIX)
def test_hex_reference_parity(name):
    g, s, dens, dt, nsub = hex_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    assert b.hex_count() == g["order"].size
    assert np.array_equal(b.hex_schedule()["hex_order"], g["order"])
    b.substep(dt)
    x1, v1 = b.positions(), b.velocities()
    b.step_frames(1, nsub - 1, dt)
    xn, vn = b.positions(), b.velocities()
    if s.poissons_ratio >= 0.5 or s.volume_passes:
        # the FP32 rounding of J decides these (see test_gpu_parity and
        # test_gpu_models): the GPU within 3x the FP32 reference's own
        # distance from the FP64 run of the same method and order after one
        # substep, and within 3x the FP32 envelope after all of them
        V1_64, Xn_64 = fp64_run(name, s, dt, nsub)
        assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
        assert rel(v1, V1_64) <= 3 * rel(g["v1"].reshape(-1, 3), V1_64) + 1e-7
        assert rel(xn, Xn_64) <= 3 * fp32_envelope(name, s, dt, nsub, Xn_64) + 1e-7
        return
    assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
    assert rel(v1, g["v1"].reshape(-1, 3)) <= 1e-3
    assert rel(xn, g["xn"].reshape(-1, 3)) <= 1e-5
    assert rel(vn, g["vn"].reshape(-1, 3)) <= 1e-3


@pytest.mark.parametrize("energy,simultaneous,comp,nu,vpasses,damping,rtype,pbd", [
    (xfem.ENERGY_MIXED_SEL, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_MIXED_SEL, 0, 1e-3, 0.40, 0, 0.01, 0, 0.0),
    (xfem.ENERGY_YEOH_SKIN_FAST, 1, 0.5, 0.45, 0, 0.01, 1, 0.0),
    (xfem.ENERGY_MIXED, 1, 1e-3, 0.45, 0, 0.01, 3, 0.03),
    (xfem.ENERGY_YEOH_SKIN, 0, 0.5, 0.45, 0, 0.01, 2, 0.0),
    (xfem.ENERGY_YEOH_SKIN_SEL, 1, 0.5, 0.49, 0, 0.0, 2, 0.05),
    (xfem.ENERGY_PIXAR_REDUCED, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_PIXAR_SEL, 1, 1e-3, 0.40, 0, 0.01, 2, 0.0),
    (20, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_CUBE_NEO, 1, 1e-3, 0.45, 0, 0.01, 1, 0.0),
    (xfem.ENERGY_CUBE_SKIN, 1, 0.5, 0.45, 1, 0.01, 3, 0.03),
])
def test_hex_oracle_parity(energy, simultaneous, comp, nu, vpasses, damping, rtype, pbd):
    """A larger jittered mirrored block, 20 substeps, against the oracle in
    the body's own hex order."""
    nodes, idx = xfem.generate_hex_block(6, 4, 3, (0.05, 0.05, 0.05), 1, 0.2)
    rng = np.random.default_rng(5)
    nodes = (nodes + rng.normal(0, 0.002, nodes.shape)).astype(np.float32)
    flags = (energy << xfem.ENERGY_BIT) | (simultaneous << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | (rtype << 20)
    vc, avc = xfem.pbd_damping_coefficients(pbd, DT, 0.05)
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, volume_and_time_corrected_pbd_damping=vc,
                              amortized_volume_and_time_corrected_pbd_damping=avc, volume_passes=vpasses)
    b = xfem.Body(nodes, idx, 800.0, s)
    order = b.hex_schedule()["hex_order"]
    o = HexOracleRun(nodes, idx, 800.0, s, order)
    o64 = HexOracleRun(nodes, idx, 800.0, xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_}), order,
                       dtype=np.float64)
    for n in (1, 19):
        b.step_frames(1, n, DT)
        for r in (o, o64):
            r.step(n, DT)
            r.s.tick_id += n
        assert rel(b.positions(), o.X) <= 1e-5, n
        if vpasses and n == 1:
            # first-substep velocities of volume passes: within 3x the FP32
            # oracle's own distance from FP64 (as for the tets)
            assert rel(b.velocities(), o64.V) <= 3 * rel(o.V, o64.V), n
        else:
            assert rel(b.velocities(), o.V) <= 1e-3, n


def test_hex_rest_state_and_volume():
    nodes, idx = xfem.generate_hex_block(5, 3, 2, (0.04, 0.05, 0.06), 1, 0.3)
    b = xfem.Body(nodes, idx, 900.0)
    ep, w = b.hex_rest_state()
    e2, w2, _ = xfem.compute_hex_rest_state(nodes, idx, 900.0)
    assert np.array_equal(ep.view(np.uint32), e2.view(np.uint32))
    assert np.array_equal(w.view(np.uint32), w2.view(np.uint32))
    assert np.array_equal(b.inverse_masses().view(np.uint32), w2.view(np.uint32))
    hexes, _ = oracle.parse_hexes(idx)
    X = nodes.astype(np.float64)
    assert abs(b.volume() - oracle.hex_volume(X, hexes, e2.astype(np.float64), np.float64)) <= 1e-6 * b.volume()
    s = xfem.default_settings(gravity=(0.0, -9.81, 0.0), flags=xfem.default_settings().flags & ~xfem.LOCK_LEFT)
    b.set_settings(s)
    b.step_frames(2, 10, DT)
    ep64 = e2.astype(np.float64)
    assert abs(b.volume() - oracle.hex_volume(b.positions().astype(np.float64), hexes, ep64, np.float64)) <= \
        1e-6 * b.volume()


def test_hex_launch_forms_agree():
    """One call, one call per substep, and the allocation-free launch."""
    g, s, dens, dt, nsub = hex_settings("hdamped_c1_nh_nu045_amortized_pbd")
    runs = []
    for form in ("frames", "split", "noalloc"):
        b = xfem.Body(g["nodes"], g["idx"], dens, s)
        if form == "frames":
            b.step_frames(1, nsub, dt)
        elif form == "split":
            for _ in range(nsub):
                b.substep(dt)
        else:
            b.step_frames_noalloc(1, nsub, dt)
        runs.append((b.positions(), b.velocities()))
    for x, v in runs[1:]:
        assert np.array_equal(x, runs[0][0])
        assert np.array_equal(v, runs[0][1])


def test_hex_batch_each_as_alone():
    """Hex bodies with different models, damping and volume passes in one
    handle: each as when run alone."""
    names = ["hvolume_c1_nh_nu045_2", "hordered_c1_pixar_nu045", "hdamped_wonky_yeohskin_serial_post",
             "hordered_c1_mixed_nu045"]
    meshes, settings, alone = [], [], []
    for name in names:
        g, s, dens, dt, nsub = hex_settings(name)
        b = xfem.Body(g["nodes"], g["idx"], dens, s)
        b.step_frames(1, 12, DT)
        alone.append((b.positions(), b.velocities()))
        meshes.append((g["nodes"], g["idx"], dens))
        settings.append(s)
    B = xfem.Body(meshes=meshes, settings=settings)
    B.step_frames(1, 12, DT)
    for k in range(len(meshes)):
        assert np.array_equal(B.positions(k), alone[k][0]), k
        assert np.array_equal(B.velocities(k), alone[k][1]), k


def test_hex_errors():
    nodes, idx = xfem.generate_hex_block(3, 2, 2, (0.05, 0.05, 0.05))
    tn, ti = xfem.generate_tet_block(3, 2, 2, (0.05, 0.05, 0.05))
    with pytest.raises(xfem.XfemError) as ex:
        xfem.Body(meshes=[(nodes, idx, 1000.0), (tn, ti, 1000.0)])
    assert ex.value.code == xfem.EUNSUPPORTED
    b = xfem.Body(nodes, idx, 1000.0)
    # an element body switching to a continuous-pressure model needs a new handle
    with pytest.raises(xfem.XfemError) as ex:
        b.set_settings(xfem.default_settings(flags=9 << xfem.ENERGY_BIT))
    assert ex.value.code == xfem.EUNSUPPORTED
    for call in (lambda: b.set_tet_mu(np.ones(12, np.float32)), lambda: b.rest_state(), lambda: b.schedule(),
                 lambda: b.adjoint_forward(2, DT, np.array([0], np.uint32))):
        with pytest.raises(xfem.XfemError) as ex:
            call()
        assert ex.value.code == xfem.EUNSUPPORTED
    # the handle still steps after the refusals
    b.step_frames(1, 4, DT)
    assert np.isfinite(b.positions()).all()
