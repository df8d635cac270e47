"""GPU quadratic-hex mode: H27s (xfem_h27.cu, one warp per element) through
the C ABI.

A hex mesh with element type H27 in flags bits 0-3 runs as GeoQuadratic3d
(XPBDFEM/Geo.cpp:836-1053): nodes on every edge and face and at every hex
centre, SolveElement on ElementParamsQuadraticHex with Nodes = 27 on the
2x2x2 and 3x3x3 rules (XPBDFEM/Fem.cpp:871-897), the Pixar models, Mixed,
MixedSel and the Yeoh models, coupled or serial, in-solve and post-step
damping, PBD damping and volume passes; the cube models leave an H27 alone.

Against the reference's own substeps run in the GPU body's H27 colour order
(the `h27ordered_*`, `h27damped_*` and `h27volume_*` fixtures) and against
the pinned oracle on a larger jittered block. Compressible materials:
positions within 1e-5 of max |x_ref|. The velocities of the stiff fixture
blocks are decided by FP32 rounding already after one substep: on
`h27ordered_c1_nh_nu045` the reference's own FP32 run is 1.5e-2 from the
FP64 run, and FP32 runs from 1-ulp perturbed starts land 1.3e-3 to 4.8e-3
from the reference (2.1e-3 from float-rounded node positions alone), where
positions agree to 3e-7. Velocities are therefore held within 3x the spread
of FP32 runs (the reference's own run and oracle runs from perturbed starts)
about the FP64 run of the same method and order, after one substep and
after all of them; so are positions with an incompressible material or
volume passes. On the softer jittered block the GPU holds the FP32 oracle's
velocities within 1e-3. The warp's sums run in another order than the
reference's loops, so the GPU is not bit-identical to the oracle. Launch
forms, call splits and batching agree bit for bit.
"""
import numpy as np
import pytest

import oracle
import xfem
from conftest import golden, golden_args
from helpers import H27OracleRun, envelope, rel

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
HFIX = ["h27ordered_c1_nh_nu045", "h27ordered_c1_nh_incompressible", "h27ordered_wonky_yeohfast_serial_nu049",
        "h27ordered_c1_mixed_nu045", "h27damped_c1_nh_nu045_amortized_pbd", "h27damped_c1_pixar_nu045_limit",
        "h27volume_wonky_nh_serial_1_post"]


def copy_settings(s):
    return xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_})


def h27_settings(name):
    """Settings of a `Qordered` / `Qdamped` fixture (refgen's argument order),
    with the element type H27."""
    a = golden_args(name)["args"]
    g = golden(name)
    dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[9:19]
    kw = dict(rtype=2, damping=0.0, pbd=0.0, drag=0.0, vc=0.0, avc=0.0, vp=0)
    if a[0] == "Qdamped":
        d = g["derived"]
        kw = dict(damping=a[19], pbd=a[20], rtype=a[22], drag=float(d[2]), vc=float(d[0]), avc=float(d[1]),
                  vp=a[24] if len(a) > 24 else 0)
    flags = (xfem.ELEMENT_H27 | (energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) |
             (xfem.LOCK_LEFT if lock else 0) | (kw["rtype"] << 20))
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=kw["damping"], pbd_damping=kw["pbd"], time_corrected_drag=kw["drag"],
                              volume_and_time_corrected_pbd_damping=kw["vc"],
                              amortized_volume_and_time_corrected_pbd_damping=kw["avc"], volume_passes=kw["vp"])
    return g, s, dens, dt, nsub


@pytest.mark.parametrize("name", HFIX)
def test_h27_reference_parity(name):
    g, s, dens, dt, nsub = h27_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    assert b.h27_count()[0] == g["order"].size and b.counts[0][0] == g["x1"].size // 3
    sch = b.h27_schedule()
    assert np.array_equal(sch["h27_order"], g["order"])
    assert np.array_equal(sch["colour_h27_begin"], g["colour_hex_begin"])
    b.substep(dt)
    x1, v1 = b.positions(), b.velocities()
    b.step_frames(1, nsub - 1, dt)
    xn, vn = b.positions(), b.velocities()
    ref, env = envelope(lambda dt_: H27OracleRun(g["nodes"], g["idx"], dens, copy_settings(s), g["order"],
                                                 dtype=dt_), (1, nsub), dt)
    (X1_64, V1_64), (Xn_64, Vn_64) = ref
    # velocities: within 3x the FP32 spread about the FP64 run (the
    # reference's own run included); see the module docstring
    ev1 = max(env[0][1], rel(g["v1"].reshape(-1, 3), V1_64))
    evn = max(env[1][1], rel(g["vn"].reshape(-1, 3), Vn_64))
    assert rel(v1, V1_64) <= 3 * ev1 + 1e-7
    assert rel(vn, Vn_64) <= 3 * evn + 1e-7
    if s.poissons_ratio >= 0.5 or s.volume_passes:
        ex1 = max(env[0][0], rel(g["x1"].reshape(-1, 3), X1_64))
        exn = max(env[1][0], rel(g["xn"].reshape(-1, 3), Xn_64))
        assert rel(x1, X1_64) <= 3 * ex1 + 1e-7
        assert rel(xn, Xn_64) <= 3 * exn + 1e-7
        return
    assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
    assert rel(xn, g["xn"].reshape(-1, 3)) <= 1e-5


@pytest.mark.parametrize("energy,simultaneous,comp,nu,vpasses,damping,rtype,pbd", [
    (xfem.ENERGY_MIXED_SEL, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_MIXED_SEL, 0, 1e-3, 0.40, 0, 0.01, 0, 0.0),
    (xfem.ENERGY_YEOH_SKIN_FAST, 1, 0.5, 0.45, 0, 0.01, 1, 0.0),
    (xfem.ENERGY_MIXED, 1, 1e-3, 0.45, 0, 0.01, 3, 0.03),
    (xfem.ENERGY_YEOH_SKIN, 0, 0.5, 0.45, 0, 0.01, 2, 0.0),
    (xfem.ENERGY_YEOH_SKIN_SEL, 1, 0.5, 0.49, 0, 0.0, 2, 0.05),
    (xfem.ENERGY_PIXAR, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_PIXAR_REDUCED, 1, 1e-3, 0.45, 0, 0.01, 2, 0.0),
    (xfem.ENERGY_PIXAR_SEL, 1, 1e-3, 0.40, 0, 0.01, 2, 0.0),
    (20, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_CUBE_NEO, 1, 1e-3, 0.45, 0, 0.01, 3, 0.03),
    (xfem.ENERGY_MIXED_SEL, 1, 1e-3, 0.45, 1, 0.01, 2, 0.0),
])
def test_h27_oracle_parity(energy, simultaneous, comp, nu, vpasses, damping, rtype, pbd):
    """A jittered mirrored 4x3x3 block, 20 substeps, against the oracle in
    the body's own H27 order."""
    nodes, idx = xfem.generate_hex_block(4, 3, 3, (0.05, 0.05, 0.05), 1, 0.2)
    rng = np.random.default_rng(5)
    nodes = (nodes + rng.normal(0, 0.002, nodes.shape)).astype(np.float32)
    flags = (xfem.ELEMENT_H27 | (energy << xfem.ENERGY_BIT) | (simultaneous << xfem.XPBD_SOLVE_BIT) |
             xfem.LOCK_LEFT | (rtype << 20))
    vc, avc = xfem.pbd_damping_coefficients(pbd, DT, 0.05)
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, volume_and_time_corrected_pbd_damping=vc,
                              amortized_volume_and_time_corrected_pbd_damping=avc, volume_passes=vpasses)
    b = xfem.Body(nodes, idx, 800.0, s)
    order = b.h27_schedule()["h27_order"]
    if vpasses:
        ref, env = envelope(lambda dt_: H27OracleRun(nodes, idx, 800.0, copy_settings(s), order, dtype=dt_),
                            (1, 20), DT)
        for k, n in enumerate((1, 19)):
            b.step_frames(1, n, DT)
            assert rel(b.positions(), ref[k][0]) <= 3 * env[k][0] + 1e-7, n
            assert rel(b.velocities(), ref[k][1]) <= 3 * env[k][1] + 1e-7, n
        return
    o = H27OracleRun(nodes, idx, 800.0, s, order)
    for n in (1, 19):
        b.step_frames(1, n, DT)
        o.step(n, DT)
        o.s.tick_id += n
        assert rel(b.positions(), o.X) <= 1e-5, n
        assert rel(b.velocities(), o.V) <= 1e-3, n


def test_h27_rest_state_and_volume():
    nodes, idx = xfem.generate_hex_block(3, 3, 2, (0.04, 0.05, 0.06), 1, 0.3)
    s = xfem.default_settings(flags=xfem.default_settings().flags | xfem.ELEMENT_H27)
    b = xfem.Body(nodes, idx, 900.0, s)
    ep, w, h27 = b.h27_rest_state()
    x, e2, w2, _ = xfem.compute_h27_rest_state(nodes, idx, 900.0)
    assert np.array_equal(ep.view(np.uint32), e2.view(np.uint32))
    assert np.array_equal(w.view(np.uint32), w2.view(np.uint32))
    assert np.array_equal(b.inverse_masses().view(np.uint32), w2.view(np.uint32))
    assert np.array_equal(h27, xfem.compute_h27_mesh(idx)[2])
    # the body's rest positions: the mesh's own, then the edge, face and centre nodes
    assert np.array_equal(b.positions(), x.astype(np.float32))
    q = oracle.QuadraticHex(nodes, idx, 900.0, np.float64)
    assert abs(b.volume() - q.volume(b.positions().astype(np.float64))) <= 1e-6 * b.volume()
    s.flags &= ~xfem.LOCK_LEFT
    s.gravity[1] = -9.81
    b.set_settings(s)
    b.step_frames(2, 10, DT)
    assert abs(b.volume() - q.volume(b.positions().astype(np.float64))) <= 1e-6 * b.volume()


def test_h27_launch_forms_agree():
    """One call, one call per substep, and the allocation-free launch."""
    g, s, dens, dt, nsub = h27_settings("h27damped_c1_nh_nu045_amortized_pbd")
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


def test_h27_batch_each_as_alone():
    """H27 bodies with different models, damping and volume passes in one
    handle: each as when run alone."""
    names = ["h27volume_wonky_nh_serial_1_post", "h27damped_c1_pixar_nu045_limit", "h27ordered_c1_mixed_nu045",
             "h27ordered_wonky_yeohfast_serial_nu049"]
    meshes, settings, alone = [], [], []
    for name in names:
        g, s, dens, dt, nsub = h27_settings(name)
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


def test_h27_errors():
    nodes, idx = xfem.generate_hex_block(3, 2, 2, (0.05, 0.05, 0.05))
    h27 = xfem.default_settings().flags | xfem.ELEMENT_H27
    # a ring body (energy 8-10) and an element body cannot share a handle
    with pytest.raises(xfem.XfemError) as ex:
        xfem.Body(meshes=[(nodes, idx, 1000.0), (nodes, idx, 1000.0)],
                  settings=[xfem.default_settings(flags=xfem.ELEMENT_H27 | (9 << xfem.ENERGY_BIT)),
                            xfem.default_settings(flags=h27)])
    assert ex.value.code == xfem.EUNSUPPORTED
    # linear and quadratic hexes cannot share a handle
    with pytest.raises(xfem.XfemError) as ex:
        xfem.Body(meshes=[(nodes, idx, 1000.0), (nodes, idx, 1000.0)],
                  settings=[xfem.default_settings(flags=h27), xfem.default_settings()])
    assert ex.value.code == xfem.EUNSUPPORTED
    b = xfem.Body(nodes, idx, 1000.0, xfem.default_settings(flags=h27))
    with pytest.raises(xfem.XfemError) as ex:
        b.set_settings(xfem.default_settings())
    assert ex.value.code == xfem.EUNSUPPORTED
    for call in (lambda: b.set_tet_mu(np.ones(12, np.float32)), lambda: b.rest_state(), lambda: b.schedule(),
                 lambda: b.hex_rest_state(), lambda: b.t10_rest_state(),
                 lambda: b.adjoint_forward(2, DT, np.array([0], np.uint32))):
        with pytest.raises(xfem.XfemError) as ex:
            call()
        assert ex.value.code == xfem.EUNSUPPORTED
    b.step_frames(1, 4, DT)
    assert np.isfinite(b.positions()).all()
