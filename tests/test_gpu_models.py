"""GPU energy models beyond MixedSel / YeohSkinFast, and volume passes.

SolveElement's dispatch on a linear tet (XPBDFEM/Fem.cpp:872-888; the
continuous-pressure models 8-10 are in test_gpu_rings.py): the Pixar
models (SolveElementPixar, XPBDFEM/Fem.cpp:361-433), Mixed, YeohSkin and
YeohSkinSel (the quadrature branch of SolveElementMixed, XPBDFEM/Fem.cpp:
459-522), the cube models (no constraint on a tet) and ids above 12
(MixedSel); and GeoLinear3d::Constrain's volume passes (SolveElementVolume,
XPBDFEM/Fem.cpp:840-867; XPBDFEM/Geo.cpp:780-783).

Against the reference's own substeps run in the GPU body's colour order (the
`model_*` and `volume_*` fixtures of tests/golden) and against the pinned
oracle on a larger jittered mesh. Tolerances as for the compressible
materials elsewhere: positions 1e-5 of max |x_ref|, velocities 1e-3 relative
(with volume passes, the first substep's velocities within 3x the FP32
reference's own distance from the FP64 run). Launch forms, call splits and
batching must agree bit for bit.
"""
import numpy as np
import pytest

import xfem
from conftest import golden, golden_args
from helpers import OracleRun, rel
from xfem import workloads as W

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
MODELS = ["model_c1_pixar_nu045_star", "model_c1_pixarsel_nu045_tet", "model_c1_mixed_nu045_star",
          "model_wonky_mixed_serial_nu045_star", "model_c1_yeohskin_nu049_tet",
          "model_wonky_yeohskinsel_serial_nu049_star", "model_c1_cube_pbd_star", "model_c1_pixar_amortized_pbd_star",
          "model_c1_pixar_paper_tet", "model_c1_mixed_limit_star", "model_wonky_yeohskin_serial_post_star",
          "volume_c1_nh_nu045_2_star", "volume_c1_yeoh_nu049_3_tet", "volume_wonky_pixar_1_post_pbd_star"]


def fixture_settings(name):
    """Settings of a `damped`-form fixture (refgen's argument order), with the
    reference's own derived values as a caller fills them."""
    a = golden_args(name)["args"]
    g = golden(name)
    W_, H, D, sx, sy, sz, wonk, dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock = a[1:18]
    damping, pbd, drag, rtype, spacing = a[18:23]
    vpasses = a[23] if len(a) > 23 else 0
    flags = ((energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) | (xfem.LOCK_LEFT if lock else 0) |
             (rtype << 20))
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, time_corrected_drag=float(g["derived"][2]),
                              volume_and_time_corrected_pbd_damping=float(g["derived"][0]),
                              amortized_volume_and_time_corrected_pbd_damping=float(g["derived"][1]), tick_id=0,
                              volume_passes=vpasses)
    # the fixture's oracle schedule mode (1 edge stars, 0 one tet per cluster)
    # as the product's cluster_mode (0 edge stars, 1 one tet per cluster)
    mode = 0 if golden_args(name)["schedule_mode"] == 1 else 1
    return g, s, dens, dt, nsub, mode


def body_of(name, **opts):
    g, s, dens, dt, nsub, mode = fixture_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s, cluster_mode=mode, **opts)
    return g, b, s, dt, nsub


def fp64_first_substep(name, s, dt):
    """The FP64 run of the same method and order (the oracle's double
    instantiation): velocities after the first substep."""
    import oracle
    g = golden(name)
    a = golden_args(name)["args"]
    tets, _ = oracle.parse_tets(g["idx"])
    ep, w, fl = oracle.init_rest(g["nodes"], tets, a[8], np.float64)
    X0 = g["nodes"].astype(np.float64)
    _, V1, _, _ = oracle.substeps(X0, np.zeros_like(X0), w, tets, ep, g["order"], 1,
                                  oracle.params_from_settings(s, dt), lock_mask=(fl & 1).astype(np.uint8),
                                  dtype=np.float64)
    return V1


@pytest.mark.parametrize("name", MODELS)
def test_model_reference_parity(name):
    g, b, s, dt, nsub = body_of(name)
    assert np.array_equal(b.schedule()["tet_order"], g["order"])
    b.substep(dt)
    assert rel(b.positions(), g["x1"].reshape(-1, 3)) <= 1e-5
    if s.volume_passes:
        # A volume pass moves the vertices by about (J - 1) / |grad J|, so the
        # rounding of J in FP32 reaches the first substep's velocity (about
        # g dt) at 1e-3 relative: the reference's own FP32 run is up to 2e-3
        # from the FP64 run there. The GPU must be as close to FP64 as that.
        v64 = fp64_first_substep(name, s, dt)
        e_ref = rel(g["v1"].reshape(-1, 3), v64)
        assert rel(b.velocities(), v64) <= 3 * e_ref, e_ref
    else:
        assert rel(b.velocities(), g["v1"].reshape(-1, 3)) <= 1e-3
    b.step_frames(1, nsub - 1, dt)
    assert rel(b.positions(), g["xn"].reshape(-1, 3)) <= 1e-5
    assert rel(b.velocities(), g["vn"].reshape(-1, 3)) <= 1e-3


@pytest.mark.parametrize("energy,simultaneous,comp,nu,vpasses,damping,rtype,pbd", [
    (xfem.ENERGY_PIXAR, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_PIXAR_SEL, 1, 1e-3, 0.40, 0, 0.01, 1, 0.0),
    (xfem.ENERGY_MIXED, 0, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_YEOH_SKIN, 1, 0.5, 0.49, 0, 0.01, 3, 0.03),
    (xfem.ENERGY_YEOH_SKIN_SEL, 0, 0.5, 0.45, 1, 0.0, 2, 0.0),
    (xfem.ENERGY_MIXED_SEL, 1, 1e-3, 0.45, 3, 0.01, 2, 0.05),
    (20, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
])
@pytest.mark.parametrize("mode", [0, 1])
def test_model_oracle_parity(energy, simultaneous, comp, nu, vpasses, damping, rtype, pbd, mode):
    """A larger jittered block, 20 substeps, against the oracle in the body's
    own order (and the multipliers after the first substep)."""
    nodes, idx = xfem.generate_tet_block(6, 3, 2, (0.05, 0.05, 0.05), 1, 0.0)
    rng = np.random.default_rng(9)
    nodes = (nodes + rng.normal(0, 0.003, nodes.shape)).astype(np.float32)
    flags = (energy << xfem.ENERGY_BIT) | (simultaneous << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | (rtype << 20)
    vc, avc = xfem.pbd_damping_coefficients(pbd, DT, 0.05)
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, volume_and_time_corrected_pbd_damping=vc,
                              amortized_volume_and_time_corrected_pbd_damping=avc, volume_passes=vpasses)
    b = xfem.Body(nodes, idx, 800.0, s, cluster_mode=mode)
    order = b.schedule()["tet_order"]
    o = OracleRun(nodes, idx, 800.0, s, order)
    o64 = OracleRun(nodes, idx, 800.0, xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_}), order,
                    dtype=np.float64)
    for n in (1, 19):
        b.step_frames(1, n, DT)
        for r in (o, o64):
            r.step(n, DT)
            r.s.tick_id += n
        assert rel(b.positions(), o.X) <= 1e-5, n
        if vpasses and n == 1:
            # first-substep velocities of volume passes: within 3x the FP32
            # oracle's own distance from FP64 (see test_model_reference_parity)
            assert rel(b.velocities(), o64.V) <= 3 * rel(o.V, o64.V), n
        else:
            assert rel(b.velocities(), o.V) <= 1e-3, n


@pytest.mark.parametrize("name", ["model_c1_pixar_amortized_pbd_star", "volume_wonky_pixar_1_post_pbd_star",
                                  "volume_c1_nh_nu045_2_star", "model_wonky_mixed_serial_nu045_star"])
def test_model_launch_forms_agree(name):
    """Persistent kernel and CUDA graph, one call or one call per substep."""
    runs = []
    for mode, split in ((1, False), (2, False), (1, True)):
        g, b, s, dt, nsub = body_of(name, sync_mode=mode)
        if split:
            for _ in range(nsub):
                b.substep(dt)
        else:
            b.step_frames(1, nsub, dt)
        runs.append((b.positions(), b.velocities()))
    for x, v in runs[1:]:
        assert np.array_equal(x, runs[0][0])
        assert np.array_equal(v, runs[0][1])


def test_batched_models_each_as_alone():
    """Bodies with different models and volume pass counts in one handle:
    each as when run alone (the handle runs the most volume sweeps; a body
    with fewer skips the rest)."""
    names = ["volume_c1_nh_nu045_2_star", "model_c1_pixar_nu045_star", "model_c1_yeohskin_nu049_tet"]
    meshes, settings, alone = [], [], []
    for name in names:
        g, s, dens, dt, nsub, mode = fixture_settings(name)
        b = xfem.Body(g["nodes"], g["idx"], dens, s)
        b.step_frames(1, 20, DT)
        alone.append((b.positions(), b.velocities()))
        meshes.append((g["nodes"], g["idx"], dens))
        settings.append(s)
    nodes2, idx2 = W.box(6, 2, 2, 0.05)
    s2 = xfem.default_settings(gravity=(0, -9.81, 0), compliance=W.nh_compliance(1e5, 0.45), poissons_ratio=0.45,
                               flags=W.NH_FLAGS)
    b2 = xfem.Body(nodes2, idx2, 1000.0, s2)
    b2.step_frames(1, 20, DT)
    alone.append((b2.positions(), b2.velocities()))
    meshes.append((nodes2, idx2, 1000.0))
    settings.append(s2)
    B = xfem.Body(meshes=meshes, settings=settings)
    B.step_frames(1, 20, DT)
    for k in range(len(meshes)):
        assert np.array_equal(B.positions(k), alone[k][0]), k
        assert np.array_equal(B.velocities(k), alone[k][1]), k


def test_switch_models_between_calls():
    """xfem_set_settings changes the model and the volume passes of a live
    handle: the run continues as a fresh body with those settings would."""
    g, s, dens, dt, nsub, mode = fixture_settings("model_c1_pixar_nu045_star")
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    b.step_frames(1, 5, dt)
    x5, v5 = b.positions(), b.velocities()
    s2 = fixture_settings("volume_c1_nh_nu045_2_star")[1]
    s2.tick_id = 5
    b.set_settings(s2)
    b.step_frames(1, 5, dt)
    c = xfem.Body(g["nodes"], g["idx"], dens, s2)
    c.step_frames(1, 1, dt)  # the lock zeroes the locked inverse masses in the first substep
    c.set_positions(x5)
    c.set_velocities(v5)
    c.set_settings(s2)
    c.step_frames(1, 5, dt)
    assert np.array_equal(b.positions(), c.positions())
    assert np.array_equal(b.velocities(), c.velocities())


def test_unsupported_models_and_limits():
    nodes, idx = W.box(3, 2, 2, 0.05)
    s = xfem.default_settings(flags=(xfem.ENERGY_PIXAR << xfem.ENERGY_BIT), poissons_ratio=0.5)
    with pytest.raises(xfem.XfemError) as ex:
        xfem.Body(nodes, idx, 1000.0, s)
    assert ex.value.code == xfem.EINVAL
    s = xfem.default_settings(volume_passes=xfem.MAX_VOLUME_PASSES + 1)
    with pytest.raises(xfem.XfemError) as ex:
        xfem.Body(nodes, idx, 1000.0, s)
    assert ex.value.code == xfem.EINVAL
    # the dataflow kernel runs only the plain solve
    s = xfem.default_settings(volume_passes=1)
    b = xfem.Body(nodes, idx, 1000.0, s, sync_mode=3)
    with pytest.raises(xfem.XfemError) as ex:
        b.step_frames(1, 2, DT)
    assert ex.value.code == xfem.EUNSUPPORTED
    # the adjoint differentiates the coupled Neo-Hookean model without volume passes
    for s in (xfem.default_settings(volume_passes=1),
              xfem.default_settings(flags=(xfem.ENERGY_PIXAR << xfem.ENERGY_BIT) | (1 << xfem.XPBD_SOLVE_BIT))):
        b = xfem.Body(nodes, idx, 1000.0, s)
        with pytest.raises(xfem.XfemError):
            b.adjoint_forward(4, DT, np.array([0], np.uint32))
