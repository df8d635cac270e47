"""GPU mixed mode: meshes mixing linear tets and linear hexes (xfem_mixed.cu)
through the C ABI.

GeoLinear3d on one tagged stream of tets and hexes (XPBDFEM/Geo.cpp:697-811):
the rest state sums the masses of all tets, then all hexes; every sweep
(the solve, each volume pass) solves every tet, then every hex; the damping
runs Rayleigh over the tets then the hexes, then PBD over the tets then the
hexes. Here each kind has a colouring of its own, and the reference's loops
run in those orders.

Against the reference's own substeps in the GPU body's tet and hex orders
(the `mixed_*` fixtures) and against the pinned oracle on a larger jittered
block. Tolerances as for the tets and hexes: compressible materials,
positions within 1e-5 of max |x_ref| and velocities 1e-3 relative; with an
incompressible material or volume passes, within 3x the FP32 reference's own
distance from the FP64 run of the same method after one substep, and within
3x the spread of FP32 runs (the reference and the FP32 oracle from 1-ulp
perturbed starts) after the whole run. Launch forms, call splits and
batching agree bit for bit.
"""
import numpy as np
import pytest

import oracle
import xfem
from conftest import golden, golden_args
from helpers import MixedOracleRun, rel

pytestmark = pytest.mark.gpu

DT = 1.0 / 1200.0
MIXED = ["mixed_c1_nh_nu045_checker", "mixed_c1_nh_incompressible_left", "mixed_wonky_yeohfast_serial_nu049_checker",
         "mixed_c1_pixar_nu045_amortized_pbd_checker", "mixed_c1_mixed_nu045_limit_left",
         "mixed_wonky_nh_paper_volume_checker", "mixed_c1_cube_neo_nu045_post_checker",
         "mixed_c1_yeohskin_nu045_post_pbd_left"]


def mixed_settings(name):
    """Settings of a `mixed` fixture (refgen's `mixed` argument order)."""
    a = golden_args(name)["args"]
    g = golden(name)
    dens, energy, simul, comp, nu, gx, gy, dt, nsub, lock, damping, pbd, _drag, rtype, _spacing, vp = a[10:26]
    d = g["derived"]
    flags = ((energy << xfem.ENERGY_BIT) | (simul << xfem.XPBD_SOLVE_BIT) | (xfem.LOCK_LEFT if lock else 0) |
             (rtype << 20))
    s = xfem.default_settings(gravity=(gx, gy, 0.0), compliance=comp, poissons_ratio=nu, flags=flags, damping=damping,
                              pbd_damping=pbd, time_corrected_drag=float(d[2]),
                              volume_and_time_corrected_pbd_damping=float(d[0]),
                              amortized_volume_and_time_corrected_pbd_damping=float(d[1]), volume_passes=vp)
    return g, s, dens, dt, nsub


def copy_settings(s):
    return xfem.default_settings(**{k: getattr(s, k) for k, _ in s._fields_})


def fp64_run(name, s, dt, nsub):
    g = golden(name)
    dens = golden_args(name)["args"][10]
    o = MixedOracleRun(g["nodes"], g["idx"], dens, copy_settings(s), g["torder"], g["horder"], dtype=np.float64)
    o.step(1, dt)
    X1, V1 = o.X.copy(), o.V.copy()
    o.s.tick_id = 1
    o.step(nsub - 1, dt)
    return X1, V1, o.X


def fp32_envelope(name, s, dt, nsub, X1_64, Xn_64, seeds=8):
    """How far FP32 runs of the method land from the FP64 run after one and
    after nsub substeps: the largest distances over the reference's own run
    and the FP32 oracle started from the rest positions perturbed by up to
    one float ulp (seeded). With an incompressible material the FP32
    rounding of J decides the pressure multiplier, and single runs spread
    over an order of magnitude."""
    g = golden(name)
    dens = golden_args(name)["args"][10]
    e1, en = rel(g["x1"].reshape(-1, 3), X1_64), rel(g["xn"].reshape(-1, 3), Xn_64)
    for seed in range(seeds):
        o = MixedOracleRun(g["nodes"], g["idx"], dens, copy_settings(s), g["torder"], g["horder"])
        o.X = o.X * (1.0 + np.random.default_rng(seed).uniform(-1.0, 1.0, o.X.shape) * 2.0 ** -24)
        o.step(1, dt)
        e1 = max(e1, rel(o.X, X1_64))
        o.s.tick_id = 1
        o.step(nsub - 1, dt)
        en = max(en, rel(o.X, Xn_64))
    return e1, en


@pytest.mark.parametrize("name", MIXED)
def test_mixed_reference_parity(name):
    g, s, dens, dt, nsub = mixed_settings(name)
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    nt, nh = g["torder"].size, g["horder"].size
    assert b.counts[0] == (g["nodes"].size // 3, nt) and b.hex_count() == nh
    # the rest state and both colourings are the reference's and the fixture's
    ep, w = b.rest_state()
    hep, w2 = b.hex_rest_state()
    assert np.array_equal(ep.reshape(-1).view(np.uint32), g["ep"].view(np.uint32))
    assert np.array_equal(hep.reshape(-1).view(np.uint32), g["hep"].view(np.uint32))
    assert np.array_equal(w.view(np.uint32), g["w"].view(np.uint32)) and np.array_equal(w2, w)
    ts, hs = b.mixed_tet_schedule(), b.hex_schedule()
    assert np.array_equal(ts["tet_order"], g["torder"]) and np.array_equal(ts["colour_tet_begin"], g["colour_tet_begin"])
    assert np.array_equal(hs["hex_order"], g["horder"]) and np.array_equal(hs["colour_hex_begin"], g["colour_hex_begin"])
    b.substep(dt)
    x1, v1 = b.positions(), b.velocities()
    b.step_frames(1, nsub - 1, dt)
    xn, vn = b.positions(), b.velocities()
    # CalculateVolume: the body's double sum against the oracle's at the
    # body's positions, and against the reference's float sum at its own
    tets, hexes, _ = oracle.parse_mixed(g["idx"])
    v64 = oracle.mixed_volume(xn.astype(np.float64), tets, hexes, g["hep"].reshape(-1, xfem.HEX_EP).astype(np.float64),
                              np.float64)
    assert abs(b.volume() - v64) <= 1e-6 * abs(v64)
    assert abs(b.volume() - float(g["volume"][0])) <= 1e-4 * abs(v64)
    if s.poissons_ratio >= 0.5 or s.volume_passes:
        # the tets' J - 1 at rest is FP32 rounding noise, and the pressure
        # multiplier follows it: the first substep already departs from the
        # reference's own rounding (as on tet meshes)
        X1_64, V1_64, Xn_64 = fp64_run(name, s, dt, nsub)
        e1, en = fp32_envelope(name, s, dt, nsub, X1_64, Xn_64)
        assert rel(x1, X1_64) <= 3 * e1 + 1e-7
        assert rel(xn, Xn_64) <= 3 * en + 1e-7
        return
    assert rel(x1, g["x1"].reshape(-1, 3)) <= 1e-5
    assert rel(v1, g["v1"].reshape(-1, 3)) <= 1e-3
    assert rel(xn, g["xn"].reshape(-1, 3)) <= 1e-5
    assert rel(vn, g["vn"].reshape(-1, 3)) <= 1e-3


def jittered_mixed_block():
    nodes, idx = oracle.mixed_block(6, 4, 3, (0.05, 0.05, 0.05), 1, 0.2, lambda x, y, z: (x * 7 + y * 3 + z) % 3 == 0)
    nodes = (nodes + np.random.default_rng(11).normal(0, 0.002, nodes.shape)).astype(np.float32)
    return nodes, idx


@pytest.mark.parametrize("energy,simultaneous,comp,nu,vpasses,damping,rtype,pbd", [
    (xfem.ENERGY_MIXED_SEL, 1, 1e-3, 0.45, 0, 0.0, 2, 0.0),
    (xfem.ENERGY_MIXED_SEL, 0, 1e-3, 0.40, 0, 0.01, 0, 0.0),
    (xfem.ENERGY_YEOH_SKIN_FAST, 1, 0.5, 0.45, 0, 0.01, 1, 0.0),
    (xfem.ENERGY_MIXED, 1, 1e-3, 0.45, 0, 0.01, 3, 0.03),
    (xfem.ENERGY_YEOH_SKIN, 0, 0.5, 0.45, 0, 0.01, 2, 0.0),
    (xfem.ENERGY_PIXAR_SEL, 1, 1e-3, 0.40, 0, 0.01, 2, 0.0),
    (xfem.ENERGY_CUBE_SKIN, 1, 0.5, 0.45, 1, 0.01, 3, 0.03),
])
def test_mixed_oracle_parity(energy, simultaneous, comp, nu, vpasses, damping, rtype, pbd):
    """A larger jittered mirrored block with a third of its cells split into
    tets, 20 substeps, against the oracle in the body's own orders."""
    nodes, idx = jittered_mixed_block()
    flags = (energy << xfem.ENERGY_BIT) | (simultaneous << xfem.XPBD_SOLVE_BIT) | xfem.LOCK_LEFT | (rtype << 20)
    vc, avc = xfem.pbd_damping_coefficients(pbd, DT, 0.05)
    s = xfem.default_settings(gravity=(0.3, -9.81, -2.0), compliance=comp, poissons_ratio=nu, flags=flags,
                              damping=damping, pbd_damping=pbd, volume_and_time_corrected_pbd_damping=vc,
                              amortized_volume_and_time_corrected_pbd_damping=avc, volume_passes=vpasses)
    b = xfem.Body(nodes, idx, 800.0, s)
    to, ho = b.mixed_tet_schedule()["tet_order"], b.hex_schedule()["hex_order"]
    o = MixedOracleRun(nodes, idx, 800.0, s, to, ho)
    o64 = MixedOracleRun(nodes, idx, 800.0, copy_settings(s), to, ho, dtype=np.float64)
    for n in (1, 19):
        b.step_frames(1, n, DT)
        for r in (o, o64):
            r.step(n, DT)
            r.s.tick_id += n
        assert rel(b.positions(), o.X) <= 1e-5, n
        if vpasses and n == 1:
            assert rel(b.velocities(), o64.V) <= 3 * rel(o.V, o64.V), n
        else:
            assert rel(b.velocities(), o.V) <= 1e-3, n
    # volume: the tets on the device plus the hexes on the host, in double
    v64 = oracle.mixed_volume(b.positions().astype(np.float64), o.tets, o.hexes, o.hep.astype(np.float64), np.float64)
    assert abs(b.volume() - v64) <= 1e-6 * abs(v64)


def test_mixed_ground_contacts_bit_exact():
    """A mixed block falling onto the ground plane with friction 0.4: the
    contact set of the landing substep and of the four after it is the
    oracle's, vertex for vertex, positions within 1e-5."""
    nodes, idx = jittered_mixed_block()
    nodes = nodes.reshape(-1, 3).copy()
    nodes[:, 1] += 0.002 - nodes[:, 1].min()
    s = xfem.default_settings(gravity=(0.0, -9.81, 0.0), compliance=1e-3, poissons_ratio=0.45,
                              flags=(xfem.ENERGY_MIXED_SEL << xfem.ENERGY_BIT) | (1 << xfem.XPBD_SOLVE_BIT),
                              ground=1, friction=0.4, ground_normal=(0.0, 1.0, 0.0), ground_offset=0.0)
    b = xfem.Body(nodes.reshape(-1), idx, 800.0, s)
    to, ho = b.mixed_tet_schedule()["tet_order"], b.hex_schedule()["hex_order"]
    o = MixedOracleRun(nodes.reshape(-1), idx, 800.0, s, to, ho)
    v0 = np.tile(np.array([0.1, -1.0, 0.0], np.float32), (nodes.shape[0], 1))
    b.set_velocities(v0)
    o.V[:] = v0
    for _ in range(120):
        b.substep(DT)
        o.step(1, DT)
        if o.contact.any() or b.contacts().any():
            break
    else:
        raise AssertionError("the body never reached the ground")
    for k in range(5):
        assert np.array_equal(b.contacts().astype(bool), o.contact.astype(bool)), k
        assert rel(b.positions(), o.X) <= 1e-5, k
        b.substep(DT)
        o.step(1, DT)


def test_mixed_launch_forms_agree():
    """One call, one call per substep, and the allocation-free launch."""
    g, s, dens, dt, nsub = mixed_settings("mixed_c1_pixar_nu045_amortized_pbd_checker")
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


def test_mixed_batch_each_as_alone():
    """Mixed bodies with different models, damping and volume passes in one
    handle: each as when run alone."""
    names = ["mixed_wonky_nh_paper_volume_checker", "mixed_c1_pixar_nu045_amortized_pbd_checker",
             "mixed_c1_yeohskin_nu045_post_pbd_left", "mixed_c1_nh_nu045_checker"]
    meshes, settings, alone = [], [], []
    for name in names:
        g, s, dens, dt, nsub = mixed_settings(name)
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


def test_mixed_errors():
    g, s, dens, dt, nsub = mixed_settings("mixed_c1_nh_nu045_checker")
    # the continuous-pressure models are refused on a mixed mesh, linear or
    # quadratic (the reference indexes a ring's hexes two ways there)
    for flags in (9 << xfem.ENERGY_BIT, (9 << xfem.ENERGY_BIT) | xfem.ELEMENT_T10):
        with pytest.raises(xfem.XfemError) as ex:
            xfem.Body(g["nodes"], g["idx"], dens, xfem.default_settings(flags=flags))
        assert ex.value.code == xfem.EUNSUPPORTED
    # mixed bodies do not share a handle with tet or hex bodies
    tn, ti = xfem.generate_tet_block(3, 2, 2, (0.05, 0.05, 0.05))
    with pytest.raises(xfem.XfemError) as ex:
        xfem.Body(meshes=[(g["nodes"], g["idx"], dens), (tn, ti, 1000.0)])
    assert ex.value.code == xfem.EUNSUPPORTED
    b = xfem.Body(g["nodes"], g["idx"], dens, s)
    for call in (lambda: b.set_tet_mu(np.ones(b.counts[0][1], np.float32)), lambda: b.schedule(),
                 lambda: b.adjoint_forward(2, DT, np.array([0], np.uint32))):
        with pytest.raises(xfem.XfemError) as ex:
            call()
        assert ex.value.code == xfem.EUNSUPPORTED
    b.step_frames(1, 4, DT)
    assert np.isfinite(b.positions()).all()
