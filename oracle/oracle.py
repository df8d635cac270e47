"""ctypes wrapper of the oracle restatement (oracle/xfem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline / reference arm. The product (libxfem.so and the
xfem package) never imports this module.

The float routines reproduce the reference (jak-xyz/xpbd-fem) bit for bit
(pinned by tests/golden/, generated from the reference's own code); the
double routines are the FP64 run of the same method.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

# Energy model ids, XPBDFEM/Settings.h:41-53
ENERGY_PIXAR = 0
ENERGY_PIXAR_REDUCED = 1
ENERGY_PIXAR_SEL = 2
ENERGY_MIXED = 3
ENERGY_MIXED_SEL = 4
ENERGY_YEOH_SKIN = 5
ENERGY_YEOH_SKIN_SEL = 6
ENERGY_YEOH_SKIN_FAST = 7
ENERGY_CONTINUOUS_PIXAR = 8
ENERGY_CONTINUOUS_MIXED = 9
ENERGY_CONTINUOUS_SKIN = 10
ENERGY_CUBE_NEO = 11
ENERGY_CUBE_SKIN = 12
REF_YEOH = (0.1095, 14.95, 4.595)  # XPBDFEM/Fem.cpp:526


class Params(C.Structure):
    """Mirror of orc_params (oracle/xfem_oracle.h)."""
    _fields_ = [
        ("gravity", C.c_float * 3), ("dt", C.c_float), ("time_corrected_drag", C.c_float),
        ("compliance", C.c_float), ("poisson", C.c_float), ("energy", C.c_uint32),
        ("simultaneous", C.c_uint32), ("yeoh", C.c_float * 3), ("lock_active", C.c_uint32),
        ("ground", C.c_uint32), ("ground_n", C.c_float * 3), ("ground_d", C.c_float),
        ("friction", C.c_float), ("damping", C.c_float), ("rayleigh_type", C.c_uint32),
        ("pbd_damping", C.c_float), ("pbd_coeff", C.c_float), ("pbd_coeff_amortized", C.c_float),
        ("tick", C.c_uint32), ("volume_passes", C.c_uint32), ("lock_right", C.c_uint32),
        ("right_target", C.c_void_p),
    ]


def make_params(dt, compliance, poisson, energy=ENERGY_MIXED_SEL, simultaneous=True,
                gravity=(0.0, 0.0, 0.0), drag=0.0, yeoh=REF_YEOH, lock=False,
                ground=False, ground_n=(0.0, 0.0, 1.0), ground_d=0.0, friction=0.0, damping=0.0, rayleigh_type=2,
                pbd_damping=0.0, pbd_coeff=0.0, pbd_coeff_amortized=0.0, tick=0, volume_passes=0,
                right_target=None):
    """right_target: the Right lock's targets (right_targets()); given, the
    Right vertices (lock mask bit 1) are held there (Settings_LockRight)."""
    p = Params()
    p.gravity[:] = [float(g) for g in gravity]
    p.dt = dt
    p.time_corrected_drag = drag
    p.compliance = compliance
    p.poisson = poisson
    p.energy = energy
    p.simultaneous = 1 if simultaneous else 0
    p.yeoh[:] = [float(c) for c in yeoh]
    p.lock_active = 1 if lock else 0
    p.ground = 1 if ground else 0
    p.ground_n[:] = [float(c) for c in ground_n]
    p.ground_d = ground_d
    p.friction = friction
    p.damping = damping
    p.rayleigh_type = rayleigh_type
    p.pbd_damping = pbd_damping
    p.pbd_coeff = pbd_coeff
    p.pbd_coeff_amortized = pbd_coeff_amortized
    p.tick = tick
    p.volume_passes = volume_passes
    if right_target is not None:
        p._right_target = np.ascontiguousarray(right_target, np.float64).reshape(-1)  # kept alive with p
        p.lock_right = 1
        p.right_target = p._right_target.ctypes.data
    return p


def right_targets(nodes, transform, origin):
    """origin + transform * vec3(X0) per vertex (XPBDFEM/Geo.cpp:327), float
    arithmetic as the reference; transform column-major (9 floats)."""
    nd = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    m = np.ascontiguousarray(transform, np.float32)
    o = np.ascontiguousarray(origin, np.float32)
    out = np.zeros(nd.size, np.float64)
    lib().orc_right_targets(nd.size // 3, _p(nd), _p(m), _p(o), _p(out))
    return out.reshape(-1, 3)


def params_from_settings(s, dt, lock=True, tick=None, nodes=None):
    """orc_params from solver settings given as an xfem Settings struct or as
    a dict of its fields (reference semantics). tick: the tickId of the first
    substep (default: the settings' tick_id). nodes: the rest positions, for
    the Right lock's targets when the settings lock the Right side."""
    def g(k, default=None):
        if isinstance(s, dict):
            return s.get(k, default) if default is not None else s[k]
        return getattr(s, k, default) if default is not None else getattr(s, k)
    flags = int(g("flags"))
    return make_params(dt=dt, compliance=g("compliance"), poisson=g("poissons_ratio"), energy=(flags >> 6) & 31,
                       simultaneous=bool((flags >> 11) & 1), gravity=tuple(g("gravity")),
                       drag=g("time_corrected_drag"), yeoh=tuple(g("yeoh")),
                       lock=lock and bool(flags & (1 << 26)), ground=bool(g("ground")),
                       ground_n=tuple(g("ground_normal")), ground_d=g("ground_offset"), friction=g("friction"),
                       damping=g("damping", 0.0), rayleigh_type=(flags >> 20) & 3,
                       pbd_damping=g("pbd_damping", 0.0),
                       pbd_coeff=g("volume_and_time_corrected_pbd_damping", 0.0),
                       pbd_coeff_amortized=g("amortized_volume_and_time_corrected_pbd_damping", 0.0),
                       tick=int(g("tick_id", 0)) if tick is None else int(tick),
                       volume_passes=int(g("volume_passes", 0)),
                       right_target=(right_targets(nodes, list(g("locked_right_transform")), list(g("origin")))
                                     if nodes is not None and lock and flags & (1 << 27) else None))


_lib = None


def build():
    """Compile oracle/liboracle.so with the oracle's own Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        u32 = C.c_uint32
        L.orc_gen_tet_block.argtypes = [u32, u32, u32, C.c_float, C.c_float, C.c_float, u32, C.c_float, P, P]
        L.orc_right_targets.argtypes = [u32, P, P, P, P]
        L.orc_right_targets.restype = None
        L.orc_parse_tets.argtypes = [P, u32, P, P, P]
        L.orc_minstd_order.argtypes = [u32, P]
        L.orc_init_rest_f.argtypes = [P, u32, P, u32, C.c_float, P, P, P]
        L.orc_init_rest_d.argtypes = [P, u32, P, u32, C.c_double, P, P, P]
        L.orc_solve_tet_f.argtypes = [P, P, P, P, P, C.c_float, P]
        L.orc_solve_tet_d.argtypes = [P, P, P, P, P, C.c_double, P]
        L.orc_substeps_f.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, P, P, P]
        L.orc_substeps_d.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, P, P, P]
        L.orc_substeps_threaded_f.argtypes = [u32, P, P, P, P, u32, P, P, P, P, P, u32, u32, P, u32]
        L.orc_volume_f.argtypes = [P, u32, P]
        L.orc_volume_f.restype = C.c_float
        L.orc_volume_d.argtypes = [P, u32, P]
        L.orc_volume_d.restype = C.c_double
        L.orc_schedule.argtypes = [P, u32, P, u32, u32, u32, P, P, P, P, P, P, P]
        L.orc_adjoint_d.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, P, u32, P, P, P, P, P, P]
        L.orc_substeps_rings_f.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, P, P]
        L.orc_hex_substeps_rings_f.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, P, P]
        L.orc_hex_substeps_rings_d.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, P, P]
        L.orc_substeps_rings_d.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, P, P]
        L.orc_ring_schedule.argtypes = [P, u32, P, u32, u32, P, P, P]
        L.orc_ring_schedule_elems.argtypes = [P, u32, P, u32, u32, u32, P, P, P]
        L.orc_gen_hex_block.argtypes = [u32, u32, u32, C.c_float, C.c_float, C.c_float, u32, C.c_float, P, P]
        L.orc_parse_hexes.argtypes = [P, u32, P, P, P]
        L.orc_hex_tables.argtypes = [P, P, P]
        L.orc_hex_init_rest_f.argtypes = [P, u32, P, u32, C.c_float, P, P, P]
        L.orc_hex_init_rest_d.argtypes = [P, u32, P, u32, C.c_double, P, P, P]
        L.orc_solve_hex_f.argtypes = [P, P, P, P, P]
        L.orc_solve_hex_d.argtypes = [P, P, P, P, P]
        L.orc_hex_substeps_f.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_hex_substeps_d.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_hex_volume_f.argtypes = [P, u32, P, P]
        L.orc_hex_volume_f.restype = C.c_float
        L.orc_hex_volume_d.argtypes = [P, u32, P, P]
        L.orc_hex_volume_d.restype = C.c_double
        L.orc_hex_schedule.argtypes = [P, u32, P, u32, u32, P, P, P, P]
        L.orc_parse_mixed.argtypes = [P, u32, P, P, P, P, P]
        L.orc_elem_schedule.argtypes = [P, u32, P, u32, u32, u32, P, P, P, P]
        L.orc_mixed_init_rest_f.argtypes = [P, u32, P, u32, P, u32, C.c_float, P, P, P, P]
        L.orc_mixed_init_rest_d.argtypes = [P, u32, P, u32, P, u32, C.c_double, P, P, P, P]
        L.orc_mixed_substeps_f.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_mixed_substeps_d.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_mixed_volume_f.argtypes = [P, u32, P, u32, P, P]
        L.orc_mixed_volume_f.restype = C.c_float
        L.orc_mixed_volume_d.argtypes = [P, u32, P, u32, P, P]
        L.orc_mixed_volume_d.restype = C.c_double
        L.orc_t10_tables.argtypes = [P, P, P]
        L.orc_tet_edges.argtypes = [P, u32, u32, P, P, P]
        L.orc_t10_init_rest_f.argtypes = [P, u32, P, u32, P, u32, P, C.c_float, P, P, P, P]
        L.orc_t10_init_rest_d.argtypes = [P, u32, P, u32, P, u32, P, C.c_double, P, P, P, P]
        L.orc_solve_t10_f.argtypes = [P, P, P, P, P]
        L.orc_solve_t10_d.argtypes = [P, P, P, P, P]
        L.orc_t10_substeps_rings_f.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, u32, P, P]
        L.orc_t10_substeps_rings_d.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, u32, P, P]
        L.orc_ring_schedule_centres.argtypes = [P, u32, P, u32, u32, u32, u32, P, P, P]
        L.orc_h27_substeps_rings_f.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, u32, P, P]
        L.orc_quad_mesh.argtypes = [P, u32, u32, P, P, P, P, P, P]
        L.orc_qmixed_init_rest_f.argtypes = [P, u32, P, u32, P, u32, P, u32, P, u32, P, P, C.c_float, P, P, P, P, P]
        L.orc_qmixed_init_rest_d.argtypes = [P, u32, P, u32, P, u32, P, u32, P, u32, P, P, C.c_double, P, P, P, P, P]
        L.orc_qmixed_substeps_f.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_qmixed_substeps_d.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_qmixed_volume_f.argtypes = [P, u32, P, P, u32, P, P]
        L.orc_qmixed_volume_f.restype = C.c_float
        L.orc_qmixed_volume_d.argtypes = [P, u32, P, P, u32, P, P]
        L.orc_qmixed_volume_d.restype = C.c_double
        L.orc_h27_substeps_rings_d.argtypes = [u32, P, P, P, P, u32, P, P, P, P, u32, u32, P, P]
        L.orc_t10_substeps_f.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_t10_substeps_d.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_t10_volume_f.argtypes = [P, u32, P, P]
        L.orc_t10_volume_f.restype = C.c_float
        L.orc_t10_volume_d.argtypes = [P, u32, P, P]
        L.orc_t10_volume_d.restype = C.c_double
        L.orc_t10_schedule.argtypes = [P, u32, P, u32, u32, P, P, P, P]
        L.orc_h27_tables.argtypes = [P, P, P, P, P]
        L.orc_h27_mesh.argtypes = [P, u32, u32, P, P, P, P, P]
        L.orc_h27_init_rest_f.argtypes = [P, u32, P, u32, P, u32, P, u32, P, C.c_float, P, P, P, P]
        L.orc_h27_init_rest_d.argtypes = [P, u32, P, u32, P, u32, P, u32, P, C.c_double, P, P, P, P]
        L.orc_solve_h27_f.argtypes = [P, P, P, P, P]
        L.orc_solve_h27_d.argtypes = [P, P, P, P, P]
        L.orc_h27_substeps_f.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_h27_substeps_d.argtypes = [u32, P, P, P, P, u32, P, P, P, u32, P, P]
        L.orc_h27_volume_f.argtypes = [P, u32, P, P]
        L.orc_h27_volume_f.restype = C.c_float
        L.orc_h27_volume_d.argtypes = [P, u32, P, P]
        L.orc_h27_volume_d.restype = C.c_double
        L.orc_h27_schedule.argtypes = [P, u32, P, u32, u32, P, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def gen_tet_block(W, H, D, scale=(1.0, 1.0, 1.0), pattern=0, wonkiness=0.0):
    nv = (W + 1) * (H + 1) * (D + 1)
    nodes = np.zeros(3 * nv, np.float32)
    idx = np.zeros(30 * W * H * D, np.uint32)
    lib().orc_gen_tet_block(W, H, D, scale[0], scale[1], scale[2], pattern, wonkiness, _p(nodes), _p(idx))
    return nodes, idx


def parse_tets(idx):
    idx = np.ascontiguousarray(idx, np.uint32)
    nt, nv = C.c_uint32(), C.c_uint32()
    if lib().orc_parse_tets(_p(idx), idx.size, None, C.byref(nt), C.byref(nv)):
        raise ValueError("index stream holds a non-tet element")
    tets = np.zeros((nt.value, 4), np.uint32)
    lib().orc_parse_tets(_p(idx), idx.size, _p(tets), C.byref(nt), C.byref(nv))
    return tets, nv.value


def minstd_order(nt):
    o = np.zeros(nt, np.uint32)
    lib().orc_minstd_order(nt, _p(o))
    return o


def init_rest(nodes, tets, density, dtype=np.float32):
    nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    tets = np.ascontiguousarray(tets, np.uint32)
    nv, nt = nodes.size // 3, tets.shape[0]
    ep = np.zeros((nt, 17), dtype)
    w = np.zeros(nv, dtype)
    fl = np.zeros(nv, np.uint8)
    f = lib().orc_init_rest_f if dtype == np.float32 else lib().orc_init_rest_d
    f(_p(nodes), nv, _p(tets), nt, density, _p(ep), _p(w), _p(fl))
    return ep, w, fl


def solve_tet(X, w, ep, params, mu_override=0.0, dtype=np.float32, O=None):
    """One element solve; O (4x3, optional): start positions for the in-solve
    Rayleigh damping."""
    X = np.array(X, np.float64).reshape(4, 3).copy()
    Oa = None if O is None else np.ascontiguousarray(O, np.float64).reshape(4, 3)
    w = np.ascontiguousarray(w, dtype)
    ep = np.ascontiguousarray(ep, dtype)
    lam = np.zeros(2, dtype)
    f = lib().orc_solve_tet_f if dtype == np.float32 else lib().orc_solve_tet_d
    if f(_p(X), _p(Oa), _p(w), _p(ep), C.byref(params), mu_override, _p(lam)):
        raise ValueError("unsupported energy model")
    return X, lam


def substeps(X, V, w, tets, ep, order, nsub, params, lock_mask=None, tet_mu=None,
             dtype=np.float32, threads=None, colour_begin=None, want_lambdas=False):
    """Run nsub substeps in the given constraint order. Returns X, V, w,
    contact mask of the last substep, and (optionally) per-tet lambdas."""
    X = np.array(X, np.float64).reshape(-1).copy()
    V = np.array(V, np.float64).reshape(-1).copy()
    w = np.array(w, dtype).copy()
    nv = w.size
    tets = np.ascontiguousarray(tets, np.uint32)
    ep = np.ascontiguousarray(ep, dtype)
    order = np.ascontiguousarray(order, np.uint32)
    lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
    tm = None if tet_mu is None else np.ascontiguousarray(tet_mu, dtype)
    contact = np.zeros(nv, np.uint8)
    lam = np.zeros(2 * tets.shape[0], dtype) if want_lambdas else None
    if threads:
        cb = np.ascontiguousarray(colour_begin, np.uint32)
        rc = lib().orc_substeps_threaded_f(nv, _p(X), _p(V), _p(w), _p(lm), tets.shape[0], _p(tets), _p(ep),
                                           _p(tm), _p(order), _p(cb), cb.size - 1, nsub, C.byref(params),
                                           int(threads))
        contact = None
    else:
        f = lib().orc_substeps_f if dtype == np.float32 else lib().orc_substeps_d
        rc = f(nv, _p(X), _p(V), _p(w), _p(lm), tets.shape[0], _p(tets), _p(ep), _p(tm), _p(order), nsub,
               C.byref(params), _p(contact), _p(lam))
    if rc:
        raise ValueError("oracle substep failed (unsupported energy model?)")
    out = (X.reshape(-1, 3), V.reshape(-1, 3), w, contact)
    return out + (lam.reshape(-1, 2),) if want_lambdas else out


def substeps_rings(X, V, w, tets, ep, torder, vorder, nsub, params, lock_mask=None, dtype=np.float32):
    """nsub substeps of a continuous-pressure model (energy 8-10): every
    vertex's one-ring solved in `vorder`, PBD damping over the tets in
    `torder`. Returns X, V, w, contact mask."""
    X = np.array(X, np.float64).reshape(-1).copy()
    V = np.array(V, np.float64).reshape(-1).copy()
    w = np.array(w, dtype).copy()
    nv = w.size
    tets = np.ascontiguousarray(tets, np.uint32)
    ep = np.ascontiguousarray(ep, dtype)
    torder = np.ascontiguousarray(torder, np.uint32)
    vorder = np.ascontiguousarray(vorder, np.uint32)
    lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
    contact = np.zeros(nv, np.uint8)
    f = lib().orc_substeps_rings_f if dtype == np.float32 else lib().orc_substeps_rings_d
    if f(nv, _p(X), _p(V), _p(w), _p(lm), tets.shape[0], _p(tets), _p(ep), _p(torder), _p(vorder), nsub,
         C.byref(params), _p(contact)):
        raise ValueError("not a continuous-pressure energy model")
    return X.reshape(-1, 3), V.reshape(-1, 3), w, contact


def ring_schedule(nodes, tets, morton=1):
    """Vertex ring order of the continuous-pressure models (colour-major) and
    the colour offsets; tets (n, 4) or, on a hex mesh, hexes (n, 8)."""
    nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    tets = np.ascontiguousarray(tets, np.uint32)
    nv = nodes.size // 3
    vorder = np.zeros(nv, np.uint32)
    cb = np.zeros(nv + 1, np.uint32)
    ncol = C.c_uint32()
    if lib().orc_ring_schedule_elems(_p(nodes), nv, _p(tets), tets.shape[1], tets.shape[0], morton, _p(vorder),
                                     _p(cb), C.byref(ncol)):
        raise ValueError("ring schedule limits exceeded")
    return dict(vert_order=vorder, colour_vert_begin=cb[:ncol.value + 1], colours=ncol.value)


def volume(X, tets, dtype=np.float32):
    X = np.ascontiguousarray(X, np.float64).reshape(-1)
    tets = np.ascontiguousarray(tets, np.uint32)
    f = lib().orc_volume_f if dtype == np.float32 else lib().orc_volume_d
    return f(_p(X), tets.shape[0], _p(tets))


def schedule(nodes, tets, mode=1, morton=1):
    nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    tets = np.ascontiguousarray(tets, np.uint32)
    nv, nt = nodes.size // 3, tets.shape[0]
    cluster_of = np.zeros(nt, np.uint32)
    colour_of = np.zeros(max(nt, 1), np.uint32)
    rank = np.zeros(nv, np.uint32)
    order = np.zeros(nt, np.uint32)
    cb = np.zeros(nt + 1, np.uint32)
    ncl, ncol = C.c_uint32(), C.c_uint32()
    rc = lib().orc_schedule(_p(nodes), nv, _p(tets), nt, mode, morton, _p(cluster_of), C.byref(ncl),
                            _p(colour_of), C.byref(ncol), _p(rank), _p(order), _p(cb))
    if rc:
        raise ValueError("schedule limits exceeded")
    return dict(cluster_of=cluster_of, clusters=ncl.value, colour_of_cluster=colour_of[:ncl.value],
                colours=ncol.value, vert_rank=rank, tet_order=order, colour_tet_begin=cb[:ncol.value + 1])


def adjoint(X0, V0, w, tets, ep, tet_mu, order, nsub, params, tips, targets, lock_mask=None, grad=True,
            want_dx=False):
    """FP64 loss and (optionally) dL/dmu per tet, dL/dV0 and (want_dx) dL/dX0
    (oracle/xfem_oracle_adjoint.c)."""
    X0 = np.ascontiguousarray(X0, np.float64).reshape(-1)
    V0 = np.ascontiguousarray(V0, np.float64).reshape(-1)
    w = np.ascontiguousarray(w, np.float64)
    tets = np.ascontiguousarray(tets, np.uint32)
    ep = np.ascontiguousarray(ep, np.float64)
    tet_mu = np.ascontiguousarray(tet_mu, np.float64)
    order = np.ascontiguousarray(order, np.uint32)
    tips = np.ascontiguousarray(tips, np.uint32)
    targets = np.ascontiguousarray(targets, np.float64)
    lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
    loss = C.c_double()
    dmu = np.zeros(tets.shape[0]) if grad else None
    dv = np.zeros(X0.size) if grad else None
    dx = np.zeros(X0.size) if grad else None
    rc = lib().orc_adjoint_d(w.size, _p(X0), _p(V0), _p(w), _p(lm), tets.shape[0], _p(tets), _p(ep), _p(tet_mu),
                             _p(order), nsub, C.byref(params), tips.size, _p(tips), _p(targets), C.byref(loss),
                             _p(dmu), _p(dv), _p(dx))
    if rc:
        raise ValueError("adjoint: coupled Neo-Hookean only")
    if not grad:
        return loss.value
    return (loss.value, dmu, dv.reshape(-1, 3), dx.reshape(-1, 3)) if want_dx else (loss.value, dmu, dv.reshape(-1, 3))


# ---- linear hexahedra (oracle/xfem_oracle_hex.inc) ----
HEX_EP = 120  # values per hex record (ElementParamsLinearHex flattened)


def gen_hex_block(W, H, D, scale=(1.0, 1.0, 1.0), pattern=0, wonkiness=0.0):
    nv = (W + 1) * (H + 1) * (D + 1)
    nodes = np.zeros(3 * nv, np.float32)
    idx = np.zeros(9 * W * H * D, np.uint32)
    lib().orc_gen_hex_block(W, H, D, scale[0], scale[1], scale[2], pattern, wonkiness, _p(nodes), _p(idx))
    return nodes, idx


def parse_hexes(idx):
    idx = np.ascontiguousarray(idx, np.uint32)
    nh, nv = C.c_uint32(), C.c_uint32()
    if lib().orc_parse_hexes(_p(idx), idx.size, None, C.byref(nh), C.byref(nv)):
        raise ValueError("index stream holds a non-hex element")
    hexes = np.zeros((nh.value, 8), np.uint32)
    lib().orc_parse_hexes(_p(idx), idx.size, _p(hexes), C.byref(nh), C.byref(nv))
    return hexes, nv.value


def hex_tables():
    """(n8[8][8], g8[8][8][3], g1[8][3]) as the oracle builds them."""
    n8, g8, g1 = np.zeros((8, 8), np.float32), np.zeros((8, 8, 3), np.float32), np.zeros((8, 3), np.float32)
    lib().orc_hex_tables(_p(n8), _p(g8), _p(g1))
    return n8, g8, g1


def hex_init_rest(nodes, hexes, density, dtype=np.float32):
    nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    hexes = np.ascontiguousarray(hexes, np.uint32)
    nv, nh = nodes.size // 3, hexes.shape[0]
    ep = np.zeros((nh, HEX_EP), dtype)
    w = np.zeros(nv, dtype)
    fl = np.zeros(nv, np.uint8)
    f = lib().orc_hex_init_rest_f if dtype == np.float32 else lib().orc_hex_init_rest_d
    f(_p(nodes), nv, _p(hexes), nh, density, _p(ep), _p(w), _p(fl))
    return ep, w, fl


def solve_hex(X, w, ep, params, O, dtype=np.float32):
    X = np.array(X, np.float64).reshape(8, 3).copy()
    O = np.ascontiguousarray(O, np.float64).reshape(8, 3)
    w = np.ascontiguousarray(w, dtype)
    ep = np.ascontiguousarray(ep, dtype)
    f = lib().orc_solve_hex_f if dtype == np.float32 else lib().orc_solve_hex_d
    if f(_p(X), _p(O), _p(w), _p(ep), C.byref(params)):
        raise ValueError("energy model not covered on hexes")
    return X


def hex_substeps(X, V, w, hexes, ep, order, nsub, params, lock_mask=None, dtype=np.float32):
    """nsub substeps of a hex mesh in the hex order `order`. Returns X, V, w,
    contact mask of the last substep."""
    X = np.array(X, np.float64).reshape(-1).copy()
    V = np.array(V, np.float64).reshape(-1).copy()
    w = np.array(w, dtype).copy()
    nv = w.size
    hexes = np.ascontiguousarray(hexes, np.uint32)
    ep = np.ascontiguousarray(ep, dtype)
    order = np.ascontiguousarray(order, np.uint32)
    lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
    contact = np.zeros(nv, np.uint8)
    f = lib().orc_hex_substeps_f if dtype == np.float32 else lib().orc_hex_substeps_d
    if f(nv, _p(X), _p(V), _p(w), _p(lm), hexes.shape[0], _p(hexes), _p(ep), _p(order), nsub, C.byref(params),
         _p(contact)):
        raise ValueError("energy model not covered on hexes")
    return X.reshape(-1, 3), V.reshape(-1, 3), w, contact


def hex_substeps_rings(X, V, w, hexes, ep, horder, vorder, nsub, params, lock_mask=None, dtype=np.float32):
    """nsub substeps of a continuous-pressure model (energy 8-10) on a hex
    mesh: every vertex's one-ring solved in `vorder`, PBD damping over the
    hexes in `horder`. Returns X, V, w, contact mask."""
    X = np.array(X, np.float64).reshape(-1).copy()
    V = np.array(V, np.float64).reshape(-1).copy()
    w = np.array(w, dtype).copy()
    nv = w.size
    hexes = np.ascontiguousarray(hexes, np.uint32)
    ep = np.ascontiguousarray(ep, dtype)
    horder = np.ascontiguousarray(horder, np.uint32)
    vorder = np.ascontiguousarray(vorder, np.uint32)
    lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
    contact = np.zeros(nv, np.uint8)
    f = lib().orc_hex_substeps_rings_f if dtype == np.float32 else lib().orc_hex_substeps_rings_d
    if f(nv, _p(X), _p(V), _p(w), _p(lm), hexes.shape[0], _p(hexes), _p(ep), _p(horder), _p(vorder), nsub,
         C.byref(params), _p(contact)):
        raise ValueError("not a continuous-pressure energy model")
    return X.reshape(-1, 3), V.reshape(-1, 3), w, contact


def hex_volume(X, hexes, ep, dtype=np.float32):
    X = np.ascontiguousarray(X, np.float64).reshape(-1)
    hexes = np.ascontiguousarray(hexes, np.uint32)
    ep = np.ascontiguousarray(ep, dtype)
    f = lib().orc_hex_volume_f if dtype == np.float32 else lib().orc_hex_volume_d
    return f(_p(X), hexes.shape[0], _p(hexes), _p(ep))


def hex_schedule(nodes, hexes, morton=1):
    """Hex order (colour-major), colour offsets and vertex ranks of the hex
    schedule."""
    nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    hexes = np.ascontiguousarray(hexes, np.uint32)
    nv, nh = nodes.size // 3, hexes.shape[0]
    rank = np.zeros(nv, np.uint32)
    order = np.zeros(nh, np.uint32)
    cb = np.zeros(nh + 1, np.uint32)
    ncol = C.c_uint32()
    if lib().orc_hex_schedule(_p(nodes), nv, _p(hexes), nh, morton, _p(rank), _p(order), _p(cb), C.byref(ncol)):
        raise ValueError("hex schedule needs more than 4096 colours")
    return dict(vert_rank=rank, hex_order=order, colour_hex_begin=cb[:ncol.value + 1], colours=ncol.value)


# ---- meshes mixing tets and hexes (oracle/xfem_oracle_mixed.inc) ----
def parse_mixed(idx):
    """(tets[nt, 4], hexes[nh, 8], vertex count) of a tagged stream of tets
    and hexes, each kind in stream order."""
    idx = np.ascontiguousarray(idx, np.uint32)
    nt, nh, nv = C.c_uint32(), C.c_uint32(), C.c_uint32()
    if lib().orc_parse_mixed(_p(idx), idx.size, None, C.byref(nt), None, C.byref(nh), C.byref(nv)):
        raise ValueError("index stream holds an element that is neither a tet nor a hex")
    tets = np.zeros((nt.value, 4), np.uint32)
    hexes = np.zeros((nh.value, 8), np.uint32)
    lib().orc_parse_mixed(_p(idx), idx.size, _p(tets), C.byref(nt), _p(hexes), C.byref(nh), C.byref(nv))
    return tets, hexes, nv.value


def tet_element_schedule(nodes, tets, morton=1):
    """The tets of a mixed mesh coloured and ordered as hexes are: tet order
    (colour-major), colour offsets, vertex ranks."""
    nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    tets = np.ascontiguousarray(tets, np.uint32)
    nv, nt = nodes.size // 3, tets.shape[0]
    rank = np.zeros(nv, np.uint32)
    order = np.zeros(nt, np.uint32)
    cb = np.zeros(nt + 1, np.uint32)
    ncol = C.c_uint32()
    if lib().orc_elem_schedule(_p(nodes), nv, _p(tets), nt, 4, morton, _p(rank), _p(order), _p(cb), C.byref(ncol)):
        raise ValueError("tet schedule needs more than 4096 colours")
    return dict(vert_rank=rank, tet_order=order, colour_tet_begin=cb[:ncol.value + 1], colours=ncol.value)


def mixed_init_rest(nodes, tets, hexes, density, dtype=np.float32):
    """GeoLinear3d::Init on a mixed mesh: (tet records, hex records, w, flags)."""
    nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
    tets = np.ascontiguousarray(tets, np.uint32)
    hexes = np.ascontiguousarray(hexes, np.uint32)
    nv, nt, nh = nodes.size // 3, tets.shape[0], hexes.shape[0]
    ep = np.zeros((nt, 17), dtype)
    hep = np.zeros((nh, HEX_EP), dtype)
    w = np.zeros(nv, dtype)
    fl = np.zeros(nv, np.uint8)
    f = lib().orc_mixed_init_rest_f if dtype == np.float32 else lib().orc_mixed_init_rest_d
    f(_p(nodes), nv, _p(tets), nt, _p(hexes), nh, density, _p(ep), _p(hep), _p(w), _p(fl))
    return ep, hep, w, fl


def mixed_substeps(X, V, w, tets, ep, torder, hexes, hep, horder, nsub, params, lock_mask=None, dtype=np.float32):
    """nsub substeps of a mixed mesh (tets in torder, then hexes in horder).
    Returns X, V, w, contact mask."""
    X = np.array(X, np.float64).reshape(-1).copy()
    V = np.array(V, np.float64).reshape(-1).copy()
    w = np.array(w, dtype).copy()
    nv = w.size
    tets = np.ascontiguousarray(tets, np.uint32)
    hexes = np.ascontiguousarray(hexes, np.uint32)
    ep = np.ascontiguousarray(ep, dtype)
    hep = np.ascontiguousarray(hep, dtype)
    torder = np.ascontiguousarray(torder, np.uint32)
    horder = np.ascontiguousarray(horder, np.uint32)
    lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
    contact = np.zeros(nv, np.uint8)
    f = lib().orc_mixed_substeps_f if dtype == np.float32 else lib().orc_mixed_substeps_d
    if f(nv, _p(X), _p(V), _p(w), _p(lm), tets.shape[0], _p(tets), _p(ep), _p(torder), hexes.shape[0], _p(hexes),
         _p(hep), _p(horder), nsub, C.byref(params), _p(contact)):
        raise ValueError("energy model not covered on mixed meshes")
    return X.reshape(-1, 3), V.reshape(-1, 3), w, contact


def mixed_volume(X, tets, hexes, hep, dtype=np.float32):
    X = np.ascontiguousarray(X, np.float64).reshape(-1)
    tets = np.ascontiguousarray(tets, np.uint32)
    hexes = np.ascontiguousarray(hexes, np.uint32)
    hep = np.ascontiguousarray(hep, dtype)
    f = lib().orc_mixed_volume_f if dtype == np.float32 else lib().orc_mixed_volume_d
    return f(_p(X), tets.shape[0], _p(tets), hexes.shape[0], _p(hexes), _p(hep))


def mixed_block(W, H, D, scale, pattern, wonkiness, split):
    """A GenerateHexBlock mesh (XPBDFEM/MeshGen.cpp:156-221) in which the
    cells that `split(x, y, z)` selects are replaced by GenerateTetBlock's six
    tets of the same corners (XPBDFEM/MeshGen.cpp:223-244), in cell order:
    a mixed stream of tag-4 and tag-8 records on the same nodes."""
    nodes, idx = gen_hex_block(W, H, D, scale, pattern, wonkiness)
    cells = idx.reshape(-1, 9)[:, 1:]
    six = ((0, 1, 5, 7), (0, 7, 3, 1), (0, 2, 3, 7), (0, 7, 6, 2), (0, 4, 6, 7), (0, 7, 5, 4))
    out = []
    k = 0
    for z in range(D):
        for y in range(H):
            for x in range(W):
                c = cells[k]
                k += 1
                if split(x, y, z):
                    for t in six:
                        out += [4] + [int(c[n]) for n in t]
                else:
                    out += [8] + [int(n) for n in c]
    return nodes, np.array(out, np.uint32)


# ---- quadratic tetrahedra (oracle/xfem_oracle_t10.inc) ----
T10_EP = 56  # values per T10 rest-state record (ElementParamsQuadraticTet flattened)


def t10_tables():
    g4, g10, w10 = np.zeros((4, 10, 3), np.float32), np.zeros((10, 10, 3), np.float32), np.zeros(10, np.float32)
    lib().orc_t10_tables(_p(g4), _p(g10), _p(w10))
    return g4, g10, w10


def tet_edges(tets, nv):
    """Connectivity3d's edge numbering and GeoQuadratic3d's T10 indices:
    (edges[ne, 2], t10[nt, 10])."""
    tets = np.ascontiguousarray(tets, np.uint32)
    nt = tets.shape[0]
    edges = np.zeros((max(6 * nt, 1), 2), np.uint32)
    t10 = np.zeros((nt, 10), np.uint32)
    ne = C.c_uint32()
    if lib().orc_tet_edges(_p(tets), nt, nv, _p(edges), C.byref(ne), _p(t10)):
        raise MemoryError("edge enumeration failed")
    return edges[:ne.value].copy(), t10


class Quadratic:
    """A T10 mesh as GeoQuadratic3d builds it from a tet mesh."""

    def __init__(self, nodes, idx, density, dtype=np.float32):
        nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
        self.tets, self.nv = parse_tets(idx)
        self.edges, self.t10 = tet_edges(self.tets, self.nv)
        n = self.nv + self.edges.shape[0]
        nt = self.tets.shape[0]
        self.X0 = np.zeros((n, 3), np.float64)
        self.ep = np.zeros((nt, T10_EP), dtype)
        self.w = np.zeros(n, dtype)
        self.flags = np.zeros(n, np.uint8)
        f = lib().orc_t10_init_rest_f if dtype == np.float32 else lib().orc_t10_init_rest_d
        f(_p(nodes), self.nv, _p(self.tets), nt, _p(self.edges), self.edges.shape[0], _p(self.t10), density,
          _p(self.X0), _p(self.ep), _p(self.w), _p(self.flags))
        self.dtype = dtype

    def schedule(self, morton=1):
        X = self.X0.astype(np.float32)
        n, nt = X.shape[0], self.t10.shape[0]
        rank = np.zeros(n, np.uint32)
        order = np.zeros(nt, np.uint32)
        cb = np.zeros(nt + 1, np.uint32)
        ncol = C.c_uint32()
        if lib().orc_t10_schedule(_p(X), n, _p(self.t10), nt, morton, _p(rank), _p(order), _p(cb), C.byref(ncol)):
            raise ValueError("T10 schedule needs more than 4096 colours")
        return dict(vert_rank=rank, tet_order=order, colour_tet_begin=cb[:ncol.value + 1], colours=ncol.value)

    def substeps(self, X, V, w, order, nsub, params, lock_mask=None):
        X = np.array(X, np.float64).reshape(-1).copy()
        V = np.array(V, np.float64).reshape(-1).copy()
        w = np.array(w, self.dtype).copy()
        order = np.ascontiguousarray(order, np.uint32)
        lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
        contact = np.zeros(w.size, np.uint8)
        f = lib().orc_t10_substeps_f if self.dtype == np.float32 else lib().orc_t10_substeps_d
        if f(w.size, _p(X), _p(V), _p(w), _p(lm), self.t10.shape[0], _p(self.t10), _p(self.ep), _p(order), nsub,
             C.byref(params), _p(contact)):
            raise ValueError("energy model not covered on quadratic tets")
        return X.reshape(-1, 3), V.reshape(-1, 3), w, contact

    def ring_schedule(self, morton=1):
        """Ring order of the continuous-pressure models over the T10s: the
        rings of the mesh's own vertices (not the edge nodes), colour-major."""
        X = self.X0.astype(np.float32).reshape(-1)
        n = self.X0.shape[0]
        vorder = np.zeros(self.nv, np.uint32)
        cb = np.zeros(self.nv + 1, np.uint32)
        ncol = C.c_uint32()
        if lib().orc_ring_schedule_centres(_p(X), n, _p(self.t10), 10, self.t10.shape[0], self.nv, morton, _p(vorder),
                                           _p(cb), C.byref(ncol)):
            raise ValueError("ring schedule limits exceeded")
        return dict(vert_order=vorder, colour_vert_begin=cb[:ncol.value + 1], colours=ncol.value)

    def substeps_rings(self, X, V, w, torder, vorder, nsub, params, lock_mask=None):
        """Substeps with a continuous-pressure model (energy 8-10)."""
        X = np.array(X, np.float64).reshape(-1).copy()
        V = np.array(V, np.float64).reshape(-1).copy()
        w = np.array(w, self.dtype).copy()
        torder = np.ascontiguousarray(torder, np.uint32)
        vorder = np.ascontiguousarray(vorder, np.uint32)
        lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
        contact = np.zeros(w.size, np.uint8)
        f = lib().orc_t10_substeps_rings_f if self.dtype == np.float32 else lib().orc_t10_substeps_rings_d
        if f(w.size, _p(X), _p(V), _p(w), _p(lm), self.t10.shape[0], _p(self.t10), _p(self.ep), _p(torder),
             _p(vorder), self.nv, nsub, C.byref(params), _p(contact)):
            raise ValueError("not a continuous-pressure model")
        return X.reshape(-1, 3), V.reshape(-1, 3), w, contact

    def volume(self, X):
        X = np.ascontiguousarray(X, np.float64).reshape(-1)
        f = lib().orc_t10_volume_f if self.dtype == np.float32 else lib().orc_t10_volume_d
        return f(_p(X), self.t10.shape[0], _p(self.t10), _p(self.ep))


def solve_t10(X, w, ep, params, O, dtype=np.float32):
    X = np.array(X, np.float64).reshape(10, 3).copy()
    O = np.ascontiguousarray(O, np.float64).reshape(10, 3)
    w = np.ascontiguousarray(w, dtype)
    ep = np.ascontiguousarray(ep, dtype)
    f = lib().orc_solve_t10_f if dtype == np.float32 else lib().orc_solve_t10_d
    if f(_p(X), _p(O), _p(w), _p(ep), C.byref(params)):
        raise ValueError("energy model not covered on quadratic tets")
    return X


H27_EP = 703  # values per H27 rest-state record (ElementParamsQuadraticHex flattened)


def h27_tables():
    """(g8[8][27][3], g27[27][27][3], n27[27][27], map27[27][8][3], w27[27])."""
    g8, g27 = np.zeros((8, 27, 3), np.float32), np.zeros((27, 27, 3), np.float32)
    n27, map27, w27 = np.zeros((27, 27), np.float32), np.zeros((27, 8, 3), np.float32), np.zeros(27, np.float32)
    lib().orc_h27_tables(_p(g8), _p(g27), _p(n27), _p(map27), _p(w27))
    return g8, g27, n27, map27, w27


def h27_mesh(hexes, nv):
    """Connectivity3d's edges and quads of a hex mesh and GeoQuadratic3d's H27
    indices: (edges[ne, 2], quads[nq, 4], h27[nh, 27])."""
    hexes = np.ascontiguousarray(hexes, np.uint32)
    nh = hexes.shape[0]
    edges = np.zeros((max(12 * nh, 1), 2), np.uint32)
    quads = np.zeros((max(6 * nh, 1), 4), np.uint32)
    h27 = np.zeros((nh, 27), np.uint32)
    ne, nq = C.c_uint32(), C.c_uint32()
    if lib().orc_h27_mesh(_p(hexes), nh, nv, _p(edges), C.byref(ne), _p(quads), C.byref(nq), _p(h27)):
        raise MemoryError("mesh enumeration failed")
    return edges[:ne.value].copy(), quads[:nq.value].copy(), h27


class QuadraticHex:
    """A hex mesh as GeoQuadratic3d builds it: H27 elements."""

    def __init__(self, nodes, idx, density, dtype=np.float32):
        nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
        self.hexes, self.nv = parse_hexes(idx)
        self.edges, self.quads, self.h27 = h27_mesh(self.hexes, self.nv)
        nh = self.hexes.shape[0]
        n = self.nv + self.edges.shape[0] + self.quads.shape[0] + nh
        self.X0 = np.zeros((n, 3), np.float64)
        self.ep = np.zeros((nh, H27_EP), dtype)
        self.w = np.zeros(n, dtype)
        self.flags = np.zeros(n, np.uint8)
        f = lib().orc_h27_init_rest_f if dtype == np.float32 else lib().orc_h27_init_rest_d
        f(_p(nodes), self.nv, _p(self.hexes), nh, _p(self.edges), self.edges.shape[0], _p(self.quads),
          self.quads.shape[0], _p(self.h27), density, _p(self.X0), _p(self.ep), _p(self.w), _p(self.flags))
        self.dtype = dtype

    def schedule(self, morton=1):
        X = self.X0.astype(np.float32)
        n, nh = X.shape[0], self.h27.shape[0]
        rank = np.zeros(n, np.uint32)
        order = np.zeros(nh, np.uint32)
        cb = np.zeros(nh + 1, np.uint32)
        ncol = C.c_uint32()
        if lib().orc_h27_schedule(_p(X), n, _p(self.h27), nh, morton, _p(rank), _p(order), _p(cb), C.byref(ncol)):
            raise ValueError("H27 schedule needs more than 4096 colours")
        return dict(vert_rank=rank, hex_order=order, colour_hex_begin=cb[:ncol.value + 1], colours=ncol.value)

    def substeps(self, X, V, w, order, nsub, params, lock_mask=None):
        X = np.array(X, np.float64).reshape(-1).copy()
        V = np.array(V, np.float64).reshape(-1).copy()
        w = np.array(w, self.dtype).copy()
        order = np.ascontiguousarray(order, np.uint32)
        lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
        contact = np.zeros(w.size, np.uint8)
        f = lib().orc_h27_substeps_f if self.dtype == np.float32 else lib().orc_h27_substeps_d
        if f(w.size, _p(X), _p(V), _p(w), _p(lm), self.h27.shape[0], _p(self.h27), _p(self.ep), _p(order), nsub,
             C.byref(params), _p(contact)):
            raise ValueError("energy model not covered on quadratic hexes")
        return X.reshape(-1, 3), V.reshape(-1, 3), w, contact

    def ring_schedule(self, morton=1):
        """Ring order of the continuous-pressure models over the H27s: the
        rings of the mesh's own vertices (not the added nodes), colour-major."""
        X = self.X0.astype(np.float32).reshape(-1)
        n = self.X0.shape[0]
        vorder = np.zeros(self.nv, np.uint32)
        cb = np.zeros(self.nv + 1, np.uint32)
        ncol = C.c_uint32()
        if lib().orc_ring_schedule_centres(_p(X), n, _p(self.h27), 27, self.h27.shape[0], self.nv, morton, _p(vorder),
                                           _p(cb), C.byref(ncol)):
            raise ValueError("ring schedule limits exceeded")
        return dict(vert_order=vorder, colour_vert_begin=cb[:ncol.value + 1], colours=ncol.value)

    def substeps_rings(self, X, V, w, horder, vorder, nsub, params, lock_mask=None):
        """Substeps with a continuous-pressure model (energy 8-10)."""
        X = np.array(X, np.float64).reshape(-1).copy()
        V = np.array(V, np.float64).reshape(-1).copy()
        w = np.array(w, self.dtype).copy()
        horder = np.ascontiguousarray(horder, np.uint32)
        vorder = np.ascontiguousarray(vorder, np.uint32)
        lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
        contact = np.zeros(w.size, np.uint8)
        f = lib().orc_h27_substeps_rings_f if self.dtype == np.float32 else lib().orc_h27_substeps_rings_d
        if f(w.size, _p(X), _p(V), _p(w), _p(lm), self.h27.shape[0], _p(self.h27), _p(self.ep), _p(horder),
             _p(vorder), self.nv, nsub, C.byref(params), _p(contact)):
            raise ValueError("not a continuous-pressure model")
        return X.reshape(-1, 3), V.reshape(-1, 3), w, contact

    def volume(self, X):
        X = np.ascontiguousarray(X, np.float64).reshape(-1)
        f = lib().orc_h27_volume_f if self.dtype == np.float32 else lib().orc_h27_volume_d
        return f(_p(X), self.h27.shape[0], _p(self.h27), _p(self.ep))


def quad_mesh(idx, nv):
    """Connectivity3d's edges and quads of a tagged stream that may mix tets
    and hexes, and GeoQuadratic3d's indices: (edges[ne, 2], quads[nq, 4],
    t10[nt, 10], h27[nh, 27])."""
    idx = np.ascontiguousarray(idx, np.uint32)
    tets, hexes, _ = parse_mixed(idx)
    nt, nh = tets.shape[0], hexes.shape[0]
    edges = np.zeros((max(6 * nt + 12 * nh, 1), 2), np.uint32)
    quads = np.zeros((max(6 * nh, 1), 4), np.uint32)
    t10 = np.zeros((nt, 10), np.uint32)
    h27 = np.zeros((nh, 27), np.uint32)
    ne, nq = C.c_uint32(), C.c_uint32()
    if lib().orc_quad_mesh(_p(idx), idx.size, nv, _p(edges), C.byref(ne), _p(quads), C.byref(nq), _p(t10), _p(h27)):
        raise ValueError("not a stream of tets and hexes")
    return edges[:ne.value].copy(), quads[:nq.value].copy(), t10, h27


class QuadraticMixed:
    """A mesh mixing tets and hexes as GeoQuadratic3d builds it: T10s and
    H27s in one body."""

    def __init__(self, nodes, idx, density, dtype=np.float32):
        nodes = np.ascontiguousarray(nodes, np.float32).reshape(-1)
        self.tets, self.hexes, self.nv = parse_mixed(idx)
        self.edges, self.quads, self.t10, self.h27 = quad_mesh(idx, self.nv)
        nt, nh = self.tets.shape[0], self.hexes.shape[0]
        ne, nq = self.edges.shape[0], self.quads.shape[0]
        n = self.nv + ne + nq + nh
        self.X0 = np.zeros((n, 3), np.float64)
        self.ept = np.zeros((nt, T10_EP), dtype)
        self.eph = np.zeros((nh, H27_EP), dtype)
        self.w = np.zeros(n, dtype)
        self.flags = np.zeros(n, np.uint8)
        f = lib().orc_qmixed_init_rest_f if dtype == np.float32 else lib().orc_qmixed_init_rest_d
        f(_p(nodes), self.nv, _p(self.edges), ne, _p(self.quads), nq, _p(self.hexes), nh, _p(self.tets), nt,
          _p(self.t10), _p(self.h27), density, _p(self.X0), _p(self.ept), _p(self.eph), _p(self.w), _p(self.flags))
        self.dtype = dtype

    def schedules(self, morton=1):
        """The T10 colouring and the H27 colouring over all vertices' ranks."""
        X = self.X0.astype(np.float32)
        n = X.shape[0]
        out = {}
        for name, el, per, fn in (("t10", self.t10, 10, lib().orc_t10_schedule),
                                  ("h27", self.h27, 27, lib().orc_h27_schedule)):
            ne = el.shape[0]
            rank = np.zeros(n, np.uint32)
            order = np.zeros(ne, np.uint32)
            cb = np.zeros(ne + 1, np.uint32)
            ncol = C.c_uint32()
            if fn(_p(X), n, _p(el), ne, morton, _p(rank), _p(order), _p(cb), C.byref(ncol)):
                raise ValueError("schedule needs more than 4096 colours")
            out[name + "_order"] = order
            out["colour_" + name + "_begin"] = cb[:ncol.value + 1]
            out["vert_rank"] = rank
        return out

    def substeps(self, X, V, w, torder, horder, nsub, params, lock_mask=None):
        X = np.array(X, np.float64).reshape(-1).copy()
        V = np.array(V, np.float64).reshape(-1).copy()
        w = np.array(w, self.dtype).copy()
        torder = np.ascontiguousarray(torder, np.uint32)
        horder = np.ascontiguousarray(horder, np.uint32)
        lm = None if lock_mask is None else np.ascontiguousarray(lock_mask, np.uint8)
        contact = np.zeros(w.size, np.uint8)
        f = lib().orc_qmixed_substeps_f if self.dtype == np.float32 else lib().orc_qmixed_substeps_d
        if f(w.size, _p(X), _p(V), _p(w), _p(lm), self.t10.shape[0], _p(self.t10), _p(self.ept), _p(torder),
             self.h27.shape[0], _p(self.h27), _p(self.eph), _p(horder), nsub, C.byref(params), _p(contact)):
            raise ValueError("energy model not covered on quadratic mixed meshes")
        return X.reshape(-1, 3), V.reshape(-1, 3), w, contact

    def volume(self, X):
        X = np.ascontiguousarray(X, np.float64).reshape(-1)
        f = lib().orc_qmixed_volume_f if self.dtype == np.float32 else lib().orc_qmixed_volume_d
        return f(_p(X), self.t10.shape[0], _p(self.t10), _p(self.ept), self.h27.shape[0], _p(self.h27), _p(self.eph))


def solve_h27(X, w, ep, params, O, dtype=np.float32):
    X = np.array(X, np.float64).reshape(27, 3).copy()
    O = np.ascontiguousarray(O, np.float64).reshape(27, 3)
    w = np.ascontiguousarray(w, dtype)
    ep = np.ascontiguousarray(ep, dtype)
    f = lib().orc_solve_h27_f if dtype == np.float32 else lib().orc_solve_h27_d
    if f(_p(X), _p(O), _p(w), _p(ep), C.byref(params)):
        raise ValueError("energy model not covered on quadratic hexes")
    return X
