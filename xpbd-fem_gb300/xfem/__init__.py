"""Python mirror of the reference's body interface over libxfem.so's C ABI.

`Body` plays the role of the reference's GeoLinear3d (XPBDFEM/Geo.h:137-153):
construct it from the tagged index stream and node array exactly as
GeoLinear3d::Init is called (XPBDFEM/Geo.cpp:697), then call `substep(dt)`
(Geo3d::Substep, XPBDFEM/Geo.cpp:305) or `step_frames(...)` (the substep loop
of Sim::Update, XPBDFEM/Demo.cpp:67-90). `Settings` mirrors struct Settings
(XPBDFEM/Settings.h:79-102). A hex stream (tag 8) is GeoLinear3d's hex
path; element type T10 or H27 in the settings' flags bits 0-3 makes a body
GeoQuadratic3d (XPBDFEM/Geo.cpp:836): a tet stream becomes T10s, a hex stream
H27s, and the body's vertices gain the added nodes. All compute runs in
libxfem.so on the GPU; there is no CPU fallback: without the library or a
CUDA device every call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libxfem.so")

OK, EINVAL, EUNSUPPORTED, ENOMEM, ECUDA, EDEVICE_TIMEOUT, ELIMIT, ENONFINITE = 0, -1, -2, -3, -4, -5, -6, -7
# failure-detection test hooks (xfem_test_hook)
HOOK_MISSING_ARRIVAL, HOOK_BARRIER_BASE, HOOK_FAIL_ALLOC = 1, 2, 3
ELEMENT_TYPE_MASK = 15  # flags bits 0-3 (Settings_ElementTypeMask)
ELEMENT_T4, ELEMENT_T10, ELEMENT_H8, ELEMENT_H27 = 5, 6, 7, 8
ENERGY_BIT = 6
# energy ids, XPBDFEM/Settings.h:41-53
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
MAX_VOLUME_PASSES = 64
XPBD_SOLVE_BIT = 11
LOCK_LEFT = 1 << 26
LOCK_RIGHT = 1 << 27
REF_YEOH = (0.1095, 14.95, 4.595)  # XPBDFEM/Fem.cpp:526


class XfemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"xfem error {code}: {msg}")
        self.code = code


class Settings(C.Structure):
    """xfem_settings (include/xfem.h); field order of Settings, XPBDFEM/Settings.h:79-91."""
    _fields_ = [
        ("time_scale", C.c_float), ("substeps_per_second", C.c_float), ("volume_passes", C.c_uint32),
        ("gravity", C.c_float * 3), ("compliance", C.c_float), ("damping", C.c_float),
        ("pbd_damping", C.c_float), ("drag", C.c_float), ("poissons_ratio", C.c_float),
        ("wonkiness", C.c_float), ("left_right_separation", C.c_float), ("flags", C.c_uint32),
        ("time_corrected_drag", C.c_float), ("yeoh", C.c_float * 3), ("ground", C.c_uint32),
        ("ground_normal", C.c_float * 3), ("ground_offset", C.c_float), ("friction", C.c_float),
        ("volume_and_time_corrected_pbd_damping", C.c_float),
        ("amortized_volume_and_time_corrected_pbd_damping", C.c_float), ("tick_id", C.c_uint32),
        ("locked_right_transform", C.c_float * 9), ("origin", C.c_float * 3),
    ]


class Options(C.Structure):
    _fields_ = [
        ("cluster_mode", C.c_uint32), ("no_morton", C.c_uint32), ("sync_mode", C.c_uint32),
        ("block_size", C.c_uint32), ("keep_lambdas", C.c_uint32), ("device", C.c_int32),
        ("stream", C.c_void_p), ("host_setup", C.c_uint32), ("wait_timeout_ms", C.c_uint32),
        ("bricks", C.c_uint32),
    ]


class Mesh(C.Structure):
    _fields_ = [("node_data", C.c_void_p), ("node_data_count", C.c_uint32), ("idx_data", C.c_void_p),
                ("idx_data_count", C.c_uint32), ("density", C.c_float)]


class Info(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("bodies", "vertices", "tets", "clusters", "colours", "isolated",
                                          "chunks", "tet_rows", "block_size", "blocks", "sync_mode",
                                          "cluster_mode", "max_chunk_deps", "bricks")] + [("device_bytes", C.c_uint64)]


# every symbol include/xfem.h declares
EXPORTS = [
    "xfem_settings_default", "xfem_create", "xfem_create_ex", "xfem_batch_create", "xfem_destroy",
    "xfem_get_info", "xfem_set_settings", "xfem_set_lock_mask", "xfem_set_tet_mu", "xfem_substep",
    "xfem_step_frames", "xfem_synchronize", "xfem_get_positions", "xfem_set_positions",
    "xfem_get_velocities", "xfem_set_velocities", "xfem_set_state", "xfem_get_inverse_masses", "xfem_get_contacts",
    "xfem_get_lambdas", "xfem_calculate_volume", "xfem_get_rest_state", "xfem_get_schedule",
    "xfem_body_counts", "xfem_time_corrected_drag", "xfem_generate_tet_block", "xfem_alloc_host",
    "xfem_free_host", "xfem_last_error", "xfem_compute_rest_state", "xfem_compute_schedule",
    "xfem_step_frames_noalloc", "xfem_adjoint_forward", "xfem_adjoint_backward", "xfem_pbd_damping_coefficients",
    "xfem_get_ring_schedule", "xfem_compute_ring_schedule", "xfem_body_hex_count", "xfem_get_hex_rest_state",
    "xfem_get_hex_schedule", "xfem_compute_hex_rest_state", "xfem_compute_hex_schedule", "xfem_generate_hex_block",
    "xfem_body_t10_count", "xfem_get_t10_rest_state", "xfem_get_t10_schedule", "xfem_compute_t10_edges",
    "xfem_compute_t10_rest_state", "xfem_compute_t10_schedule", "xfem_body_h27_count", "xfem_get_h27_rest_state",
    "xfem_get_h27_schedule", "xfem_compute_h27_mesh", "xfem_compute_h27_rest_state", "xfem_compute_h27_schedule",
    "xfem_test_hook", "xfem_get_mixed_tet_schedule", "xfem_compute_mixed_rest_state", "xfem_compute_mixed_schedule",
]
HEX_EP = 120  # floats per hex rest-state record (ElementParamsLinearHex flattened)
T10_EP = 56  # floats per T10 rest-state record (ElementParamsQuadraticTet flattened)
H27_EP = 703  # floats per H27 rest-state record (ElementParamsQuadraticHex flattened)

_lib = None


def lib():
    """Loads libxfem.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing; build it with xpbd-fem_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        P, u32, f32 = C.c_void_p, C.c_uint32, C.c_float
        for name in EXPORTS:
            getattr(L, name).restype = C.c_int
        L.xfem_last_error.restype = C.c_char_p
        L.xfem_time_corrected_drag.restype = C.c_float
        L.xfem_time_corrected_drag.argtypes = [f32, f32]
        L.xfem_alloc_host.restype = P
        L.xfem_alloc_host.argtypes = [C.c_size_t]
        L.xfem_free_host.restype = None
        L.xfem_free_host.argtypes = [P]
        L.xfem_settings_default.argtypes = [P]
        L.xfem_create_ex.argtypes = [P, u32, P, u32, f32, P, P, P]
        L.xfem_create.argtypes = [P, u32, P, u32, f32, P, P]
        L.xfem_batch_create.argtypes = [u32, P, P, P, P]
        L.xfem_destroy.argtypes = [P]
        L.xfem_get_info.argtypes = [P, P]
        L.xfem_set_settings.argtypes = [P, u32, P]
        L.xfem_set_lock_mask.argtypes = [P, u32, P]
        L.xfem_set_tet_mu.argtypes = [P, u32, P]
        L.xfem_substep.argtypes = [P, f32]
        L.xfem_step_frames.argtypes = [P, u32, u32, f32]
        L.xfem_synchronize.argtypes = [P]
        L.xfem_step_frames_noalloc.argtypes = [P, u32, u32, f32]
        L.xfem_test_hook.argtypes = [P, u32, u32]
        for n in ("xfem_get_positions", "xfem_set_positions", "xfem_get_velocities", "xfem_set_velocities",
                  "xfem_get_inverse_masses", "xfem_get_contacts", "xfem_get_lambdas", "xfem_calculate_volume"):
            getattr(L, n).argtypes = [P, u32, P]
        L.xfem_set_state.argtypes = [P, u32, P, P]
        L.xfem_get_rest_state.argtypes = [P, u32, P, P]
        L.xfem_get_schedule.argtypes = [P, u32, P, P, P, P]
        L.xfem_body_counts.argtypes = [P, u32, P, P]
        L.xfem_compute_rest_state.argtypes = [P, u32, P, u32, f32, P, P, P]
        L.xfem_compute_schedule.argtypes = [P, u32, P, u32, u32, u32, P, P, P, P, P]
        L.xfem_generate_tet_block.argtypes = [u32, u32, u32, f32, f32, f32, u32, f32, P, P]
        L.xfem_adjoint_forward.argtypes = [P, u32, f32, u32, u32, P, P]
        L.xfem_pbd_damping_coefficients.argtypes = [f32, f32, f32, P]
        L.xfem_adjoint_backward.argtypes = [P, P, P, P, P, P, P]
        L.xfem_body_hex_count.argtypes = [P, u32, P]
        L.xfem_get_hex_rest_state.argtypes = [P, u32, P, P]
        L.xfem_get_hex_schedule.argtypes = [P, u32, P, P, P, P]
        L.xfem_compute_hex_rest_state.argtypes = [P, u32, P, u32, f32, P, P, P]
        L.xfem_compute_hex_schedule.argtypes = [P, u32, P, u32, u32, P, P, P, P]
        L.xfem_generate_hex_block.argtypes = [u32, u32, u32, f32, f32, f32, u32, f32, P, P]
        L.xfem_body_t10_count.argtypes = [P, u32, P, P]
        L.xfem_get_t10_rest_state.argtypes = [P, u32, P, P, P, P]
        L.xfem_get_t10_schedule.argtypes = [P, u32, P, P, P, P]
        L.xfem_compute_t10_edges.argtypes = [P, u32, P, P, P]
        L.xfem_compute_t10_rest_state.argtypes = [P, u32, P, u32, f32, P, P, P, P]
        L.xfem_compute_t10_schedule.argtypes = [P, u32, P, u32, u32, P, P, P, P]
        L.xfem_body_h27_count.argtypes = [P, u32, P, P, P]
        L.xfem_get_h27_rest_state.argtypes = [P, u32, P, P, P]
        L.xfem_get_h27_schedule.argtypes = [P, u32, P, P, P, P]
        L.xfem_compute_h27_mesh.argtypes = [P, u32, P, P, P, P, P]
        L.xfem_compute_h27_rest_state.argtypes = [P, u32, P, u32, f32, P, P, P, P]
        L.xfem_compute_h27_schedule.argtypes = [P, u32, P, u32, u32, P, P, P, P]
        L.xfem_get_mixed_tet_schedule.argtypes = [P, u32, P, P, P]
        L.xfem_compute_mixed_rest_state.argtypes = [P, u32, P, u32, f32, P, P, P, P]
        L.xfem_compute_mixed_schedule.argtypes = [P, u32, P, u32, u32, P, P, P, P, P, P, P]
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        raise XfemError(rc, lib().xfem_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_settings(**kw):
    s = Settings()
    _check(lib().xfem_settings_default(C.byref(s)))
    for k, v in kw.items():
        if k in ("gravity", "yeoh", "ground_normal", "locked_right_transform", "origin"):
            getattr(s, k)[:] = [float(x) for x in v]
        else:
            setattr(s, k, v)
    return s


def as_settings(s):
    """A Settings struct from a Settings struct or a dict of its fields."""
    return default_settings(**s) if isinstance(s, dict) else s


def pbd_damping_coefficients(pbd_damping, substep_dt, spacing):
    """(volumeAndTimeCorrectedPbdDamping, its amortized form) for a substep of
    substep_dt and element spacing `spacing` (XPBDFEM/Demo.cpp:53-61)."""
    out = (C.c_float * 2)()
    _check(lib().xfem_pbd_damping_coefficients(pbd_damping, substep_dt, spacing, out))
    return float(out[0]), float(out[1])


def time_corrected_drag(drag, substep_dt):
    """1 - (1 - drag)^(1000 dt), XPBDFEM/Demo.cpp:63."""
    return lib().xfem_time_corrected_drag(drag, substep_dt)


def generate_tet_block(W, H, D, scale=(1.0, 1.0, 1.0), pattern=0, wonkiness=0.0):
    """GenerateTetBlock (XPBDFEM/MeshGen.cpp:223): returns (node_data, idx_data)."""
    nodes = np.zeros(3 * (W + 1) * (H + 1) * (D + 1), np.float32)
    idx = np.zeros(30 * W * H * D, np.uint32)
    _check(lib().xfem_generate_tet_block(W, H, D, scale[0], scale[1], scale[2], pattern, wonkiness,
                                         _p(nodes), _p(idx)))
    return nodes, idx


def generate_hex_block(W, H, D, scale=(1.0, 1.0, 1.0), pattern=0, wonkiness=0.0):
    """GenerateHexBlock (XPBDFEM/MeshGen.cpp:156): returns (node_data, idx_data)."""
    nodes = np.zeros(3 * (W + 1) * (H + 1) * (D + 1), np.float32)
    idx = np.zeros(9 * W * H * D, np.uint32)
    _check(lib().xfem_generate_hex_block(W, H, D, scale[0], scale[1], scale[2], pattern, wonkiness,
                                         _p(nodes), _p(idx)))
    return nodes, idx


def compute_hex_rest_state(node_data, idx_data, density):
    """Host-only rest state of a hex mesh (no GPU): (ep[nh, 120], w[nv], flags[nv])."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nv, nh = nd.size // 3, ix.size // 9
    ep = np.zeros((nh, HEX_EP), np.float32)
    w = np.zeros(nv, np.float32)
    fl = np.zeros(nv, np.uint8)
    _check(lib().xfem_compute_hex_rest_state(_p(nd), nd.size, _p(ix), ix.size, density, _p(ep), _p(w), _p(fl)))
    return ep, w, fl


def compute_hex_schedule(node_data, idx_data, morton=True):
    """Host-only hex schedule (no GPU), in the form of Body.hex_schedule()."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nv, nh = nd.size // 3, ix.size // 9
    rank = np.zeros(nv, np.uint32)
    order = np.zeros(nh, np.uint32)
    cb = np.zeros(nh + 1, np.uint32)
    ncol = C.c_uint32()
    _check(lib().xfem_compute_hex_schedule(_p(nd), nd.size, _p(ix), ix.size, 0 if morton else 1, _p(rank), _p(order),
                                           _p(cb), C.byref(ncol)))
    return dict(vert_rank=rank, hex_order=order, colour_hex_begin=cb[:ncol.value + 1], colours=ncol.value)


def _mixed_counts(idx_data):
    """(tets, hexes) of a tagged stream of tets (tag 4) and hexes (tag 8)."""
    nt = nh = i = 0
    while i < idx_data.size:
        tag = int(idx_data[i])
        nt += tag == 4
        nh += tag == 8
        i += tag + 1
    return nt, nh


def compute_mixed_rest_state(node_data, idx_data, density):
    """Host-only rest state of a mesh mixing tets and hexes (no GPU):
    (ep[nt, 17], hep[nh, 120], w[nv], flags[nv])."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nt, nh = _mixed_counts(ix)
    nv = nd.size // 3
    ep = np.zeros((nt, 17), np.float32)
    hep = np.zeros((nh, HEX_EP), np.float32)
    w = np.zeros(nv, np.float32)
    fl = np.zeros(nv, np.uint8)
    _check(lib().xfem_compute_mixed_rest_state(_p(nd), nd.size, _p(ix), ix.size, density, _p(ep), _p(hep), _p(w),
                                               _p(fl)))
    return ep, hep, w, fl


def compute_mixed_schedule(node_data, idx_data, morton=True):
    """Host-only schedule of a mesh mixing tets and hexes (no GPU): vertex
    ranks, the tets' and the hexes' colourings."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nt, nh = _mixed_counts(ix)
    rank = np.zeros(nd.size // 3, np.uint32)
    to, ho = np.zeros(nt, np.uint32), np.zeros(nh, np.uint32)
    tcb, hcb = np.zeros(nt + 1, np.uint32), np.zeros(nh + 1, np.uint32)
    tn, hn = C.c_uint32(), C.c_uint32()
    _check(lib().xfem_compute_mixed_schedule(_p(nd), nd.size, _p(ix), ix.size, 0 if morton else 1, _p(rank), _p(to),
                                             _p(tcb), C.byref(tn), _p(ho), _p(hcb), C.byref(hn)))
    return dict(vert_rank=rank, tet_order=to, colour_tet_begin=tcb[:tn.value + 1], tet_colours=tn.value,
                hex_order=ho, colour_hex_begin=hcb[:hn.value + 1], hex_colours=hn.value)


def compute_t10_edges(idx_data):
    """Connectivity3d's edges of a tet mesh and GeoQuadratic3d's T10 indices
    (no GPU): (edges[ne, 2], t10[nt, 10])."""
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nt = ix.size // 5
    edges = np.zeros((max(6 * nt, 1), 2), np.uint32)
    t10 = np.zeros((nt, 10), np.uint32)
    ne = C.c_uint32()
    _check(lib().xfem_compute_t10_edges(_p(ix), ix.size, _p(edges), _p(t10), C.byref(ne)))
    return edges[:ne.value].copy(), t10


def compute_t10_rest_state(node_data, idx_data, density):
    """Host-only rest state of a tet mesh read as T10s (no GPU):
    (x[nv, 3] double, ep[nt, 56], w[nv], flags[nv]) over all vertices (the
    mesh's own, then one per edge)."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    edges, t10 = compute_t10_edges(ix)
    nv, nt = nd.size // 3 + edges.shape[0], t10.shape[0]
    x = np.zeros((nv, 3), np.float64)
    ep = np.zeros((nt, T10_EP), np.float32)
    w = np.zeros(nv, np.float32)
    fl = np.zeros(nv, np.uint8)
    _check(lib().xfem_compute_t10_rest_state(_p(nd), nd.size, _p(ix), ix.size, density, _p(x), _p(ep), _p(w),
                                             _p(fl)))
    return x, ep, w, fl


def compute_t10_schedule(node_data, idx_data, morton=True):
    """Host-only T10 schedule (no GPU), in the form of Body.t10_schedule()."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    edges, t10 = compute_t10_edges(ix)
    nv, nt = nd.size // 3 + edges.shape[0], t10.shape[0]
    rank = np.zeros(nv, np.uint32)
    order = np.zeros(nt, np.uint32)
    cb = np.zeros(nt + 1, np.uint32)
    ncol = C.c_uint32()
    _check(lib().xfem_compute_t10_schedule(_p(nd), nd.size, _p(ix), ix.size, 0 if morton else 1, _p(rank), _p(order),
                                           _p(cb), C.byref(ncol)))
    return dict(vert_rank=rank, t10_order=order, colour_t10_begin=cb[:ncol.value + 1], colours=ncol.value)


def compute_h27_mesh(idx_data):
    """Connectivity3d's edges and quads of a hex mesh and GeoQuadratic3d's H27
    indices (no GPU): (edges[ne, 2], quads[nq, 4], h27[nh, 27])."""
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nh = ix.size // 9
    edges = np.zeros((max(12 * nh, 1), 2), np.uint32)
    quads = np.zeros((max(6 * nh, 1), 4), np.uint32)
    h27 = np.zeros((nh, 27), np.uint32)
    ne, nq = C.c_uint32(), C.c_uint32()
    _check(lib().xfem_compute_h27_mesh(_p(ix), ix.size, _p(edges), _p(quads), _p(h27), C.byref(ne), C.byref(nq)))
    return edges[:ne.value].copy(), quads[:nq.value].copy(), h27


def compute_h27_rest_state(node_data, idx_data, density):
    """Host-only rest state of a hex mesh read as H27s (no GPU):
    (x[nv, 3] double, ep[nh, 703], w[nv], flags[nv]) over all vertices."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    edges, quads, h27 = compute_h27_mesh(ix)
    nh = h27.shape[0]
    nv = nd.size // 3 + edges.shape[0] + quads.shape[0] + nh
    x = np.zeros((nv, 3), np.float64)
    ep = np.zeros((nh, H27_EP), np.float32)
    w = np.zeros(nv, np.float32)
    fl = np.zeros(nv, np.uint8)
    _check(lib().xfem_compute_h27_rest_state(_p(nd), nd.size, _p(ix), ix.size, density, _p(x), _p(ep), _p(w),
                                             _p(fl)))
    return x, ep, w, fl


def compute_h27_schedule(node_data, idx_data, morton=True):
    """Host-only H27 schedule (no GPU), in the form of Body.h27_schedule()."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    edges, quads, h27 = compute_h27_mesh(ix)
    nh = h27.shape[0]
    nv = nd.size // 3 + edges.shape[0] + quads.shape[0] + nh
    rank = np.zeros(nv, np.uint32)
    order = np.zeros(nh, np.uint32)
    cb = np.zeros(nh + 1, np.uint32)
    ncol = C.c_uint32()
    _check(lib().xfem_compute_h27_schedule(_p(nd), nd.size, _p(ix), ix.size, 0 if morton else 1, _p(rank), _p(order),
                                           _p(cb), C.byref(ncol)))
    return dict(vert_rank=rank, h27_order=order, colour_h27_begin=cb[:ncol.value + 1], colours=ncol.value)


def compute_rest_state(node_data, idx_data, density):
    """Host-only rest state (no GPU): (ep[nt, 17], w[nv], flags[nv])."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nv, nt = nd.size // 3, ix.size // 5
    ep = np.zeros((nt, 17), np.float32)
    w = np.zeros(nv, np.float32)
    fl = np.zeros(nv, np.uint8)
    _check(lib().xfem_compute_rest_state(_p(nd), nd.size, _p(ix), ix.size, density, _p(ep), _p(w), _p(fl)))
    return ep, w, fl


def compute_schedule(node_data, idx_data, cluster_mode=0, morton=True):
    """Host-only schedule (no GPU), in the form of Body.schedule()."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nv, nt = nd.size // 3, ix.size // 5
    rank = np.zeros(nv, np.uint32)
    order = np.zeros(nt, np.uint32)
    cb = np.zeros(nt + 1, np.uint32)
    ncol, ncl = C.c_uint32(), C.c_uint32()
    _check(lib().xfem_compute_schedule(_p(nd), nd.size, _p(ix), ix.size, cluster_mode, 0 if morton else 1,
                                       _p(rank), _p(order), _p(cb), C.byref(ncol), C.byref(ncl)))
    return dict(vert_rank=rank, tet_order=order, colour_tet_begin=cb[:ncol.value + 1], colours=ncol.value,
                clusters=ncl.value)


def compute_ring_schedule(node_data, idx_data, morton=True):
    """Host-only ring schedule of the continuous-pressure models (no GPU)."""
    nd = np.ascontiguousarray(node_data, np.float32).reshape(-1)
    ix = np.ascontiguousarray(idx_data, np.uint32).reshape(-1)
    nv = nd.size // 3
    order = np.zeros(nv, np.uint32)
    cb = np.zeros(nv + 1, np.uint32)
    ncol = C.c_uint32()
    _check(lib().xfem_compute_ring_schedule(_p(nd), nd.size, _p(ix), ix.size, 0 if morton else 1, _p(order), _p(cb),
                                            C.byref(ncol)))
    return dict(vert_order=order, colour_vert_begin=cb[:ncol.value + 1], colours=ncol.value)


def _options(cluster_mode=0, morton=True, sync_mode=0, block_size=0, keep_lambdas=False, device=0, stream=None,
             host_setup=False, wait_timeout_ms=0, bricks=0):
    o = Options()
    o.cluster_mode, o.no_morton, o.sync_mode = cluster_mode, 0 if morton else 1, sync_mode
    o.block_size, o.keep_lambdas, o.device, o.stream = block_size, 1 if keep_lambdas else 0, device, stream
    o.host_setup = 1 if host_setup else 0
    o.wait_timeout_ms = wait_timeout_ms
    o.bricks = bricks
    return o


def test_hook(body, hook, value):
    """xfem_test_hook: make a detected failure happen on purpose (HOOK_*);
    body is a Body, or None for the process-wide HOOK_FAIL_ALLOC."""
    _check(lib().xfem_test_hook(body._h if body is not None else None, hook, value))


class Body:
    """One handle: a single body (GeoLinear3d) or a batch of bodies."""

    def __init__(self, node_data=None, idx_data=None, density=1000.0, settings=None, meshes=None, **opts):
        self._h = C.c_void_p()
        self._opts = _options(**opts)
        if meshes is None:
            meshes = [(node_data, idx_data, density)]
            settings = [settings] if settings is not None else None
        self._keep = []
        arr = (Mesh * len(meshes))()
        for i, (nd, ix, dens) in enumerate(meshes):
            nd = np.ascontiguousarray(nd, np.float32).reshape(-1)
            ix = np.ascontiguousarray(ix, np.uint32).reshape(-1)
            self._keep += [nd, ix]
            arr[i] = Mesh(_p(nd), nd.size, _p(ix), ix.size, float(dens))
        sarr = None
        if settings is not None:
            sarr = (Settings * len(meshes))(*[as_settings(s) if s is not None else default_settings()
                                               for s in settings])
        _check(lib().xfem_batch_create(len(meshes), arr, sarr, C.byref(self._opts), C.byref(self._h)))
        self._keep = []
        self.nbodies = len(meshes)
        self.counts = []
        for b in range(self.nbodies):
            nv, nt = C.c_uint32(), C.c_uint32()
            _check(lib().xfem_body_counts(self._h, b, C.byref(nv), C.byref(nt)))
            self.counts.append((nv.value, nt.value))

    # -- lifecycle
    def close(self):
        if self._h:
            lib().xfem_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        i = Info()
        _check(lib().xfem_get_info(self._h, C.byref(i)))
        return {n: getattr(i, n) for n, _ in Info._fields_}

    # -- parameters
    def set_settings(self, s, body=0):
        _check(lib().xfem_set_settings(self._h, body, C.byref(as_settings(s))))

    def set_lock_mask(self, mask, body=0):
        m = np.ascontiguousarray(mask, np.uint8)
        _check(lib().xfem_set_lock_mask(self._h, body, _p(m)))

    def set_tet_mu(self, mu, body=0):
        m = None if mu is None else np.ascontiguousarray(mu, np.float32)
        _check(lib().xfem_set_tet_mu(self._h, body, _p(m)))

    # -- stepping
    def substep(self, dt):
        _check(lib().xfem_substep(self._h, dt))

    def step_frames(self, frames, substeps, dt):
        _check(lib().xfem_step_frames(self._h, frames, substeps, dt))

    def step_frames_noalloc(self, frames, substeps, dt):
        """xfem_step_frames_noalloc: the same stepping without any device
        allocation (see include/xfem.h)."""
        _check(lib().xfem_step_frames_noalloc(self._h, frames, substeps, dt))

    def synchronize(self):
        _check(lib().xfem_synchronize(self._h))

    # -- state
    def _get(self, fn, body, width, dtype=np.float32, out=None):
        nv = self.counts[body][0]
        if out is None:
            out = np.zeros(nv * width, dtype)
        elif out.dtype != dtype or out.size != nv * width or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous %s array of %d values" % (np.dtype(dtype).name, nv * width))
        _check(fn(self._h, body, _p(out)))
        return out.reshape(nv, width) if width > 1 else out

    def positions(self, body=0, out=None):
        """Positions in caller vertex order; `out` (optional): a caller array
        of 3 * vertices floats to read into (for instance pinned memory)."""
        return self._get(lib().xfem_get_positions, body, 3, out=out)

    def velocities(self, body=0, out=None):
        return self._get(lib().xfem_get_velocities, body, 3, out=out)

    def inverse_masses(self, body=0):
        return self._get(lib().xfem_get_inverse_masses, body, 1)

    def contacts(self, body=0):
        return self._get(lib().xfem_get_contacts, body, 1, np.uint8)

    def set_positions(self, x, body=0):
        a = np.ascontiguousarray(x, np.float32).reshape(-1)
        _check(lib().xfem_set_positions(self._h, body, _p(a)))

    def set_velocities(self, v, body=0):
        a = np.ascontiguousarray(v, np.float32).reshape(-1)
        _check(lib().xfem_set_velocities(self._h, body, _p(a)))

    def set_state(self, x, v, body=0):
        """Positions and velocities with one synchronisation."""
        a = np.ascontiguousarray(x, np.float32).reshape(-1)
        c = np.ascontiguousarray(v, np.float32).reshape(-1)
        _check(lib().xfem_set_state(self._h, body, _p(a), _p(c)))

    def lambdas(self, body=0):
        nt = self.counts[body][1]
        out = np.zeros(2 * nt, np.float32)
        _check(lib().xfem_get_lambdas(self._h, body, _p(out)))
        return out.reshape(nt, 2)

    def volume(self, body=0):
        v = C.c_double()
        _check(lib().xfem_calculate_volume(self._h, body, C.byref(v)))
        return v.value

    def rest_state(self, body=0):
        nv, nt = self.counts[body]
        ep = np.zeros((nt, 17), np.float32)
        w = np.zeros(nv, np.float32)
        _check(lib().xfem_get_rest_state(self._h, body, _p(ep), _p(w)))
        return ep, w

    def schedule(self, body=0):
        nv, nt = self.counts[body]
        rank = np.zeros(nv, np.uint32)
        order = np.zeros(nt, np.uint32)
        ncol = C.c_uint32()
        _check(lib().xfem_get_schedule(self._h, body, None, None, None, C.byref(ncol)))
        cb = np.zeros(ncol.value + 1, np.uint32)
        _check(lib().xfem_get_schedule(self._h, body, _p(rank), _p(order), _p(cb), C.byref(ncol)))
        return dict(vert_rank=rank, tet_order=order, colour_tet_begin=cb, colours=ncol.value)

    def hex_count(self, body=0):
        n = C.c_uint32()
        _check(lib().xfem_body_hex_count(self._h, body, C.byref(n)))
        return n.value

    def hex_rest_state(self, body=0):
        """Rest state of a hex body: (ep[nh, 120], w[nv])."""
        nv, nh = self.counts[body][0], self.hex_count(body)
        ep = np.zeros((nh, HEX_EP), np.float32)
        w = np.zeros(nv, np.float32)
        _check(lib().xfem_get_hex_rest_state(self._h, body, _p(ep), _p(w)))
        return ep, w

    def hex_schedule(self, body=0):
        """Vertex ranks, hex order (colour-major) and colour offsets of a hex body."""
        nv, nh = self.counts[body][0], self.hex_count(body)
        rank = np.zeros(nv, np.uint32)
        order = np.zeros(nh, np.uint32)
        cb = np.zeros(nh + 1, np.uint32)
        ncol = C.c_uint32()
        _check(lib().xfem_get_hex_schedule(self._h, body, _p(rank), _p(order), _p(cb), C.byref(ncol)))
        return dict(vert_rank=rank, hex_order=order, colour_hex_begin=cb[:ncol.value + 1], colours=ncol.value)

    def mixed_tet_schedule(self, body=0):
        """The tets' own colouring of a mesh mixing tets and hexes: tet order
        (colour-major, caller ids) and colour offsets."""
        nt = self.counts[body][1]
        order = np.zeros(nt, np.uint32)
        cb = np.zeros(nt + 1, np.uint32)
        ncol = C.c_uint32()
        _check(lib().xfem_get_mixed_tet_schedule(self._h, body, _p(order), _p(cb), C.byref(ncol)))
        return dict(tet_order=order, colour_tet_begin=cb[:ncol.value + 1], colours=ncol.value)

    def h27_count(self, body=0):
        """(H27s, edge nodes, face nodes) of an H27 body."""
        n, ne, nq = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(lib().xfem_body_h27_count(self._h, body, C.byref(n), C.byref(ne), C.byref(nq)))
        return n.value, ne.value, nq.value

    def h27_rest_state(self, body=0):
        """Rest state of an H27 body: (ep[nh, 703], w[nv], h27[nh, 27])."""
        nv = self.counts[body][0]
        nh = self.h27_count(body)[0]
        ep = np.zeros((nh, H27_EP), np.float32)
        w = np.zeros(nv, np.float32)
        h27 = np.zeros((nh, 27), np.uint32)
        _check(lib().xfem_get_h27_rest_state(self._h, body, _p(ep), _p(w), _p(h27)))
        return ep, w, h27

    def h27_schedule(self, body=0):
        """Vertex ranks, H27 order (colour-major) and colour offsets of an H27 body."""
        nv = self.counts[body][0]
        nh = self.h27_count(body)[0]
        rank = np.zeros(nv, np.uint32)
        order = np.zeros(nh, np.uint32)
        cb = np.zeros(nh + 1, np.uint32)
        ncol = C.c_uint32()
        _check(lib().xfem_get_h27_schedule(self._h, body, _p(rank), _p(order), _p(cb), C.byref(ncol)))
        return dict(vert_rank=rank, h27_order=order, colour_h27_begin=cb[:ncol.value + 1], colours=ncol.value)

    def t10_count(self, body=0):
        """(T10s, edge nodes) of a T10 body."""
        n, ne = C.c_uint32(), C.c_uint32()
        _check(lib().xfem_body_t10_count(self._h, body, C.byref(n), C.byref(ne)))
        return n.value, ne.value

    def t10_rest_state(self, body=0):
        """Rest state of a T10 body: (ep[nt, 56], w[nv], t10[nt, 10], edges[ne, 2])."""
        nv = self.counts[body][0]
        nt, ne = self.t10_count(body)
        ep = np.zeros((nt, T10_EP), np.float32)
        w = np.zeros(nv, np.float32)
        t10 = np.zeros((nt, 10), np.uint32)
        edges = np.zeros((ne, 2), np.uint32)
        _check(lib().xfem_get_t10_rest_state(self._h, body, _p(ep), _p(w), _p(t10), _p(edges)))
        return ep, w, t10, edges

    def t10_schedule(self, body=0):
        """Vertex ranks, T10 order (colour-major) and colour offsets of a T10 body."""
        nv = self.counts[body][0]
        nt, _ = self.t10_count(body)
        rank = np.zeros(nv, np.uint32)
        order = np.zeros(nt, np.uint32)
        cb = np.zeros(nt + 1, np.uint32)
        ncol = C.c_uint32()
        _check(lib().xfem_get_t10_schedule(self._h, body, _p(rank), _p(order), _p(cb), C.byref(ncol)))
        return dict(vert_rank=rank, t10_order=order, colour_t10_begin=cb[:ncol.value + 1], colours=ncol.value)

    def ring_schedule(self, body=0):
        """The ring order of a continuous-pressure body (energy 8-10)."""
        nv, nt = self.counts[body]
        order = np.zeros(nv, np.uint32)
        cb = np.zeros(nv + 1, np.uint32)
        ncol = C.c_uint32()
        _check(lib().xfem_get_ring_schedule(self._h, body, _p(order), _p(cb), C.byref(ncol)))
        # a T10 or H27 body rings its mesh vertices only, not the added nodes
        return dict(vert_order=order[:cb[ncol.value]], colour_vert_begin=cb[:ncol.value + 1], colours=ncol.value)

    # -- reverse-mode adjoint (no reference counterpart; see include/xfem.h)
    def total_counts(self):
        """Vertices and tets of the whole handle (concatenated caller order)."""
        return sum(c[0] for c in self.counts), sum(c[1] for c in self.counts)

    def adjoint_forward(self, substeps, dt, tips, checkpoint_every=0):
        """Steps `substeps` substeps recording the tape; returns the tip
        trajectory, shape (substeps, len(tips), 3)."""
        t = np.ascontiguousarray(tips, np.uint32).reshape(-1)
        traj = np.zeros((substeps, t.size, 3), np.float32)
        _check(lib().xfem_adjoint_forward(self._h, substeps, dt, checkpoint_every, t.size, _p(t), _p(traj)))
        return traj

    def adjoint_backward(self, grad_traj, grad_x=None, grad_v=None):
        """Reverse pass of the last adjoint_forward. Returns (dL/dmu per tet,
        dL/dX0, dL/dV0) in the handle's concatenated caller order."""
        nv, nt = self.total_counts()
        g = np.ascontiguousarray(grad_traj, np.float32).reshape(-1)
        gx = None if grad_x is None else np.ascontiguousarray(grad_x, np.float32).reshape(-1)
        gv = None if grad_v is None else np.ascontiguousarray(grad_v, np.float32).reshape(-1)
        dmu = np.zeros(nt, np.float32)
        dx = np.zeros((nv, 3), np.float32)
        dv = np.zeros((nv, 3), np.float32)
        _check(lib().xfem_adjoint_backward(self._h, _p(g), _p(gx), _p(gv), _p(dmu), _p(dx), _p(dv)))
        return dmu, dx, dv
