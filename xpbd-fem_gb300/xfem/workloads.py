"""Seeded synthetic workloads: the cantilever, drop, throughput, batched and
differentiation configurations, built from GenerateTetBlock meshes
(XPBDFEM/MeshGen.cpp:223) with the project's own generator (splitmix64 with
Box-Muller; no library distribution is used, so values are identical on every
machine). Pure numpy: nothing here loads libxfem.so, so the CPU reference arm
of the benchmark can build the same inputs. Settings are plain dicts of
xfem_settings fields (xfem.default_settings(**d) turns one into the struct).

Material mapping to the reference's parameters (XPBDFEM/Fem.cpp:445-449):
  Neo-Hookean  mu = E / (2 (1 + nu)), mu_ref = mu / 2, compliance = 1 / mu_ref
               = 4 (1 + nu) / E;
  Yeoh         W = C10 I + C20 I^2 + C30 I^3 with I = I1 - 3 becomes
               compliance = 1 / C10 and multipliers (1, C20 / C10, C30 / C10).
"""
import math

import numpy as np

ENERGY_BIT, ENERGY_MIXED_SEL, ENERGY_YEOH_SKIN_FAST, XPBD_SOLVE_BIT = 6, 4, 7, 11
LOCK_LEFT = 1 << 26

NH_FLAGS = (ENERGY_MIXED_SEL << ENERGY_BIT) | (1 << XPBD_SOLVE_BIT) | LOCK_LEFT
YEOH_FLAGS = (ENERGY_YEOH_SKIN_FAST << ENERGY_BIT) | (1 << XPBD_SOLVE_BIT) | LOCK_LEFT



def default_settings(**kw):
    """A settings dict (the fields the solver reads; the rest keep the
    defaults of xfem_settings_default)."""
    d = dict(gravity=(0.0, -9.81, 0.0), compliance=0.01, poissons_ratio=0.45,
             flags=(ENERGY_MIXED_SEL << ENERGY_BIT) | (1 << XPBD_SOLVE_BIT), time_corrected_drag=0.0,
             yeoh=(0.1095, 14.95, 4.595), ground=0, ground_normal=(0.0, 0.0, 1.0), ground_offset=0.0, friction=0.0)
    d.update(kw)
    return d


_SPLIT = np.array([[0, 1, 5, 7], [0, 7, 3, 1], [0, 2, 3, 7], [0, 7, 6, 2], [0, 4, 6, 7], [0, 7, 5, 4]])


def hex_block(W, H, D, scale):
    """GenerateHexBlock (XPBDFEM/MeshGen.cpp:156-221) with the uniform pattern
    and no wonkiness, in float32 arithmetic: node_data, idx_data (tag 8)."""
    sc = np.asarray(scale, np.float32)
    mn = sc * np.array([-0.5 * W, -0.5 * H, -0.5 * D], np.float32)
    z, y, x = np.meshgrid(np.arange(D + 1), np.arange(H + 1), np.arange(W + 1), indexing="ij")
    c = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float32)
    nodes = (mn + sc * c).astype(np.float32).reshape(-1)
    cz, cy, cx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    base = (cx + cy * (W + 1) + cz * (W + 1) * (H + 1)).reshape(-1)
    corner = np.array([i + j * (W + 1) + k * (W + 1) * (H + 1) for k in (0, 1) for j in (0, 1) for i in (0, 1)])
    hexes = base[:, None] + corner[None, :]
    idx = np.concatenate([np.full((hexes.shape[0], 1), 8), hexes], 1).astype(np.uint32).reshape(-1)
    return nodes, idx


def tet_block(W, H, D, scale):
    """GenerateTetBlock (XPBDFEM/MeshGen.cpp:156-244) with the uniform pattern
    and no wonkiness, in float32 arithmetic: node_data, idx_data."""
    sc = np.asarray(scale, np.float32)
    mn = sc * np.array([-0.5 * W, -0.5 * H, -0.5 * D], np.float32)
    z, y, x = np.meshgrid(np.arange(D + 1), np.arange(H + 1), np.arange(W + 1), indexing="ij")
    c = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float32)
    nodes = (mn + sc * c).astype(np.float32).reshape(-1)
    cz, cy, cx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    base = (cx + cy * (W + 1) + cz * (W + 1) * (H + 1)).reshape(-1)
    corner = np.array([i + j * (W + 1) + k * (W + 1) * (H + 1) for k in (0, 1) for j in (0, 1) for i in (0, 1)])
    hexes = base[:, None] + corner[None, :]
    tets = hexes[:, _SPLIT].reshape(-1, 4)
    idx = np.concatenate([np.full((tets.shape[0], 1), 4), tets], 1).astype(np.uint32).reshape(-1)
    return nodes, idx


class Rng:
    """splitmix64 stream; uniform() in [0, 1) with 53 bits, normal() by Box-Muller."""

    def __init__(self, seed):
        self.state = np.uint64(seed)

    def _next(self, n):
        with np.errstate(over="ignore"):
            i = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + i * np.uint64(0x9E3779B97F4A7C15)
            self.state = self.state + np.uint64(n) * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            return z ^ (z >> np.uint64(31))

    def uniform(self, n):
        return (self._next(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def integers(self, lo, hi, n):
        """Uniform integers in [lo, hi] inclusive."""
        return lo + (self._next(n) % np.uint64(hi - lo + 1)).astype(np.int64)

    def normal(self, n):
        m = (n + 1) // 2
        u1 = 1.0 - self.uniform(m)  # (0, 1]
        u2 = self.uniform(m)
        r = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
        return z[:n]


def nh_compliance(E, nu=0.5):
    return 4.0 * (1.0 + nu) / E


def random_rotation(rng):
    """Uniform random rotation (Shoemake's quaternion method) as a 3x3 matrix."""
    u1, u2, u3 = rng.uniform(3)
    a, b = math.sqrt(1 - u1), math.sqrt(u1)
    x, y, z, w = a * math.sin(2 * math.pi * u2), a * math.cos(2 * math.pi * u2), b * math.sin(2 * math.pi * u3), \
        b * math.cos(2 * math.pi * u3)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def box(W, H, D, edge):
    return tet_block(W, H, D, (edge, edge, edge))


def lock_mask_axis(nodes, axis, frac=0.02):
    """Vertices within `frac` of the minimum along `axis` (the reference's Left
    rule, XPBDFEM/Geo.cpp:724, on any axis)."""
    x = nodes.reshape(-1, 3)[:, axis].astype(np.float32)
    lo, hi = x.min(), x.max()
    return ((x - lo) / (hi - lo) < np.float32(frac)).astype(np.uint8)


def cantilever_small():
    """8x2x2 cubes of 0.1 m (192 tets, 81 nodes), Neo-Hookean E = 1e5 Pa,
    nu = 0.5, density 1000, gravity -9.81 z, x = 0 face fixed, dt = 1/60 s
    with 20 substeps, 100 frames, no collision."""
    nodes, idx = box(8, 2, 2, 0.1)
    n = nodes.reshape(-1, 3)
    n[:, 0] -= n[:, 0].min()
    s = default_settings(gravity=(0.0, 0.0, -9.81), compliance=nh_compliance(1e5), poissons_ratio=0.5,
                         flags=NH_FLAGS)
    return dict(name="cantilever 8x2x2 (192 tets) Neo-Hookean", nodes=nodes, idx=idx, density=1000.0,
                settings=s, lock=lock_mask_axis(nodes, 0), dt=1.0 / 60.0, substeps=20, frames=100)


def drop_yeoh(seed=2, W=64, H=16, D=16, height=0.5, nu=0.5):
    """64x16x16 cubes of 0.02 m (98,304 tets), Yeoh C10 = 3e4, C20 = 1e3,
    C30 = 1e2 Pa, incompressible, dropped from 0.5 m with a random rotation
    onto z = 0 with Coulomb friction 0.4; dt = 1/60, 30 substeps, 300 frames.
    W, H, D, height and nu give scaled copies (same cube edge, coefficients,
    rotation draw and ground) for tests whose oracle must finish in seconds."""
    rng = Rng(seed)
    nodes, idx = box(W, H, D, 0.02)
    n = nodes.reshape(-1, 3).astype(np.float64)
    n = (n - n.mean(0)) @ random_rotation(rng).T
    n[:, 2] += height - n[:, 2].min()
    nodes = n.astype(np.float32).reshape(-1)
    C10, C20, C30 = 3e4, 1e3, 1e2
    s = default_settings(gravity=(0.0, 0.0, -9.81), compliance=1.0 / C10, poissons_ratio=nu,
                         flags=YEOH_FLAGS & ~LOCK_LEFT, yeoh=(1.0, C20 / C10, C30 / C10), ground=1,
                         ground_normal=(0.0, 0.0, 1.0), ground_offset=0.0, friction=0.4)
    return dict(name=f"drop {W}x{H}x{D} ({6 * W * H * D} tets) Yeoh", nodes=nodes, idx=idx, density=1000.0,
                settings=s, lock=None, dt=1.0 / 60.0, substeps=30, frames=300)


def throughput(seed=3, W=128, H=64, D=32):
    """128x64x32 cubes (1,572,864 tets, 276,705 nodes) of 0.1 m, Neo-Hookean
    E = 5e5 Pa incompressible, nodes jittered by N(0, (0.05 edge)^2), bottom
    face fixed, gravity, dt = 1/60 with 20 substeps, 50 frames."""
    rng = Rng(seed)
    edge = 0.1
    nodes, idx = box(W, H, D, edge)
    nodes = (nodes + (0.05 * edge) * rng.normal(nodes.size)).astype(np.float32)
    s = default_settings(gravity=(0.0, 0.0, -9.81), compliance=nh_compliance(5e5), poissons_ratio=0.5,
                         flags=NH_FLAGS)
    return dict(name=f"throughput {W}x{H}x{D} ({6 * W * H * D} tets) Neo-Hookean", nodes=nodes, idx=idx,
                density=1000.0, settings=s, lock=lock_mask_axis(nodes, 2), dt=1.0 / 60.0, substeps=20, frames=50)


def throughput_hex(seed=3, W=128, H=64, D=32):
    """The throughput configuration's grid as linear hexahedra: 128x64x32
    hexes (262,144 hexes on the same 276,705 jittered nodes), Neo-Hookean
    (MixedSel) E = 5e5 Pa incompressible, bottom face fixed, gravity, dt =
    1/60 with 20 substeps."""
    rng = Rng(seed)
    edge = 0.1
    nodes, idx = hex_block(W, H, D, (edge, edge, edge))
    nodes = (nodes + (0.05 * edge) * rng.normal(nodes.size)).astype(np.float32)
    s = default_settings(gravity=(0.0, 0.0, -9.81), compliance=nh_compliance(5e5), poissons_ratio=0.5,
                         flags=NH_FLAGS)
    return dict(name=f"throughput hexes {W}x{H}x{D} ({W * H * D} hexes) Neo-Hookean", nodes=nodes, idx=idx,
                density=1000.0, settings=s, lock=lock_mask_axis(nodes, 2), dt=1.0 / 60.0, substeps=20, frames=50)


def batched(seed=4, nbodies=512, lo=2, hi=24, height=0.5, nu=0.5):
    """nbodies boxes of a x b x c cubes, a, b, c ~ U{lo..hi}, coin-flip
    Neo-Hookean / Yeoh, E ~ LogUniform(1e4, 1e6) Pa, each dropped from 0.5 m
    with a random rotation onto its own ground (z = 0, friction 0.4),
    20 substeps per frame of 1/60 s. height and nu give variants for tests
    (bodies that reach the ground within a frame; a compressible material)."""
    rng = Rng(seed)
    dims = rng.integers(lo, hi, 3 * nbodies).reshape(nbodies, 3)
    coins = rng.uniform(nbodies)
    logE = np.log(1e4) + (np.log(1e6) - np.log(1e4)) * rng.uniform(nbodies)
    meshes, settings = [], []
    edge = 0.02
    for b in range(nbodies):
        a_, b_, c_ = (int(v) for v in dims[b])
        nodes, idx = box(a_, b_, c_, edge)
        n = nodes.reshape(-1, 3).astype(np.float64)
        n = (n - n.mean(0)) @ random_rotation(rng).T
        n[:, 2] += height - n[:, 2].min()
        nodes = n.astype(np.float32).reshape(-1)
        E = float(np.exp(logE[b]))
        if coins[b] < 0.5:
            s = default_settings(gravity=(0, 0, -9.81), compliance=nh_compliance(E, nu), poissons_ratio=nu,
                                 flags=NH_FLAGS & ~LOCK_LEFT, ground=1, ground_normal=(0, 0, 1), friction=0.4)
        else:
            # Yeoh: C10 = E / 6 (the Neo-Hookean limit) and the reference's own
            # coefficient ratios (XPBDFEM/Fem.cpp:526) for C20 / C10, C30 / C10
            s = default_settings(gravity=(0, 0, -9.81), compliance=nh_compliance(E, nu), poissons_ratio=nu,
                                 flags=YEOH_FLAGS & ~LOCK_LEFT, ground=1, ground_normal=(0, 0, 1), friction=0.4,
                                 yeoh=(1.0, 14.95 / 0.1095, 4.595 / 0.1095))
        meshes.append((nodes, idx, 1000.0))
        settings.append(s)
    return dict(name=f"batched {nbodies} bodies", meshes=meshes, settings=settings, dt=1.0 / 60.0, substeps=20,
                frames=1, dims=dims)


def adjoint_beam(seed=5, W=32, H=8, D=8, nsub=200, ntips=20, nu=0.45):
    """Differentiation workload: a 32x8x8-cube beam (12,288 tets, 2,673
    nodes) of 0.025 m cubes, x = min face fixed, gravity -z, Neo-Hookean with
    nu = 0.45 (compressible, so the coupled solve is well conditioned and the
    derivative is smooth) and a per-tet Young's modulus log E ~ N(log 1e5,
    0.3^2). 20 tip nodes spread over the free end face; the target
    trajectory is that of the same beam under a second field drawn from the
    same distribution. 200 substeps of 1/1200 s. Returns the two per-tet mu
    fields (the reference's mu = 1/compliance = E / (4 (1 + nu)))."""
    rng = Rng(seed)
    nodes, idx = box(W, H, D, 0.025)
    n = nodes.reshape(-1, 3)
    n[:, 0] -= n[:, 0].min()
    nt = 6 * W * H * D
    mu = np.exp(math.log(1e5) + 0.3 * rng.normal(nt)) / (4.0 * (1.0 + nu))
    mu_target = np.exp(math.log(1e5) + 0.3 * rng.normal(nt)) / (4.0 * (1.0 + nu))
    face = np.nonzero(n[:, 0] == n[:, 0].max())[0]
    tips = face[np.linspace(0, face.size - 1, ntips).round().astype(np.int64)].astype(np.uint32)
    s = default_settings(gravity=(0.0, 0.0, -9.81), compliance=nh_compliance(1e5, nu), poissons_ratio=nu,
                         flags=NH_FLAGS)
    return dict(name=f"adjoint beam {W}x{H}x{D} ({nt} tets)", nodes=nodes, idx=idx, density=1000.0, settings=s,
                lock=lock_mask_axis(nodes, 0), mu=mu.astype(np.float32), mu_target=mu_target.astype(np.float32),
                tips=tips, dt=1.0 / 1200.0, substeps=nsub)
