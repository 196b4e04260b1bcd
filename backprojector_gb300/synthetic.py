"""Seeded synthetic NLOS captures for the five benchmark configurations.

The reference reconstructs captures of the Zaragoza NLOS dataset (HDF5); that dataset is
not available here, so seeded synthetic scenes with the configurations' shapes stand in
for it.  Scenes are point scatterers and surface samples of spheres, boxes and tori,
rendered per (laser, SPAD) pair with 1/r^2 per leg (bpgb_synth_render) and optional
Poisson noise.  Geometry shared by all configurations:

* relay wall: the plane y = 0, grids on it span x and z, row-major [gx, gy, 3] with
  grid[i, j] = (x_i, 0, z_j), x_i and z_j from linspace(-size/2, size/2, n);
* laser origin (0, -0.5, -0.4) m and SPAD origin (0, -0.5, 0.4) m (given for the
  exhaustive configuration and used for all), so every pair carries both wall legs;
* hidden volumes lie behind the wall (y > 0);
* t0 = floor(min path / deltaT) * deltaT, the shortest laser-volume-SPAD path rounded
  down to a bin (the exhaustive configuration's literal t0 = 0 puts every path outside
  its 1.536 m window);
* "V over X m^3" volumes are cubes of edge X m.

Seeds: capture seed s drives the scene, s + 2 the Poisson noise.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi

LASER_ORIGIN = (0.0, -0.5, -0.4)
SPAD_ORIGIN = (0.0, -0.5, 0.4)


@dataclass
class CaptureSpec:
    name: str
    laser_grid: tuple[int, int] | None   # None: one laser point at the wall centre
    spad_grid: tuple[int, int]
    wall_size: float
    T: int
    deltaT: float
    volume_position: tuple[float, float, float]
    volume_edge: float
    voxels: int
    scene: str                           # "points", "points+sphere", "objects"
    scene_params: dict = field(default_factory=dict)
    noise_peak: float | None = None
    wavelength_spacings: float | None = None  # phasor wavelength in SPAD spacings
    confocal: bool = False


SPECS: dict[str, CaptureSpec] = {
    # Plain dense FP32, exhaustive 16x16 lasers x 16x16 SPADs on a 1 x 1 m wall.
    "dense_exhaustive_16": CaptureSpec(
        "dense_exhaustive_16", (16, 16), (16, 16), 1.0, 512, 0.003, (0.0, 0.6, 0.0), 0.5, 32,
        "points", {"n": 8, "albedo": (0.2, 1.0)}, noise_peak=1e4),
    # Precision study: one laser, 64x64 SPADs over 2 x 2 m, 64^3 over 1 m^3 1 m behind.
    "precision_64": CaptureSpec(
        "precision_64", None, (64, 64), 2.0, 2048, 0.001, (0.0, 1.0, 0.0), 1.0, 64,
        "points+sphere", {"n": 32, "sphere_diameter": 0.3, "sphere_points": 2000,
                          "albedo": (0.2, 1.0)}, noise_peak=1e4),
    # Phasor field, complex64: one laser, 128x128 SPADs, 128^3 over 1.5 m^3.
    "phasor_128": CaptureSpec(
        "phasor_128", None, (128, 128), 2.0, 4096, 0.0005, (0.0, 1.0, 0.0), 1.5, 128,
        "objects", {"count": (3, 3), "kinds": ("box", "sphere"), "points": 5000,
                    "albedo": (0.3, 1.0)}, wavelength_spacings=4.0),
    # Learned-octree target: one laser, 128x128 SPADs, T = 4096, 256^3 over 1.5 m^3.
    # deltaT is not given; 1.5 mm makes T * deltaT = 6.1 m cover every path (1.8-7.5 m).
    "octree_256": CaptureSpec(
        "octree_256", None, (128, 128), 2.0, 4096, 0.0015, (0.0, 1.0, 0.0), 1.5, 256,
        "objects", {"count": (1, 5), "kinds": ("sphere", "box", "torus"), "points": 10000,
                    "albedo": (0.3, 1.0)}),
}

# Reduced shapes of the same configurations (tests and quick runs).
SMALL = {
    "dense_exhaustive_16": dict(laser_grid=(4, 4), spad_grid=(8, 8), T=512, voxels=16),
    "precision_64": dict(spad_grid=(16, 16), T=1024, voxels=24),
    "phasor_128": dict(spad_grid=(16, 16), T=1024, deltaT=0.002, voxels=20),
    "octree_256": dict(spad_grid=(16, 16), T=1024, deltaT=0.006, voxels=32),
}


@dataclass
class Capture:
    spec: CaptureSpec
    seed: int
    H: np.ndarray                # [P, T] float32, pair-major
    pairs: np.ndarray            # PAIR_DTYPE [P]
    laser_grid: np.ndarray       # [lx, ly, 3]
    camera_grid: np.ndarray      # [cx, cy, 3]
    laser_position: np.ndarray
    camera_position: np.ndarray
    t0: float
    deltaT: float
    volume_position: np.ndarray
    volume_size: np.ndarray
    voxels_per_side: np.ndarray  # uint32 [3]
    zero: np.ndarray             # volume_zero_pos
    inc: np.ndarray              # voxel_inc [9]
    points: np.ndarray
    albedo: np.ndarray
    wavelength: float | None

    @property
    def T(self) -> int:
        return int(self.H.shape[-1])

    @property
    def P(self) -> int:
        return len(self.pairs)

    @property
    def nvox(self) -> int:
        return int(np.prod(self.voxels_per_side.astype(np.int64)))

    @property
    def updates(self) -> int:
        return self.nvox * self.P

    def transient_array(self) -> np.ndarray:
        """H reshaped as the reference's row-major capture array."""
        cx, cy = self.camera_grid.shape[:2]
        if self.spec.confocal:
            return self.H.reshape(cx, cy, self.T)
        lx, ly = self.laser_grid.shape[:2]
        return self.H.reshape(lx, ly, cx, cy, self.T)


def wall_grid(n: tuple[int, int], size: float) -> np.ndarray:
    xs = np.linspace(-size / 2, size / 2, n[0], dtype=np.float64)
    zs = np.linspace(-size / 2, size / 2, n[1], dtype=np.float64)
    g = np.zeros((n[0], n[1], 3), np.float32)
    g[:, :, 0] = xs[:, None]
    g[:, :, 2] = zs[None, :]
    return g


def _leg(o: np.ndarray, pts: np.ndarray) -> np.ndarray:
    """|o - p| with an FP32 difference and FP64 squares (the reference's bp::distance)."""
    d = (o[None, :].astype(np.float32) - pts.astype(np.float32)).astype(np.float64)
    return np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).astype(np.float32)


def make_pairs(laser_position, laser_grid, camera_position, camera_grid, confocal=False) -> np.ndarray:
    """Pair list in precompute_distances order (backproject.hpp:374-413), numpy."""
    cg = camera_grid.reshape(-1, 3).astype(np.float32)
    cw = _leg(np.asarray(camera_position, np.float32), cg)
    if confocal:
        out = np.zeros(len(cg), capi.PAIR_DTYPE)
        out["camera_point"] = cg
        out["laser_point"] = cg
        out["camera_wall"] = cw
        out["laser_wall"] = cw
        return out
    lg = laser_grid.reshape(-1, 3).astype(np.float32)
    lw = _leg(np.asarray(laser_position, np.float32), lg)
    L, S = len(lg), len(cg)
    out = np.zeros(L * S, capi.PAIR_DTYPE)
    out["laser_point"] = np.repeat(lg, S, axis=0)
    out["laser_wall"] = np.repeat(lw, S)
    out["camera_point"] = np.tile(cg, (L, 1))
    out["camera_wall"] = np.tile(cw, L)
    return out


def _box_dist(p: np.ndarray, lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
    c = np.clip(p, lo, hi)
    return np.linalg.norm(p - c, axis=-1)


def min_path(pairs: np.ndarray, lo: np.ndarray, hi: np.ndarray) -> float:
    lp = pairs["laser_point"].astype(np.float64)
    cp = pairs["camera_point"].astype(np.float64)
    d = (pairs["laser_wall"] + pairs["camera_wall"]).astype(np.float64)
    d = d + _box_dist(lp, lo, hi) + _box_dist(cp, lo, hi)
    return float(d.min())


# ---------------------------------------------------------------- scenes

def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _rotation(rng):
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return q


def sphere_points(rng, center, radius, n):
    return center + radius * _unit(rng, n)


def box_points(rng, center, half, n):
    """Area-uniform samples of an axis-aligned box surface, randomly rotated."""
    areas = np.array([half[1] * half[2], half[0] * half[2], half[0] * half[1]] * 2)
    face = rng.choice(6, size=n, p=areas / areas.sum())
    uv = rng.uniform(-1, 1, size=(n, 3))
    axis = face % 3
    sign = np.where(face < 3, 1.0, -1.0)
    uv[np.arange(n), axis] = sign
    return center + (uv * half) @ _rotation(rng).T


def torus_points(rng, center, R, r, n):
    u = rng.uniform(0, 2 * np.pi, n)
    v = rng.uniform(0, 2 * np.pi, n)
    p = np.stack([(R + r * np.cos(v)) * np.cos(u), r * np.sin(v), (R + r * np.cos(v)) * np.sin(u)], 1)
    return center + p @ _rotation(rng).T


def make_scene(spec: CaptureSpec, rng: np.random.Generator, lo: np.ndarray, hi: np.ndarray):
    p = spec.scene_params
    a_lo, a_hi = p.get("albedo", (0.2, 1.0))
    pts, alb = [], []
    edge = hi - lo
    if spec.scene in ("points", "points+sphere"):
        n = p["n"]
        pts.append(rng.uniform(lo, hi, size=(n, 3)))
        alb.append(rng.uniform(a_lo, a_hi, n))
    if spec.scene == "points+sphere":
        r = p["sphere_diameter"] / 2
        c = rng.uniform(lo + r, hi - r)
        m = p["sphere_points"]
        pts.append(sphere_points(rng, c, r, m))
        alb.append(np.full(m, rng.uniform(a_lo, a_hi)))
    if spec.scene == "objects":
        kmin, kmax = p["count"]
        k = int(rng.integers(kmin, kmax + 1))
        m = p["points"]
        for _ in range(k):
            kind = p["kinds"][int(rng.integers(len(p["kinds"])))]
            size = rng.uniform(0.08, 0.22) * float(edge.min())
            c = rng.uniform(lo + 1.6 * size, hi - 1.6 * size)
            if kind == "sphere":
                q = sphere_points(rng, c, size, m)
            elif kind == "box":
                q = box_points(rng, c, rng.uniform(0.5, 1.0, 3) * size, m)
            else:
                q = torus_points(rng, c, size, 0.35 * size, m)
            pts.append(q)
            alb.append(np.full(m, rng.uniform(a_lo, a_hi)))
    return np.concatenate(pts).astype(np.float32), np.concatenate(alb).astype(np.float32)


class ProductBackend:
    """Host functions of a synthetic capture, from the product library: the volume basis
    (bpgb_volume_basis), the renderer (bpgb_synth_render) and Poisson noise."""

    @staticmethod
    def volume_basis(volume_position, volume_size, voxels_per_side):
        return capi.volume_basis(volume_position, volume_size, voxels_per_side)

    @staticmethod
    def render(pairs, T, t0, deltaT, points, albedo):
        return capi.synth_render(pairs, T, t0, deltaT, points, albedo)

    @staticmethod
    def poisson(H, peak, seed):
        return capi.synth_poisson(H, peak, seed)


def make_capture(name: str, seed: int = 0, small: bool = False, render: bool = True,
                 backend=None, **overrides) -> Capture:
    """Builds (and renders) a seeded capture of configuration `name`.  `backend` supplies
    volume_basis / render / poisson (default: the product library's); another backend
    with the same arithmetic gives the same capture."""
    be = backend or ProductBackend
    spec = SPECS[name]
    fields = dict(spec.__dict__)
    if small:
        fields.update(SMALL[name])
    fields.update(overrides)
    spec = CaptureSpec(**fields)
    rng = np.random.default_rng(seed)
    cam_grid = wall_grid(spec.spad_grid, spec.wall_size)
    if spec.laser_grid is None:
        las_grid = np.zeros((1, 1, 3), np.float32)
    else:
        las_grid = wall_grid(spec.laser_grid, spec.wall_size)
    lpos = np.asarray(LASER_ORIGIN, np.float32)
    cpos = np.asarray(SPAD_ORIGIN, np.float32)
    pairs = make_pairs(lpos, las_grid, cpos, cam_grid, spec.confocal)
    vpos = np.asarray(spec.volume_position, np.float32)
    vsize = np.full(3, spec.volume_edge, np.float32)
    n = np.full(3, spec.voxels, np.uint32)
    zero, inc = be.volume_basis(vpos, vsize, n)
    lo = vpos.astype(np.float64) - spec.volume_edge / 2
    hi = vpos.astype(np.float64) + spec.volume_edge / 2
    dT = float(np.float32(spec.deltaT))
    t0 = float(np.float32(math.floor(min_path(pairs, lo, hi) / dT) * dT))
    points, albedo = make_scene(spec, rng, lo, hi)
    if render:
        H = be.render(pairs, spec.T, t0, dT, points, albedo)
        if spec.noise_peak:
            be.poisson(H, spec.noise_peak, seed + 2)
    else:
        H = np.zeros((len(pairs), spec.T), np.float32)
    wl = None
    if spec.wavelength_spacings:
        spacing = spec.wall_size / (spec.spad_grid[0] - 1)
        wl = float(np.float32(spec.wavelength_spacings * spacing))
    return Capture(spec, seed, H, pairs, las_grid, cam_grid, lpos, cpos, t0, dT, vpos, vsize, n,
                   zero, inc, points, albedo, wl)


# ---------------------------------------------------------------- batches

BATCH_GRIDS = (16, 32, 48, 64, 96)
BATCH_T = (512, 1024, 2048)
BATCH_VOXELS = (32, 48, 64, 96)


def make_batch(n: int = 64, seed: int = 0, render: bool = True, grids=BATCH_GRIDS,
               Ts=BATCH_T, voxels=BATCH_VOXELS, exhaustive_frac: float = 0.25,
               exhaustive_grid: int = 16, backend=None) -> list[Capture]:
    """Seeded uneven batch: n captures with SPAD grids g^2 (g from `grids`), T from `Ts`,
    volumes v^3 (v from `voxels`) and 4-40 point scatterers each.

    A fraction `exhaustive_frac` of the captures has a laser grid equal to its SPAD grid;
    those take the `exhaustive_grid`^2 grid (16^2: 65,536 pairs, the dense exhaustive
    shape), the others one
    laser at the wall centre.  Wall 1 x 1 m, deltaT 3 mm, volume a 0.5 m cube 0.6 m behind
    the wall (the dense configuration's geometry).  Capture i uses seed `seed * 1000 + i`."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        exhaustive = bool(rng.random() < exhaustive_frac)
        g = exhaustive_grid if exhaustive else int(rng.choice(grids))
        T = int(rng.choice(Ts))
        v = int(rng.choice(voxels))
        k = int(rng.integers(4, 41))
        out.append(make_capture(
            "dense_exhaustive_16", seed=seed * 1000 + i, render=render, backend=backend,
            laser_grid=(g, g) if exhaustive else None, spad_grid=(g, g), T=T, voxels=v,
            scene_params={"n": k, "albedo": (0.2, 1.0)}))
    return out


def batch_geometry(caps: list[Capture], scales=None) -> list[dict]:
    """Per-capture geometry dicts for capi.Batch (scales: per-capture H scale)."""
    return [{"pairs": c.pairs, "T": c.T, "voxels_per_side": c.voxels_per_side, "zero": c.zero,
             "inc": c.inc, "t0": c.t0, "deltaT": c.deltaT,
             "h_scale": 1.0 if scales is None else float(scales[i])} for i, c in enumerate(caps)]


def fp16_scales(caps: list[Capture]) -> np.ndarray:
    """Per-capture scale s with H / s inside FP16 range (peak at 2^15)."""
    return np.array([max(float(np.abs(c.H).max()), 1e-30) / 32768.0 for c in caps], np.float32)


def pack_batch(caps: list[Capture], row_offsets, pitch: int, dtype=np.float16,
               scales=None) -> np.ndarray:
    """Packed H [total_rows, pitch]: capture c's rows at row_offsets[c], divided by its
    scale and converted to `dtype`; bins beyond a capture's T are zero."""
    total = int(row_offsets[-1]) + caps[-1].P
    H = np.zeros((total, pitch), dtype)
    for i, c in enumerate(caps):
        r = int(row_offsets[i])
        h = c.H if scales is None else c.H / np.float32(scales[i])
        H[r:r + c.P, :c.T] = h.astype(dtype)
    return H
