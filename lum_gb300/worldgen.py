"""Seeded synthetic worlds for the radiance pass.

Everything is drawn from a counter-based splitmix64 stream, so a (seed, stream, index) triple
gives the same value on every machine and numpy version.

A world is:
  grid      (Z, Y, X) int16 block ids, x-fastest in memory (Lum's table3d order); 0 = air
  palette   (n_slots, 16, 16, 16) uint8 voxels indexed [slot, z, y, x] (x-fastest, the layout of
            one 16^3 slot of Lum's palette image); slot 0 is air
  materials (256, 6) float32: r, g, b, a, emission, roughness (LumInternal::Material)

Terrain: a 2D value-noise heightmap in voxel units (lattice every 32 voxels, smoothstep
interpolation, 3 octaves of halving spacing and amplitude), height in [0.25, 0.6] of the world's
voxel height; a block is solid when its centre lies below the height at its column's centre.
Block types: per type an air fraction U(0, 0.3); solid voxels draw from 4 type-specific
material ids in 1..255.  Materials: albedo U(0,1)^3, 5% emissive with emission U(1,8),
roughness U(0,1); entry 0 is air (all zero).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n doubles in [0, 1) from stream `stream` of `seed`."""
    with np.errstate(over="ignore"):
        base = _splitmix64(np.array([seed & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64))[0]
        base = _splitmix64(np.array([base ^ np.uint64(stream & 0xFFFFFFFFFFFFFFFF)], dtype=np.uint64))[0]
        idx = np.arange(n, dtype=np.uint64) + base
    return (_splitmix64(idx) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def randint(seed: int, stream: int, n: int, lo: int, hi: int) -> np.ndarray:
    """n integers in [lo, hi)."""
    return (lo + np.floor(uniform(seed, stream, n) * (hi - lo))).astype(np.int64)


@dataclass
class World:
    grid: np.ndarray
    palette: np.ndarray
    materials: np.ndarray
    seed: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def dims(self) -> tuple[int, int, int]:
        z, y, x = self.grid.shape
        return x, y, z

    @property
    def n_blocks(self) -> int:
        return int(self.grid.size)

    def block_voxels(self, slot: int) -> np.ndarray:
        """Slot as Lum's BlockVoxels[x][y][z] (z fastest), the lum_load_block layout."""
        return np.ascontiguousarray(self.palette[slot].transpose(2, 1, 0))


# streams
_S_HEIGHT, _S_TYPES, _S_EXTRA_POS, _S_EXTRA_TYPE, _S_PAL, _S_MAT, _S_SUBSET = range(1, 8)


def materials(seed: int) -> np.ndarray:
    u = uniform(seed, _S_MAT, 256 * 6).reshape(256, 6)
    m = np.zeros((256, 6), dtype=np.float32)
    m[:, 0:3] = u[:, 0:3]
    m[:, 3] = 1.0
    emissive = u[:, 3] < 0.05
    m[:, 4] = np.where(emissive, 1.0 + 7.0 * u[:, 4], 0.0)
    m[:, 5] = u[:, 5]
    m[0] = 0.0
    return m


def block_types(seed: int, n_types: int) -> np.ndarray:
    """(n_types+1, 16, 16, 16) uint8 palette indexed [slot, z, y, x]; slot 0 is air."""
    pal = np.zeros((n_types + 1, 16, 16, 16), dtype=np.uint8)
    for t in range(1, n_types + 1):
        u = uniform(seed, _S_PAL * 100003 + t, 4096 * 2 + 5)
        air = 0.3 * u[0]
        mats = 1 + np.floor(u[1:5] * 255).astype(np.int64)
        is_air = u[5:5 + 4096] < air
        pick = np.floor(u[5 + 4096:5 + 8192] * 4).astype(np.int64)
        vox = np.where(is_air, 0, mats[pick]).astype(np.uint8)
        pal[t] = vox.reshape(16, 16, 16)
    return pal


def _value_noise_height(seed: int, X: int, Y: int, Z: int) -> np.ndarray:
    """Height (voxels) at block-column centres, shape (Y, X)."""
    vx = np.arange(X) * 16 + 8.0
    vy = np.arange(Y) * 16 + 8.0
    total = np.zeros((Y, X))
    amp_sum = 0.0
    for octave in range(3):
        cell = 32.0 / (2 ** octave)
        amp = 1.0 / (2 ** octave)
        nx = int(np.ceil(X * 16 / cell)) + 2
        ny = int(np.ceil(Y * 16 / cell)) + 2
        lat = uniform(seed, _S_HEIGHT * 1000 + octave, nx * ny).reshape(ny, nx)
        fx = vx / cell
        fy = vy / cell
        ix = np.floor(fx).astype(np.int64)
        iy = np.floor(fy).astype(np.int64)
        tx = fx - ix
        ty = fy - iy
        sx = tx * tx * (3 - 2 * tx)
        sy = ty * ty * (3 - 2 * ty)
        a = lat[iy[:, None], ix[None, :]]
        b = lat[iy[:, None], ix[None, :] + 1]
        c = lat[iy[:, None] + 1, ix[None, :]]
        d = lat[iy[:, None] + 1, ix[None, :] + 1]
        top = a + (b - a) * sx[None, :]
        bot = c + (d - c) * sx[None, :]
        total += amp * (top + (bot - top) * sy[:, None])
        amp_sum += amp
    h = total / amp_sum
    return (0.25 + 0.35 * h) * 16.0 * Z


def terrain_world(dims: tuple[int, int, int], seed: int = 1234, n_types: int = 32,
                  extra_blocks: int = 0) -> World:
    """Terrain world of dims (X, Y, Z) blocks, optionally with `extra_blocks` random blocks."""
    X, Y, Z = dims
    height = _value_noise_height(seed, X, Y, Z)
    zc = np.arange(Z) * 16 + 8.0
    solid = zc[:, None, None] < height[None, :, :]
    types = randint(seed, _S_TYPES, X * Y * Z, 1, n_types + 1).reshape(Z, Y, X)
    grid = np.where(solid, types, 0).astype(np.int16)
    if extra_blocks:
        pos = randint(seed, _S_EXTRA_POS, extra_blocks, 0, X * Y * Z)
        typ = randint(seed, _S_EXTRA_TYPE, extra_blocks, 1, n_types + 1)
        flat = grid.reshape(-1)
        flat[pos] = typ
    return World(grid=np.ascontiguousarray(grid), palette=block_types(seed, n_types),
                 materials=materials(seed), seed=seed,
                 meta={"dims": dims, "n_types": n_types, "extra_blocks": extra_blocks})


def all_probes(dims: tuple[int, int, int]) -> np.ndarray:
    """(W, 4) int16 requests (x, y, z, 0) of every block, in z, y, x scan order."""
    X, Y, Z = dims
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    out = np.zeros((X * Y * Z, 4), dtype=np.int16)
    out[:, 0] = x.reshape(-1)
    out[:, 1] = y.reshape(-1)
    out[:, 2] = z.reshape(-1)
    return out


def probe_subset(dims: tuple[int, int, int], fraction: float, seed: int, stream: int = 0) -> np.ndarray:
    """A seeded subset of round(fraction*W) distinct probes, in scan order."""
    allp = all_probes(dims)
    W = allp.shape[0]
    k = max(1, int(round(fraction * W)))
    keys = uniform(seed, _S_SUBSET * 1000003 + stream, W)
    idx = np.sort(np.argsort(keys, kind="stable")[:k])
    return np.ascontiguousarray(allp[idx])


def mixed_worlds(n: int = 256, seed: int = 1234, max_dims=(32, 32, 16), min_dims=(4, 4, 4),
                 rays=(32, 64, 128, 256)):
    """The batching workload: n independent terrain worlds with dims uniform per axis in
    [min, max], each with a seeded update list of U(1%, 100%) of its probes and rays per probe
    drawn from `rays`.  Returns [(World, requests, rays_per_probe)]."""
    out = []
    u = uniform(seed, 9001, 5 * n).reshape(n, 5)
    for i in range(n):
        dims = tuple(int(lo + np.floor(u[i, a] * (hi - lo + 1))) for a, (lo, hi) in enumerate(zip(min_dims, max_dims)))
        w = terrain_world(dims, seed=seed * 1000 + i, n_types=32)
        frac = 0.01 + 0.99 * u[i, 3]
        req = probe_subset(dims, frac, seed=seed * 1000 + i, stream=0)
        r = int(rays[min(int(u[i, 4] * len(rays)), len(rays) - 1)])
        out.append((w, req, r))
    return out


_S_EDIT = 11


def edit_request(dims, fraction: float, seed: int, stream: int, n_types: int = 32) -> np.ndarray:
    """A relight request's edits: round(fraction * blocks) (at least 1) seeded block-type changes
    at uniform positions (repeats allowed; the last edit of a block wins), new ids uniform in
    0..n_types (0 digs the block out).  (n, 4) int16 rows (x, y, z, block)."""
    X, Y, Z = dims
    n = max(1, int(round(fraction * X * Y * Z)))
    u = uniform(seed, _S_EDIT * 1000003 + stream, 4 * n).reshape(n, 4)
    out = np.empty((n, 4), dtype=np.int16)
    out[:, 0] = np.floor(u[:, 0] * X)
    out[:, 1] = np.floor(u[:, 1] * Y)
    out[:, 2] = np.floor(u[:, 2] * Z)
    out[:, 3] = np.floor(u[:, 3] * (n_types + 1))
    return out


def apply_edits(grid: np.ndarray, edits: np.ndarray) -> np.ndarray:
    """The grid (Z, Y, X) after the edits, applied in order."""
    g = grid.copy()
    for x, y, z, b in edits:
        g[z, y, x] = b
    return g


def dirty_probes(dims, edits: np.ndarray, radius: int = 2) -> np.ndarray:
    """Probes within Chebyshev distance `radius` of any edit, (n, 4) int16 (x, y, z, 0) in
    x-fastest scan order."""
    X, Y, Z = dims
    mask = np.zeros((Z, Y, X), dtype=bool)
    for x, y, z, _ in edits:
        mask[max(z - radius, 0):z + radius + 1, max(y - radius, 0):y + radius + 1, max(x - radius, 0):x + radius + 1] = True
    zz, yy, xx = np.nonzero(mask)
    out = np.zeros((zz.size, 4), dtype=np.int16)
    out[:, 0], out[:, 1], out[:, 2] = xx, yy, zz
    return out


def serving_worlds(n: int = 64, seed: int = 1234, lo: int = 8 ** 3, hi: int = 64 * 64 * 32):
    """The serving workload's worlds: block counts lognormal (median sqrt(lo*hi), 2 sigma = half
    the log range) clipped to [lo, hi]; dims X = Y = round(cbrt(2n)) in [8, 64], Z = n/(X*Y) in
    [8, 32].  Returns [World]."""
    u = uniform(seed, 9101, 2 * n).reshape(n, 2)
    # Box-Muller normal from two uniforms
    g = np.sqrt(-2.0 * np.log(np.maximum(u[:, 0], 1e-300))) * np.cos(2.0 * np.pi * u[:, 1])
    mu = 0.5 * (np.log(lo) + np.log(hi))
    sigma = 0.25 * (np.log(hi) - np.log(lo))
    blocks = np.clip(np.exp(mu + sigma * g), lo, hi)
    out = []
    for i, b in enumerate(blocks):
        xy = int(np.clip(round((2.0 * b) ** (1.0 / 3.0)), 8, 64))
        z = int(np.clip(round(b / (xy * xy)), 8, 32))
        out.append(terrain_world((xy, xy, z), seed=seed * 1000 + 500 + i, n_types=32))
    return out


def poisson_arrivals(n: int, rate: float, seed: int) -> np.ndarray:
    """n arrival times (s) of a Poisson process of `rate` per second, starting at 0."""
    u = uniform(seed, 9201, n)
    gaps = -np.log(np.maximum(1.0 - u, 1e-300)) / rate
    t = np.cumsum(gaps)
    return t - t[0]


def small_world(dims=(8, 8, 8), seed: int = 1234) -> World:
    """The 8x8x8 terrain world with 32 block types."""
    return terrain_world(dims, seed=seed, n_types=32)


def demo_world(seed: int = 1234) -> World:
    """The 64x64x16 terrain world plus 2000 random blocks of 32 types."""
    return terrain_world((64, 64, 16), seed=seed, n_types=32, extra_blocks=2000)
