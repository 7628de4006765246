"""Lum's world and block files: the scene grid and MagicaVoxel .vox blocks and palettes.

Restates the loaders of src/renderer/src/load_stuff.cpp that produce the radiance pass's inputs:
  load_scene        (:187-210) ivec3 header + int16 x-fastest grid, ids clamped to [0, slots]
  load_block        (:308-334) one 16^3 model -> BlockVoxels[x][y][z]
  extract_palette   (:233-285) 256 .vox palette entries + MATL -> Material (color/256, emission
                    emit*(2 + 4*flux) for emissive materials, roughness by material type)
The .vox reader follows the published MagicaVoxel file format: RIFF-like chunks
(id, content size, children size); SIZE and XYZI give a model, RGBA the 256-colour palette
(file entry i is colour index i+1), MATL a material dictionary per colour index.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np


@dataclass
class VoxFile:
    models: list = field(default_factory=list)        # [(size_xyz, voxel_data uint8 [x + sx*(y + sy*z)])]
    palette: np.ndarray | None = None                  # (256, 4) uint8 rgba, indexed by colour index
    materials: dict = field(default_factory=dict)      # colour index -> {key: value} (MATL dictionary)


def _read_string(b: bytes, off: int) -> tuple[str, int]:
    n = struct.unpack_from("<i", b, off)[0]
    return b[off + 4:off + 4 + n].decode("utf-8", "replace"), off + 4 + n


def read_vox(path: str) -> VoxFile:
    b = open(path, "rb").read()
    if b[:4] != b"VOX ":
        raise ValueError(f"{path}: not a .vox file")
    out = VoxFile()
    size = None

    def walk(off: int, end: int):
        nonlocal size
        while off + 12 <= end:
            cid = b[off:off + 4]
            n, m = struct.unpack_from("<ii", b, off + 4)
            body = off + 12
            if cid == b"SIZE":
                size = struct.unpack_from("<iii", b, body)
            elif cid == b"XYZI":
                count = struct.unpack_from("<i", b, body)[0]
                xyzi = np.frombuffer(b, dtype=np.uint8, count=4 * count, offset=body + 4).reshape(count, 4)
                sx, sy, sz = size
                vox = np.zeros(sx * sy * sz, dtype=np.uint8)
                vox[xyzi[:, 0].astype(np.int64) + sx * (xyzi[:, 1].astype(np.int64) + sy * xyzi[:, 2].astype(np.int64))] = xyzi[:, 3]
                out.models.append((tuple(size), vox))
            elif cid == b"RGBA":
                raw = np.frombuffer(b, dtype=np.uint8, count=1024, offset=body).reshape(256, 4)
                pal = np.zeros((256, 4), dtype=np.uint8)
                pal[1:] = raw[:255]       # file entry i is colour index i + 1
                pal[0] = raw[255]
                out.palette = pal
            elif cid == b"MATL":
                mid = struct.unpack_from("<i", b, body)[0]
                pairs = struct.unpack_from("<i", b, body + 4)[0]
                o = body + 8
                d = {}
                for _ in range(pairs):
                    k, o = _read_string(b, o)
                    v, o = _read_string(b, o)
                    d[k] = v
                out.materials[mid] = d
            walk(body + n, body + n + m)
            off = body + n + m

    walk(8, len(b))
    return out


def load_block(path: str) -> np.ndarray:
    """A 16^3 block as BlockVoxels[x][y][z] (load_stuff.cpp:308-334)."""
    v = read_vox(path)
    if len(v.models) != 1:
        raise ValueError(f"{path}: expected one model")
    (sx, sy, sz), data = v.models[0]
    out = np.zeros((16, 16, 16), dtype=np.uint8)
    xs, ys, zs = min(sx, 16), min(sy, 16), min(sz, 16)
    grid = data.reshape(sz, sy, sx)
    out[:xs, :ys, :zs] = grid[:zs, :ys, :xs].transpose(2, 1, 0)
    return out


def material_palette(path: str) -> np.ndarray:
    """256 materials (r, g, b, a, emission, roughness) from a .vox palette (load_stuff.cpp:233-271)."""
    v = read_vox(path)
    if v.palette is None:
        raise ValueError(f"{path}: no RGBA palette chunk")
    m = np.zeros((256, 6), dtype=np.float32)
    m[:, :4] = (v.palette.astype(np.float64) / 256.0).astype(np.float32)
    for i in range(256):
        d = v.materials.get(i, {})
        kind = d.get("_type", "_diffuse")
        rough = 0.0
        if kind == "_diffuse":
            rough = 1.0
        elif kind == "_emit":
            emit = float(d.get("_emit", "0"))
            flux = float(d.get("_flux", "0"))
            m[i, 4] = np.float32(emit * (2.0 + flux * 4.0))
            rough = 0.5
        elif kind == "_metal":
            rough = (float(d.get("_rough", "0")) + (1.0 - float(d.get("_metal", "0")))) / 2.0
        m[i, 5] = np.float32(rough)
    return m


def save_scene(path: str, grid: np.ndarray) -> None:
    """A scene file as save_scene writes it (load_stuff.cpp:218-231): the ivec3 world size (x, y, z)
    and the int16 grid, x-fastest.  grid is (Z, Y, X)."""
    g = np.ascontiguousarray(grid, dtype="<i2")
    Z, Y, X = g.shape
    with open(path, "wb") as f:
        f.write(struct.pack("<iii", X, Y, Z) + g.tobytes())


def load_scene(path: str, world_size, palette_slots: int) -> np.ndarray:
    """The int16 grid (Z, Y, X) of a scene file (load_stuff.cpp:187-210): an ivec3 header and an
    x-fastest int16 grid; the part inside world_size is read, ids clamped to [0, palette_slots]."""
    b = open(path, "rb").read()
    X, Y, Z = world_size
    out = np.zeros((Z, Y, X), dtype=np.int16)
    if len(b) < 12:
        return out
    sx, sy, sz = struct.unpack_from("<iii", b, 0)
    stored = np.frombuffer(b, dtype=np.int16, offset=12, count=(len(b) - 12) // 2)
    rx, ry, rz = (max(0, min(a, c)) for a, c in ((sx, X), (sy, Y), (sz, Z)))
    for z in range(rz):
        for y in range(ry):
            row = stored[sx * y + sx * sy * z: sx * y + sx * sy * z + rx]
            out[z, y, :rx] = np.clip(row, 0, palette_slots)
    return out
