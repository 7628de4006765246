"""The scene and .vox loaders (lum_gb300/vox.py) on files written here, and on the reference's
demo assets where they are present."""
import os
import struct

import numpy as np
import pytest

from lum_gb300 import vox


def _chunk(cid: bytes, content: bytes, children: bytes = b"") -> bytes:
    return cid + struct.pack("<ii", len(content), len(children)) + content + children


def _string(s: str) -> bytes:
    b = s.encode()
    return struct.pack("<i", len(b)) + b


def write_vox(path, size, voxels, rgba, matl):
    xyzi = struct.pack("<i", len(voxels)) + b"".join(struct.pack("<BBBB", *v) for v in voxels)
    body = _chunk(b"SIZE", struct.pack("<iii", *size)) + _chunk(b"XYZI", xyzi) + _chunk(b"RGBA", rgba.tobytes())
    for mid, d in matl.items():
        content = struct.pack("<ii", mid, len(d)) + b"".join(_string(k) + _string(v) for k, v in d.items())
        body += _chunk(b"MATL", content)
    with open(path, "wb") as f:
        f.write(b"VOX " + struct.pack("<i", 200) + _chunk(b"MAIN", b"", body))


def test_block_and_palette_round_trip(tmp_path):
    rgba = np.arange(1024, dtype=np.uint32).astype(np.uint8).reshape(256, 4)
    voxels = [(0, 0, 0, 5), (15, 1, 2, 7), (3, 15, 15, 200)]
    p = tmp_path / "b.vox"
    write_vox(p, (16, 16, 16), voxels, rgba, {7: {"_type": "_emit", "_emit": "2", "_flux": "0.5"},
                                              5: {"_type": "_metal", "_rough": "0.2", "_metal": "0.6"}})
    b = vox.load_block(str(p))
    assert b[0, 0, 0] == 5 and b[15, 1, 2] == 7 and b[3, 15, 15] == 200 and (b > 0).sum() == 3
    m = vox.material_palette(str(p))
    assert np.allclose(m[7, :4], rgba[6] / 256.0)          # colour index i is file entry i-1
    assert m[7, 4] == np.float32(2 * (2 + 0.5 * 4)) and m[7, 5] == 0.5
    assert np.isclose(m[5, 5], (0.2 + 0.4) / 2)
    assert m[1, 5] == 1.0 and m[1, 4] == 0.0                 # no MATL: diffuse


def test_scene_clamps_and_crops(tmp_path):
    g = np.arange(5 * 4 * 3, dtype=np.int16).reshape(3, 4, 5) - 10
    p = tmp_path / "scene"
    with open(p, "wb") as f:
        f.write(struct.pack("<iii", 5, 4, 3) + g.tobytes())
    out = vox.load_scene(str(p), (4, 4, 2), 15)
    assert out.shape == (2, 4, 4)
    assert np.array_equal(out, np.clip(g[:2, :, :4], 0, 15))


from oracle import build_ref  # noqa: E402  (where the reference tree is, when it is present)

REF = os.path.join(build_ref.REFERENCE, "assets")


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference assets absent")
def test_reference_demo_assets():
    g = vox.load_scene(os.path.join(REF, "scene"), (48, 48, 16), 15)
    assert g.shape == (16, 48, 48) and g.max() == 14
    b = vox.load_block(os.path.join(REF, "dirt.vox"))
    assert b.shape == (16, 16, 16) and (b > 0).mean() > 0.5
    m = vox.material_palette(os.path.join(REF, "tank_body.vox"))
    assert (m[:, 4] > 0).sum() > 0


def test_scene_round_trip(tmp_path):
    from lum_gb300 import worldgen
    w = worldgen.terrain_world((9, 7, 5), seed=3, n_types=12)
    p = str(tmp_path / "scene")
    vox.save_scene(p, w.grid)
    assert np.array_equal(vox.load_scene(p, w.dims, 12), w.grid)
    # a smaller world reads the corner that fits
    assert np.array_equal(vox.load_scene(p, (4, 3, 2), 12), w.grid[:2, :3, :4])
