"""Golden fixtures produced by the reference shader (tests/golden/make_golden.py).

Each fixture holds a pass's inputs and the radiance volumes that Lum's own radiance.comp,
compiled as C++, produced.  The CPU oracle and the GPU library (through the C ABI, with the
reference's i8vec4 request encoding) must reproduce them within 1e-5 relative (FP32; observed
bit-identical).  Fixtures marked with the rgb10_a2 storage hold volumes in the image's own
10-bit format: there the GPU (LUMRAD_PRECISION_RGB10A2) and the oracle must match bit for bit.
"""
import glob
import os

import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def load(path):
    d = np.load(path)
    w = worldgen.World(grid=d["grid"], palette=d["palette"], materials=d["materials"])
    rays, max_dist, blend, seed, size, shift, passes = d["params"]
    p = dict(rays=int(rays), max_dist=float(max_dist), blend=float(blend), time_seed=int(seed), size=int(size),
             shift=int(shift))
    storage = str(d["storage"]) if "storage" in d.files else "fp32"
    return w, d["requests"], d["prev"], d["expected"], int(passes), p, storage


def test_fixtures_present():
    names = {os.path.basename(f) for f in FIXTURES}
    assert {"demo_scene.npz", "terrain_c1.npz", "slicing_r256.npz", "odd_ids.npz", "demo_scene_rgb10a2.npz",
            "terrain_rgb10a2.npz"} <= names


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_oracle_reproduces_reference(path):
    import oracle
    w, req, prev, expected, passes, p, storage = load(path)
    cur = prev
    for i in range(passes):
        q = dict(p)
        q["time_seed"] = p["time_seed"] + i
        cur, _, _ = oracle.radiance_pass(w, req, prev=cur, unorm10=storage == "rgb10a2", **q)
        assert cur.tobytes() == expected[i].tobytes(), f"pass {i}"


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_gpu_reproduces_reference(path):
    import lum_gb300
    w, req, prev, expected, passes, p, storage = load(path)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=storage) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        for i in range(passes):
            q = dict(p)
            q["time_seed"] = p["time_seed"] + i
            rw.radiance_pass(req.astype(np.int8), lum_gb300.pass_params(**q))
            got = rw.get_radiance()
            if storage == "rgb10a2":   # the reference's own volume format: bit for bit
                assert got.tobytes() == expected[i].tobytes(), (i, np.abs(got - expected[i]).max())
            else:
                assert rel_err(got, expected[i]).max() <= RTOL, (i, rel_err(got, expected[i]).max())
