"""The no-allocation pass (lumrad_radiance_pass_noalloc) against the regular pass.

Some callers of this library may not allocate device memory while they run — an engine that
reserved its whole budget at start-up, or a host whose own allocator owns the device heap.  For
them the library has one entry point that allocates nothing: they hand it device pointers to the
world, the request list and the two radiance volumes, and the working buffers live in a fixed
array inside the library.  This test allocates the caller's buffers (with torch, as such a caller
would with its own allocator), runs two passes in a row through that entry point, and checks both
results against lumrad_radiance_pass on a context, within the parity tolerance of the other GPU
tests.  It is collected last so that a failure here cannot hide the results of the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rays", [64, 256])
def test_noalloc_pass_matches_context_pass_twice(rays):
    import torch

    import lum_gb300
    from lum_gb300._native import check, load

    lib = load()
    w = worldgen.terrain_world((12, 10, 6), seed=41, extra_blocks=30)
    req = worldgen.probe_subset(w.dims, 0.6, seed=3)
    prev = random_prev(w)
    seeds = [0, 1]
    params = [lum_gb300.pass_params(rays=rays, max_dist=256.0, blend=0.1, time_seed=s) for s in seeds]

    # regular path: a context that owns its device memory
    want = []
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        for p in params:
            rw.radiance_pass(req, p)
            want.append(rw.get_radiance())

    # caller-owned device buffers
    dev = torch.device("cuda", 0)
    grid = torch.from_numpy(np.ascontiguousarray(w.grid)).to(dev)
    pal = torch.from_numpy(np.ascontiguousarray(w.palette.reshape(-1))).to(dev)
    mats = torch.from_numpy(np.ascontiguousarray(w.materials[:, [0, 1, 2, 4]])).to(dev)
    reqs = torch.from_numpy(np.ascontiguousarray(req)).to(dev)
    vol = [torch.zeros(w.grid.shape + (4,), dtype=torch.float32, device=dev) for _ in range(2)]
    vol[0][..., :3] = torch.from_numpy(prev).to(dev)
    vol[0][..., 3] = 1.0
    ws = (C.c_int * 3)(*w.dims)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for i, p in enumerate(params):
        src, dst = vol[i % 2], vol[(i + 1) % 2]
        check(lib.lumrad_radiance_pass_noalloc(ws, grid.data_ptr(), pal.data_ptr(), w.palette.shape[0],
                                               mats.data_ptr(), reqs.data_ptr(), req.shape[0], src.data_ptr(),
                                               dst.data_ptr(), C.byref(p), stream))
        torch.cuda.synchronize(dev)
        got = dst[..., :3].cpu().numpy()
        assert rel_err(got, want[i]).max() <= RTOL, (i, rel_err(got, want[i]).max())


def test_noalloc_rejects_oversized_world():
    import lum_gb300
    from lum_gb300._native import LUMRAD_EINVAL, load

    lib = load()
    ws = (C.c_int * 3)(1024, 1024, 1)   # 2^20 blocks, above LUMRAD_NOALLOC_MAX_BLOCKS
    p = lum_gb300.pass_params(rays=64)
    rc = lib.lumrad_radiance_pass_noalloc(ws, 1, 1, 8, 1, 1, 1, 1, 1, C.byref(p), None)
    assert rc == LUMRAD_EINVAL
    assert b"LUMRAD_NOALLOC_MAX_BLOCKS" in lib.lumrad_last_error()
