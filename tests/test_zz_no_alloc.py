"""The no-allocation pass (lumrad_radiance_pass_noalloc) against the regular pass and the oracle.

Some callers of this library may not allocate device memory while they run — an engine that
reserved its whole budget at start-up, or a host whose own allocator owns the device heap.  For
them the library has one entry point that allocates nothing: they hand it device pointers to the
world, the request list and the two radiance volumes, and the working buffers live in a fixed
array inside the library.  These tests allocate the caller's buffers (with torch, as such a caller
would with its own allocator), run passes in a row through that entry point, and check the
results against lumrad_radiance_pass on a context or against the CPU oracle, within the parity
tolerance of the other GPU tests.  They cover passes of one round and of many rounds (the array
holds the rays of 4,096 subgroups at a time), time slicing, and the block ids whose compact form
is built separately here (negative ids, ids without a palette slot, SPECIAL_BLOCK, a non-empty
slot 0).  This file is collected last so that a failure here cannot hide the results of the other
tests.
"""
import ctypes as C

import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err

pytestmark = pytest.mark.gpu


def _context_passes(w, req, prev, params):
    import lum_gb300
    want = []
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        for p in params:
            rw.radiance_pass(req, p)
            want.append(rw.get_radiance())
    return want


def _noalloc_passes(w, req, prev, params):
    """The passes through the no-allocation entry point on caller-owned device buffers, ping-pong
    between two volumes; returns each pass's volume as (Z, Y, X, 3)."""
    import torch

    from lum_gb300._native import check, load

    lib = load()
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
    out = []
    for i, p in enumerate(params):
        src, dst = vol[i % 2], vol[(i + 1) % 2]
        check(lib.lumrad_radiance_pass_noalloc(ws, grid.data_ptr(), pal.data_ptr(), w.palette.shape[0],
                                               mats.data_ptr(), reqs.data_ptr(), req.shape[0], src.data_ptr(),
                                               dst.data_ptr(), C.byref(p), stream))
        torch.cuda.synchronize(dev)
        out.append(dst[..., :3].cpu().numpy())
    err = C.c_int(-1)
    check(lib.lumrad_radiance_pass_noalloc_status(stream, C.byref(err)))   # every pass completed
    assert err.value == 0
    return out


@pytest.mark.parametrize("rays", [64, 256])
def test_noalloc_pass_matches_context_pass_twice(rays):
    import lum_gb300
    w = worldgen.terrain_world((12, 10, 6), seed=41, extra_blocks=30)
    req = worldgen.probe_subset(w.dims, 0.6, seed=3)
    prev = random_prev(w)
    params = [lum_gb300.pass_params(rays=rays, max_dist=256.0, blend=0.1, time_seed=s) for s in (0, 1)]
    want = _context_passes(w, req, prev, params)
    got = _noalloc_passes(w, req, prev, params)
    for i in range(2):
        assert rel_err(got[i], want[i]).max() <= RTOL, (i, rel_err(got[i], want[i]).max())


@pytest.mark.parametrize("size,shift", [(1, 0), (3, 1)])
def test_noalloc_pass_of_many_rounds(size, shift):
    """8,192 probes x 256 rays: 65,536 subgroups, 16 rounds of the array's 4,096 (the queue reset by
    the last warp of each round, the round's ray results re-based), and a sliced list (size 3,
    shift 1: 2,730 probes, 6 rounds, the last one partial), two passes in a row."""
    import lum_gb300
    w = worldgen.terrain_world((32, 32, 8), seed=44, extra_blocks=200)
    req = worldgen.all_probes(w.dims)
    prev = random_prev(w)
    params = [lum_gb300.pass_params(rays=256, max_dist=256.0, blend=0.1, time_seed=s, size=size, shift=shift)
              for s in (5, 6)]
    want = _context_passes(w, req, prev, params)
    got = _noalloc_passes(w, req, prev, params)
    for i in range(2):
        assert rel_err(got[i], want[i]).max() <= RTOL, (i, rel_err(got[i], want[i]).max())


def test_noalloc_odd_ids_match_oracle():
    """Negative ids (OpSMod palette aliasing), ids past the loaded slots, SPECIAL_BLOCK and a
    non-empty palette slot 0, against the CPU oracle: the no-allocation path builds its own
    compact ids (ids without a palette slot share one empty entry)."""
    import lum_gb300
    import oracle
    w = worldgen.terrain_world((9, 9, 5), seed=30, n_types=8)
    g = w.grid.reshape(-1).copy()
    idx = worldgen.randint(31, 1, 60, 0, g.size)
    vals = np.array([-1, -5, -63, -64, -200, 9, 40, 4095, 32767, 12], dtype=np.int16)
    g[idx] = vals[np.arange(60) % vals.size]
    pal = w.palette.copy()
    pal[0, 3:5, :, 6:9] = 17
    w2 = worldgen.World(grid=g.reshape(w.grid.shape), palette=pal, materials=w.materials)
    req = worldgen.all_probes(w2.dims)
    prev = random_prev(w2)
    p = [dict(rays=64, max_dist=160.0, blend=0.2, time_seed=s) for s in (4, 5)]
    got = _noalloc_passes(w2, req, prev, [lum_gb300.pass_params(**q) for q in p])
    ref = prev
    for i, q in enumerate(p):
        ref, _, _ = oracle.radiance_pass(w2, req, prev=ref, **q)
        assert rel_err(got[i], ref).max() <= RTOL, (i, rel_err(got[i], ref).max())


def test_noalloc_rejects_bad_arguments():
    import lum_gb300
    from lum_gb300._native import LUMRAD_EINVAL, load

    lib = load()
    p = lum_gb300.pass_params(rays=64)
    ws = (C.c_int * 3)(1024, 1024, 1)   # 2^20 blocks, above LUMRAD_NOALLOC_MAX_BLOCKS
    rc = lib.lumrad_radiance_pass_noalloc(ws, 1, 1, 8, 1, 1, 1, 1, 1 << 30, C.byref(p), None)
    assert rc == LUMRAD_EINVAL
    assert b"LUMRAD_NOALLOC_MAX_BLOCKS" in lib.lumrad_last_error()
    ws = (C.c_int * 3)(4, 4, 4)          # 64 probes = 1,024 B per volume
    for prev, nxt in [(1 << 20, 1 << 20), (1 << 20, (1 << 20) + 1008), ((1 << 20) + 1008, 1 << 20)]:
        rc = lib.lumrad_radiance_pass_noalloc(ws, 1, 1, 8, 1, 1, 1, prev, nxt, C.byref(p), None)
        assert rc == LUMRAD_EINVAL and b"overlap" in lib.lumrad_last_error(), (prev, nxt)
