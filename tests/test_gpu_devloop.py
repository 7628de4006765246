"""The relight server's device-resident request loop (settings.device_loop = 1).

The loop runs on the GPU as one CUDA graph with a WHILE node: it polls a host-written ring of
requests (a bounded wait), applies each request's edits, derives the dirty probes on the device
and relights them, and writes completions back.  Its results must equal the host loop's bit for
bit (both run the same pass kernels over the same lists) and the CPU oracle's within the FP32
tolerance; a world's result must be the same alone and among other worlds' requests; the loop
must start again after it ended idle.
"""
import time

import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err
from tests.test_gpu_serve import DIMS, _requests, _submit, _worlds

pytestmark = pytest.mark.gpu


def _serve(worlds, which, reqs, precision="fp32", **kw):
    import lum_gb300
    srv = lum_gb300.RadianceServer(precision=precision, **kw)
    rws = []
    for i in which:
        w = worlds[i]
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=precision)
        rw.load(w)
        rw.set_radiance(random_prev(w, seed=200 + i))
        srv.add_world(rw)
        rws.append(rw)
    _submit(srv, reqs, which)
    srv.run(timeout_s=300)
    done = srv.poll(len(reqs) + 8)
    vols = [srv.get_radiance(k) for k in range(len(which))]
    stats = srv.stats()
    srv.close()
    for rw in rws:
        rw.close()
    return vols, done, stats


@pytest.mark.parametrize("precision", ["fp32", "rgb10a2"])
def test_device_loop_equals_host_loop_and_oracle(precision):
    import dataclasses

    import oracle
    worlds = _worlds()
    reqs = _requests(3)
    which = list(range(len(DIMS)))
    host, _, _ = _serve(worlds, which, reqs, precision, max_inflight=2)
    dev, done, st = _serve(worlds, which, reqs, precision, device_loop=True)
    assert len(done) == len(reqs) and (done["status"] == 0).all()
    assert (done["done_s"] >= done["arrival_s"] - 1e-4).all()
    for i in which:
        assert dev[i].tobytes() == host[i].tobytes(), i
    if precision != "fp32":
        return
    for i in which:
        w = worlds[i]
        cur = random_prev(w, seed=200 + i)
        grid = w.grid
        for j, e, r, seed in reqs:
            if j != i:
                continue
            grid = worldgen.apply_edits(grid, e)
            we = dataclasses.replace(w, grid=grid)
            cur, _, _ = oracle.radiance_pass(we, worldgen.dirty_probes(w.dims, e, 2), rays=r, max_dist=64.0, blend=0.1,
                                             time_seed=seed, prev=cur)
        assert rel_err(dev[i], cur).max() <= RTOL, i


def test_device_loop_alone_equals_mix():
    worlds = _worlds()
    reqs = _requests(2, seed=5)
    mix, _, _ = _serve(worlds, [0, 1, 2, 3], reqs, device_loop=True)
    for i in range(len(DIMS)):
        alone, _, _ = _serve(worlds, [i], reqs, device_loop=True)
        assert alone[0].tobytes() == mix[i].tobytes(), i


def test_device_loop_last_edit_wins_and_restarts_after_idle():
    """A request that edits one block twice (the later edit wins, as on the host loop), and
    requests published after the loop ended idle (poll 0.2 ms): the host starts it again."""
    import lum_gb300
    w = worldgen.terrain_world((10, 9, 6), seed=71, n_types=16)
    e1 = np.array([[2, 3, 1, 5], [4, 4, 2, 0], [2, 3, 1, 9], [7, 1, 5, -3]], np.int16)   # (2,3,1) twice
    e2 = worldgen.edit_request(w.dims, 0.03, seed=72, stream=0)
    out = {}
    for mode in ("host", "device"):
        srv = lum_gb300.RadianceServer(device_loop=(mode == "device"), poll_ms=0.2)
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0])
        rw.load(w)
        rw.set_radiance(random_prev(w, seed=73))
        srv.add_world(rw)
        srv.submit(0, e1, lum_gb300.pass_params(rays=64, max_dist=96.0, blend=0.2, time_seed=1))
        srv.run(timeout_s=60)
        time.sleep(0.05)   # the device loop has ended (no request within 0.2 ms)
        srv.submit(0, e2, lum_gb300.pass_params(rays=128, max_dist=96.0, blend=0.2, time_seed=2))
        srv.run(timeout_s=60)
        d = srv.poll(8)
        assert len(d) == 2 and (d["status"] == 0).all()
        out[mode] = srv.get_radiance(0)
        if mode == "device":
            assert srv.stats()["launches"] >= 2
        srv.close()
        assert rw.get_world_block(2, 3, 1) == 9   # the context got the edited grid back
        rw.close()
    assert out["device"].tobytes() == out["host"].tobytes()


def test_device_loop_future_arrivals_and_cancel():
    import lum_gb300
    w = worldgen.terrain_world((8, 8, 6), seed=74, n_types=16)
    with lum_gb300.RadianceServer(device_loop=True) as srv:
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0])
        rw.load(w)
        srv.add_world(rw)
        t = srv.now()
        ids = [srv.submit(0, worldgen.edit_request(w.dims, 0.02, seed=75, stream=k),
                          lum_gb300.pass_params(rays=32, time_seed=k), t + 0.02 * (k + 1)) for k in range(3)]
        assert srv.cancel(ids[2]) is True
        srv.run(timeout_s=60)
        d = srv.poll(8)
        assert sorted(d["request"].tolist()) == ids
        ok = d[d["status"] == 0]
        assert len(ok) == 2 and (ok["start_s"] >= ok["arrival_s"] - 1e-6).all()
        assert (d[d["request"] == ids[2]]["status"] == lum_gb300._native.LUMRAD_ECANCELED).all()
        rw.close()


def test_device_loop_rejects_what_it_cannot_run():
    import lum_gb300
    from lum_gb300 import _native as N
    w = worldgen.terrain_world((6, 5, 4), seed=76, n_types=8)
    with lum_gb300.RadianceServer(device_loop=True) as srv:
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0])
        rw.load(w)
        srv.add_world(rw)
        with pytest.raises(lum_gb300.LumRadError) as ei:
            srv.submit(0, np.zeros((1, 4), np.int16), lum_gb300.pass_params(rays=96))
        assert ei.value.code == N.LUMRAD_EINVAL
        big = lum_gb300.RadianceWorld(w.dims, max_block_types=200)
        with pytest.raises(lum_gb300.LumRadError) as ei:
            srv.add_world(big)
        assert ei.value.code == N.LUMRAD_EINVAL
        big.close()
        rw.close()
