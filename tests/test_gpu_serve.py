"""Relight server (lumrad_server_*): continuously batched edit + relight requests.

Each request's result must equal the CPU oracle's pass over the edited world with the request's
dirty-probe list; a world's result must be identical alone and in a mix with other worlds'
requests (several launches in flight); the HBM budget must gate admission without changing any
result."""
import dataclasses

import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err

pytestmark = pytest.mark.gpu

DIMS = [(8, 8, 8), (12, 6, 5), (16, 16, 4), (5, 9, 7)]
RAYS = [64, 32, 128, 64]


def _worlds():
    return [worldgen.terrain_world(d, seed=40 + i, n_types=32) for i, d in enumerate(DIMS)]


def _requests(n_per_world, seed=1):
    """[(world, edits, rays, time_seed)] interleaved over the worlds."""
    out = []
    for k in range(n_per_world):
        for i, d in enumerate(DIMS):
            e = worldgen.edit_request(d, 0.01 + 0.04 * ((k + i) % 3) / 2, seed=seed, stream=100 * i + k)
            out.append((i, e, RAYS[i], 1000 * i + k))
    return out


def _server(worlds, which, **kw):
    import lum_gb300
    srv = lum_gb300.RadianceServer(**kw)
    rws = []
    for i in which:
        w = worlds[i]
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0])
        rw.load(w)
        rw.set_radiance(random_prev(w, seed=200 + i))
        srv.add_world(rw)
        rws.append(rw)
    return srv, rws


def _submit(srv, reqs, which):
    import lum_gb300
    idx = {w: k for k, w in enumerate(which)}
    for i, e, r, seed in reqs:
        if i in idx:
            srv.submit(idx[i], e, lum_gb300.pass_params(rays=r, max_dist=64.0, blend=0.1, time_seed=seed))


def test_server_matches_oracle():
    import oracle
    worlds = _worlds()
    reqs = _requests(3)
    which = list(range(len(DIMS)))
    srv, rws = _server(worlds, which, max_inflight=2)
    _submit(srv, reqs, which)
    srv.run(timeout_s=300)
    done = srv.poll()
    assert len(done) == len(reqs) and (done["status"] == 0).all()
    got = [srv.get_radiance(i) for i in which]
    for i in which:
        w = worlds[i]
        cur = random_prev(w, seed=200 + i)
        grid = w.grid
        for j, e, r, seed in reqs:
            if j != i:
                continue
            grid = worldgen.apply_edits(grid, e)
            req = worldgen.dirty_probes(w.dims, e, 2)
            we = dataclasses.replace(w, grid=grid)
            cur, _, _ = oracle.radiance_pass(we, req, rays=r, max_dist=64.0, blend=0.1, time_seed=seed, prev=cur)
        err = rel_err(got[i], cur).max()
        assert err <= RTOL, (i, err)
        # the server's grid is the edited grid
        for x, y, z in [(0, 0, 0), (w.dims[0] - 1, w.dims[1] - 1, w.dims[2] - 1)]:
            assert rws[i].get_world_block(x, y, z) == grid[z, y, x]
    # every request's probe count is its dirty list's length
    lens = {}
    for j, e, r, seed in reqs:
        lens.setdefault(j, []).append(worldgen.dirty_probes(DIMS[j], e, 2).shape[0])
    for j in which:
        assert list(done[done["world"] == j]["probes"]) == lens[j]
    srv.close()
    for rw in rws:
        rw.close()


def test_alone_equals_mix():
    worlds = _worlds()
    reqs = _requests(4, seed=2)
    mix, mix_rws = _server(worlds, [0, 1, 2, 3], max_inflight=3)
    _submit(mix, reqs, [0, 1, 2, 3])
    mix.run(timeout_s=300)
    st = mix.stats()
    assert st["requests"] == len(reqs)
    for i in range(len(DIMS)):
        alone, rws = _server(worlds, [i], max_inflight=1)
        _submit(alone, reqs, [i])
        alone.run(timeout_s=300)
        assert alone.get_radiance(0).tobytes() == mix.get_radiance(i).tobytes(), i
        alone.close()
        for rw in rws:
            rw.close()
    mix.close()
    for rw in mix_rws:
        rw.close()


def test_budget_gates_admission():
    import lum_gb300
    worlds = _worlds()
    reqs = _requests(2, seed=3)
    # one launch slot: a launch takes every due request (with more slots they are split)
    free, free_rws = _server(worlds, [0, 1, 2, 3], max_inflight=1)
    _submit(free, reqs, [0, 1, 2, 3])
    free.run(timeout_s=300)
    st0 = free.stats()
    assert st0["max_requests_in_launch"] == 4
    # room for the worlds, the launch buffers and about one request at a time (a request here
    # needs at most ~10 KB: its dirty list bound, edits and table entry)
    headroom = 12_000
    tight_budget = st0["resident_bytes"] + st0["launch_bytes"] + headroom
    tight, tight_rws = _server(worlds, [0, 1, 2, 3], max_inflight=1, hbm_budget_bytes=tight_budget)
    _submit(tight, reqs, [0, 1, 2, 3])
    tight.run(timeout_s=300)
    st1 = tight.stats()
    assert st1["requests"] == len(reqs)
    # every admitted byte fits: resident worlds + launch buffers + requests in flight
    assert 0 < st1["peak_inflight_bytes"] and st1["peak_device_bytes"] <= tight_budget
    assert st1["max_requests_in_launch"] < 4 or st1["evictions"] > 0
    for i in range(4):
        assert tight.get_radiance(i).tobytes() == free.get_radiance(i).tobytes()
    for s in (free, tight):
        s.close()
    for rw in free_rws + tight_rws:
        rw.close()


def test_request_that_never_fits_is_refused():
    import lum_gb300
    worlds = _worlds()
    probe, rws = _server(worlds, [2])
    st = probe.stats()
    probe.close()
    for rw in rws:
        rw.close()
    tiny, rws = _server(worlds, [2], hbm_budget_bytes=st["resident_bytes"] + st["launch_bytes"] + 1000)
    before = tiny.get_radiance(0)
    big = worldgen.edit_request(DIMS[2], 0.5, seed=9, stream=0)
    tiny.submit(0, big, lum_gb300.pass_params(rays=64))
    tiny.run(timeout_s=60)
    d = tiny.poll()
    assert len(d) == 1 and d["status"][0] == lum_gb300._native.LUMRAD_ENOMEM
    assert tiny.get_radiance(0).tobytes() == before.tobytes()
    x, y, z = (int(v) for v in big[-1][:3])
    assert rws[0].get_world_block(x, y, z) == worlds[2].grid[z, y, x]
    tiny.close()
    for rw in rws:
        rw.close()


def test_owned_context_rejects_direct_calls():
    import lum_gb300
    worlds = _worlds()
    srv, rws = _server(worlds, [0])
    with pytest.raises(lum_gb300.LumRadError) as ei:
        rws[0].radiance_pass(worldgen.all_probes(DIMS[0]), lum_gb300.pass_params())
    assert ei.value.code == lum_gb300._native.LUMRAD_ESTATE
    with pytest.raises(lum_gb300.LumRadError):
        rws[0].set_world_block(0, 0, 0, 3)
    srv.close()
    # released by the server: direct calls work again
    rws[0].radiance_pass(worldgen.all_probes(DIMS[0]), lum_gb300.pass_params())
    rws[0].synchronize()
    rws[0].close()


def test_eviction_under_a_tight_budget_changes_nothing():
    """A budget that holds the launch buffers and about two worlds: the server evicts and
    re-admits worlds, and every world ends bit-identical to the unconstrained server's."""
    import lum_gb300
    worlds = _worlds()
    reqs = _requests(3, seed=4)
    free, free_rws = _server(worlds, [0, 1, 2, 3])
    _submit(free, reqs, [0, 1, 2, 3])
    free.run(timeout_s=300)
    st0 = free.stats()
    budget = st0["launch_bytes"] + st0["resident_bytes"] / 2 + 40_000   # about two of the four worlds
    tight, tight_rws = _server(worlds, [0, 1, 2, 3], hbm_budget_bytes=budget)
    _submit(tight, reqs, [0, 1, 2, 3])
    tight.run(timeout_s=300)
    st1 = tight.stats()
    assert st1["requests"] == len(reqs) and st1["evictions"] > 0 and st1["readmissions"] > 0
    assert st1["peak_device_bytes"] <= budget
    for i in range(4):   # evicted worlds read from their host copy, resident ones from the device
        assert tight.get_radiance(i).tobytes() == free.get_radiance(i).tobytes()
    tight.close()
    # the contexts come back resident and usable
    for rw in tight_rws:
        rw.radiance_pass(worldgen.all_probes(rw.dims)[:5], lum_gb300.pass_params(rays=32))
        rw.synchronize()
    free.close()
    for rw in free_rws + tight_rws:
        rw.close()


def test_cancel_before_launch():
    import lum_gb300
    worlds = _worlds()
    reqs = _requests(2, seed=5)
    a, a_rws = _server(worlds, [0, 1])
    b, b_rws = _server(worlds, [0, 1])
    mine = [(i, e, lum_gb300.pass_params(rays=r, max_dist=64.0, blend=0.1, time_seed=seed))
            for i, e, r, seed in reqs if i in (0, 1)]
    skip = [k for k, (i, _, _) in enumerate(mine) if i == 1][1]   # world 1's second request
    dropped = None
    for k, (i, e, p) in enumerate(mine):
        rid = a.submit(i, e, p)
        if k == skip:
            dropped = rid
        else:
            b.submit(i, e, p)
    assert a.cancel(dropped) is True
    assert a.cancel(dropped) is False
    a.run(timeout_s=120)
    b.run(timeout_s=120)
    d = a.poll()
    assert (d[d["request"] == dropped]["status"] == lum_gb300._native.LUMRAD_ECANCELED).all()
    for i in (0, 1):
        assert a.get_radiance(i).tobytes() == b.get_radiance(i).tobytes()
    for s in (a, b):
        s.close()
    for rw in a_rws + b_rws:
        rw.close()


def test_server_with_probes_spanning_ctas():
    """Requests of 96 and 512 rays (subgroups combined across finalize CTAs) in the same launches
    as 64-ray ones: the general finalize kernel; each world equals the oracle's chain of passes."""
    import oracle
    worlds = _worlds()
    which = [0, 1, 3]
    rays = {0: 96, 1: 512, 3: 64}
    reqs = []
    for k in range(2):
        for i in which:
            e = worldgen.edit_request(DIMS[i], 0.02, seed=7, stream=10 * i + k)
            reqs.append((i, e, rays[i], 500 + 10 * i + k))
    srv, rws = _server(worlds, which, max_inflight=2)
    _submit(srv, reqs, which)
    srv.run(timeout_s=300)
    done = srv.poll()
    assert len(done) == len(reqs) and (done["status"] == 0).all()
    for k, i in enumerate(which):
        w = worlds[i]
        cur = random_prev(w, seed=200 + i)
        grid = w.grid
        for j, e, r, seed in reqs:
            if j != i:
                continue
            grid = worldgen.apply_edits(grid, e)
            we = dataclasses.replace(w, grid=grid)
            cur, _, _ = oracle.radiance_pass(we, worldgen.dirty_probes(w.dims, e, 2), rays=r, max_dist=64.0,
                                             blend=0.1, time_seed=seed, prev=cur)
        assert rel_err(srv.get_radiance(k), cur).max() <= RTOL, i
    srv.close()
    for rw in rws:
        rw.close()


@pytest.mark.parametrize("device_loop", [False, True])
def test_queue_bound_sheds_late_requests(device_loop):
    """max_queue_ms: requests that waited past the bound when their turn came complete with
    LUMRAD_ETIMEOUT without running (their edits not applied); every request that ran started within
    the bound, and the worlds equal a server without the bound that ran only those requests."""
    import lum_gb300
    from lum_gb300 import _native as N
    worlds = _worlds()
    which = list(range(len(DIMS)))
    # all due at one moment (50 ms after submission): the queue builds up; the device loop needs
    # more than its publish window (2 x 64 per lane) to hold requests back on the host
    reqs = _requests(100 if device_loop else 12, seed=9)
    bound_ms = 0.3
    srv, rws = _server(worlds, which, device_loop=device_loop, max_queue_ms=bound_ms)
    due = srv.now() + 0.05
    for i, e, r, seed in reqs:
        srv.submit(i, e, lum_gb300.pass_params(rays=r, max_dist=64.0, blend=0.1, time_seed=seed), due)
    srv.run(timeout_s=300)
    done = srv.poll(len(reqs) + 8)
    assert len(done) == len(reqs)
    ok = done[done["status"] == 0]
    shed = done[done["status"] == N.LUMRAD_ETIMEOUT]
    assert len(ok) + len(shed) == len(reqs)
    assert len(ok) >= 1 and len(shed) > 0   # (how many run depends on the host's launch pace)
    assert srv.stats()["shed"] == len(shed)
    assert (ok["start_s"] - ok["arrival_s"] <= bound_ms * 1e-3 + 1e-4).all()
    got = [srv.get_radiance(k) for k in which]
    srv.close()
    for rw in rws:
        rw.close()
    ran = set(ok["request"].tolist())
    ref, rrws = _server(worlds, which)
    # the same submission order, only the requests that ran (ids are 0, 1, ... in submission order)
    kept = [q for rid, q in enumerate(reqs) if rid in ran]
    _submit(ref, kept, which)
    ref.run(timeout_s=300)
    d2 = ref.poll(len(kept) + 8)
    assert len(d2) == len(kept) and (d2["status"] == 0).all()
    for k in which:
        assert ref.get_radiance(k).tobytes() == got[k].tobytes(), k
    ref.close()
    for rw in rrws:
        rw.close()
