"""Host-side fault injection: invalid arguments return their status (nothing aborts, nothing is
half-applied), and the context still runs a correct pass afterwards."""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err

pytestmark = pytest.mark.gpu


def _code(fn, *a):
    import lum_gb300
    with pytest.raises(lum_gb300.LumRadError) as ei:
        fn(*a)
    return ei.value.code


def test_create_rejects_bad_settings():
    import lum_gb300
    from lum_gb300 import _native as N
    for dims, slots, prec in [((0, 4, 4), 8, "fp32"), ((2048, 1, 1), 8, "fp32"), ((4, 4, 4), 0, "fp32"),
                              ((4, 4, 4), 5000, "fp32")]:
        assert _code(lum_gb300.RadianceWorld, dims, slots, prec) == N.LUMRAD_EINVAL


def test_bad_calls_leave_the_context_usable():
    import lum_gb300
    import oracle
    from lum_gb300 import _native as N
    w = worldgen.terrain_world((6, 5, 4), seed=51, n_types=8)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        prev = random_prev(w)
        rw.set_radiance(prev)
        assert _code(rw.pass_stats) == N.LUMRAD_ESTATE   # no pass yet
        assert _code(rw.get_hits) == N.LUMRAD_ESTATE
        req = worldgen.all_probes(w.dims)
        for bad in [dict(rays=33), dict(rays=0), dict(rays=2048), dict(max_dist=0.0), dict(max_dist=-1.0),
                    dict(max_dist=float("nan")), dict(blend=-0.1), dict(blend=1.5), dict(size=-1),
                    dict(size=2, shift=2)]:
            assert _code(rw.radiance_pass, req, lum_gb300.pass_params(**bad)) == N.LUMRAD_EINVAL, bad
        assert _code(rw.set_world_block, 6, 0, 0, 1) == N.LUMRAD_EINVAL
        assert _code(rw.get_world_block, 0, -1, 0) == N.LUMRAD_EINVAL
        assert _code(rw.load_block, w.palette.shape[0], np.zeros((16, 16, 16), np.uint8)) == N.LUMRAD_EINVAL
        assert _code(rw.load_block, -1, np.zeros((16, 16, 16), np.uint8)) == N.LUMRAD_EINVAL
        assert _code(rw.request_update, 0, 0, 4) == N.LUMRAD_EINVAL
        assert _code(rw.build_dirty_list, np.array([[6, 0, 0, 1]], np.int16)) == N.LUMRAD_EINVAL
        assert _code(rw.blockify, 0, []) == N.LUMRAD_EINVAL
        assert _code(rw.blockify, 1, [(5, (0, 0, 0, 1), (0, 0, 0))]) == N.LUMRAD_EINVAL   # unknown model
        # nothing above changed the world: a pass still matches the oracle
        p = dict(rays=64, max_dist=128.0, blend=0.1, time_seed=2)
        rw.radiance_pass(req, lum_gb300.pass_params(**p))
        got = rw.get_radiance()
        ref, _, _ = oracle.radiance_pass(w, req, prev=prev, **p)
        assert rel_err(got, ref).max() <= RTOL


def test_batch_and_server_reject_bad_requests():
    import lum_gb300
    from lum_gb300 import _native as N
    w = worldgen.terrain_world((6, 5, 4), seed=52, n_types=8)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        req = worldgen.all_probes(w.dims)
        with lum_gb300.RadianceBatch([rw]) as b:
            assert _code(b.set_requests, 1, req, lum_gb300.pass_params()) == N.LUMRAD_EINVAL
            assert _code(b.set_requests, 0, req, lum_gb300.pass_params(size=0)) == N.LUMRAD_EINVAL
            assert _code(b.set_requests, 0, req, lum_gb300.pass_params(record_hits=True)) == N.LUMRAD_EINVAL
            assert _code(b.run, 0) == N.LUMRAD_ESTATE   # no requests set yet
            # a claimed chunk's task count has 12 bits in the march queue's words
            assert _code(b.set_tuning, 2, 4096, 0) == N.LUMRAD_EINVAL
            assert _code(b.set_tuning, 2, -1, 0) == N.LUMRAD_EINVAL
            b.set_tuning(2, 4095, 0)
            assert _code(b.stats) == N.LUMRAD_ESTATE
        with lum_gb300.RadianceServer() as srv:
            i = srv.add_world(rw)
            assert _code(srv.add_world, rw) == N.LUMRAD_ESTATE   # already registered
            assert _code(srv.submit, i + 1, np.zeros((1, 4), np.int16), lum_gb300.pass_params()) == N.LUMRAD_EINVAL
            assert _code(srv.submit, i, np.array([[0, 5, 0, 1]], np.int16), lum_gb300.pass_params()) == N.LUMRAD_EINVAL
            assert _code(srv.submit, i, np.zeros((1, 4), np.int16), lum_gb300.pass_params(rays=40)) == N.LUMRAD_EINVAL
            assert _code(srv.get_radiance, i + 1) == N.LUMRAD_EINVAL
            assert srv.cancel(12345) is False
        with pytest.raises(Exception):
            lum_gb300.RadianceServer(precision="fp32", max_inflight=9)


def test_finalize_error_word_reported_and_context_recovers():
    """The finalize kernel's error path, driven from the host: a pass whose probes span finalize
    CTAs (R = 96: 3 subgroups, 8 per CTA) launched with the variant that has no cross-CTA combine.
    That kernel stores nothing for such probes and sets bit 2 of the context's error word; the next
    call that reads the word returns LUMRAD_EDEVICE, resets it, and the context's next pass equals
    the oracle (on the volume the failed pass left: its copy of the previous one)."""
    import lum_gb300
    import oracle
    from lum_gb300 import _native as N
    w = worldgen.terrain_world((7, 6, 5), seed=53, n_types=8)
    req = worldgen.all_probes(w.dims)
    prev = random_prev(w)
    p = dict(rays=96, max_dist=128.0, blend=0.1)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        N.check(rw.lib.lumrad_test_hook(rw.h, N.LUMRAD_TEST_LEAN_FINALIZE, 1.0))
        rw.radiance_pass(req, lum_gb300.pass_params(time_seed=1, **p))   # enqueued; not awaited
        with pytest.raises(lum_gb300.LumRadError) as ei:
            rw.synchronize()
        assert ei.value.code == N.LUMRAD_EDEVICE and "spanning CTAs" in str(ei.value)
        rw.synchronize()   # the word was reset
        assert np.array_equal(rw.get_radiance(), np.clip(prev, 0, 1))   # nothing was stored
        N.check(rw.lib.lumrad_test_hook(rw.h, N.LUMRAD_TEST_LEAN_FINALIZE, 0.0))
        rw.radiance_pass(req, lum_gb300.pass_params(time_seed=2, **p))
        got = rw.get_radiance()
    ref, _, _ = oracle.radiance_pass(w, req, prev=prev, time_seed=2, **p)
    assert rel_err(got, ref).max() <= RTOL


def test_unknown_test_hook_rejected():
    import lum_gb300
    from lum_gb300 import _native as N
    with lum_gb300.RadianceWorld((2, 2, 2), max_block_types=2) as rw:
        assert rw.lib.lumrad_test_hook(rw.h, 99, 1.0) == N.LUMRAD_EINVAL
