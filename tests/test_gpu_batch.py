"""Batches: many worlds in one graph-replayed launch (lumrad_batch_*).

Each world's result in the batch must equal the CPU oracle's for that world alone (worlds are
independent: a ray's seed depends only on its own world's workgroup and ray index), equal the
world run alone through its own context, and the per-world baseline path must agree too.
"""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err

pytestmark = pytest.mark.gpu


def _make(mix, precision="fp32", first=0):
    import lum_gb300
    rws = []
    for i, (w, req, r) in enumerate(mix, start=first):
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=precision)
        rw.load(w)
        rw.set_radiance(random_prev(w, seed=100 + i))
        rws.append(rw)
    return rws


def test_batch_matches_oracle_and_solo_runs():
    import lum_gb300
    import oracle
    mix = worldgen.mixed_worlds(n=7, seed=5, max_dims=(12, 10, 8))
    rws = _make(mix)
    with lum_gb300.RadianceBatch(rws) as b:
        for i, (w, req, r) in enumerate(mix):
            b.set_requests(i, req, lum_gb300.pass_params(rays=r, max_dist=128.0, blend=0.1))
        for seed in (3, 4):
            b.run(seed)
        b.synchronize()
        got = [rw.get_radiance() for rw in rws]
        st = b.stats()
    for i, (w, req, r) in enumerate(mix):
        cur = random_prev(w, seed=100 + i)
        for seed in (3, 4):
            cur, _, _ = oracle.radiance_pass(w, req, rays=r, max_dist=128.0, blend=0.1, time_seed=seed, prev=cur)
        assert rel_err(got[i], cur).max() <= RTOL, (i, rel_err(got[i], cur).max())
    assert st["rays"] == sum(req.shape[0] * r for _, req, r in mix)
    for rw in rws:
        rw.close()


def test_per_world_path_and_autotune_restore():
    import lum_gb300
    mix = worldgen.mixed_worlds(n=5, seed=9, max_dims=(10, 10, 6))
    a = _make(mix)
    bws = _make(mix)
    with lum_gb300.RadianceBatch(a) as ba, lum_gb300.RadianceBatch(bws) as bb:
        for i, (w, req, r) in enumerate(mix):
            p = lum_gb300.pass_params(rays=r, max_dist=200.0, blend=0.2)
            ba.set_requests(i, req, p)
            bb.set_requests(i, req, p)
        best = ba.autotune(repeats=1)
        assert best["max_chunk"] >= 1 and best["pass_ms"] > 0
        ba.run(7)
        bb.run_per_world(7)
        ba.synchronize()
        bb.synchronize()
        for x, y in zip(a, bws):
            assert np.array_equal(x.get_radiance(), y.get_radiance())
    for rw in a + bws:
        rw.close()


def test_batch_results_do_not_depend_on_tuning():
    """The queue settings change only the schedule: single-task claims, the largest chunk the
    queue words carry (LUMRAD_MAX_CHUNK), a divisor that forces one-task claims and one CTA per SM
    all give the default's volumes bit for bit (small batches claim through the CTA queue, a
    batch with more tasks than 32 per warp through the per-warp queue)."""
    import lum_gb300
    from lum_gb300 import _native as N
    big = [(worldgen.terrain_world((56, 48, 8), seed=23, n_types=32), worldgen.all_probes((56, 48, 8)), 256),
           (worldgen.terrain_world((24, 20, 8), seed=24, n_types=32),
            worldgen.probe_subset((24, 20, 8), 0.5, seed=24, stream=0), 128)]   # 179,712 tasks
    for mix in (worldgen.mixed_worlds(n=6, seed=21, max_dims=(10, 10, 6)), big):
        results = {}
        for tuning in (None, (1, 1, 0), (2, N.LUMRAD_MAX_CHUNK, 0), (1000, 32, 0), (2, 32, 1)):
            rws = _make(mix)
            with lum_gb300.RadianceBatch(rws) as b:
                for i, (w, req, r) in enumerate(mix):
                    b.set_requests(i, req, lum_gb300.pass_params(rays=r, max_dist=128.0, blend=0.1))
                if tuning is not None:
                    b.set_tuning(*tuning)
                for seed in (5, 6):
                    b.run(seed)
                b.synchronize()
                results[tuning] = [rw.get_radiance() for rw in rws]
            for rw in rws:
                rw.close()
        for tuning, got in results.items():
            for i in range(len(mix)):
                assert np.array_equal(got[i], results[None][i]), (tuning, i)


def test_batch_in_the_mix_equals_alone():
    """A world's result is identical whether it runs alone or in a batch with others."""
    import lum_gb300
    mix = worldgen.mixed_worlds(n=6, seed=11, max_dims=(12, 12, 6))
    rws = _make(mix)
    solo = _make(mix[2:3], first=2)
    with lum_gb300.RadianceBatch(rws) as b, lum_gb300.RadianceBatch(solo) as s:
        for i, (w, req, r) in enumerate(mix):
            b.set_requests(i, req, lum_gb300.pass_params(rays=r, blend=0.1))
        w, req, r = mix[2]
        s.set_requests(0, req, lum_gb300.pass_params(rays=r, blend=0.1))
        b.run(1)
        s.run(1)
        b.synchronize()
        s.synchronize()
        assert rws[2].get_radiance().tobytes() == solo[0].get_radiance().tobytes()
    for rw in rws + solo:
        rw.close()


@pytest.mark.parametrize("rays", [(96, 64), (512, 32, 128)])
def test_batch_with_probes_spanning_ctas(rays):
    """Batches holding ray counts whose subgroups do not fit one finalize CTA (96, 512) run the
    general finalize kernel (cross-CTA combine) for the whole launch; each world equals the oracle."""
    import lum_gb300
    import oracle
    mix = worldgen.mixed_worlds(n=5, seed=13, max_dims=(9, 8, 6), rays=rays)
    assert any((r // 32) > 1 and 8 % (r // 32) for _, _, r in mix)
    rws = _make(mix, first=20)
    with lum_gb300.RadianceBatch(rws) as b:
        for i, (w, req, r) in enumerate(mix):
            b.set_requests(i, req, lum_gb300.pass_params(rays=r, max_dist=96.0, blend=0.1))
        b.run(7)
        b.synchronize()
        got = [rw.get_radiance() for rw in rws]
    for i, (w, req, r) in enumerate(mix):
        ref, _, _ = oracle.radiance_pass(w, req, rays=r, max_dist=96.0, blend=0.1, time_seed=7,
                                         prev=random_prev(w, seed=120 + i))
        assert rel_err(got[i], ref).max() <= RTOL, (i, r)
    for rw in rws:
        rw.close()
