"""The continuous-batching server: every request's result is the same alone and in the
mix, admission waits for free arena memory, and dead-locked trajectories retire."""
import numpy as np
import pytest

from kmos_gb300 import configs, engine as E, serving

pytestmark = pytest.mark.gpu


def small_stream(n=24, seed=11):
    reqs, progs = configs.serving_requests(rate=2000.0, duration=1.0, seed=seed, steps_scale=0.002,
                                           side_range=(10, 40))
    return reqs[:n], progs


def serve(reqs, progs, arena=512 << 20, quantum=2000):
    srv = serving.Server(arena_bytes=arena, max_slots=256, quantum=quantum)
    for k, p in progs.items():
        srv.add_model(k, p)
    out = srv.serve(reqs)
    srv.close()
    return {r.rid: r for r in out}


def clone(r):
    return serving.Request(model=r.model, size=r.size, rates=r.rates, steps=r.steps, seed=r.seed,
                           traj_id=r.traj_id, rid=r.rid, arrival=0.0)


def test_each_result_is_the_same_alone_and_in_the_mix():
    reqs, progs = small_stream()
    mixed = serve(reqs, progs)
    assert len(mixed) == len(reqs)
    for r in reqs[:8]:
        alone = serve([clone(r)], progs)[r.rid]
        a, b = alone.result, mixed[r.rid].result
        assert a["kmc_step"] == b["kmc_step"] and a["status"] == b["status"]
        np.testing.assert_array_equal(a["procstat"], b["procstat"])
        assert a["kmc_time"] == b["kmc_time"]
        np.testing.assert_array_equal(a["coverage"], b["coverage"])
        np.testing.assert_array_equal(a["integ_rates"], b["integ_rates"])


def test_admission_waits_for_free_memory():
    reqs, progs = small_stream(n=16)
    # size the arena for about three of the largest trajectories at a time
    probe = serving.Server(arena_bytes=1 << 20, max_slots=4)
    for k, p in progs.items():
        probe.add_model(k, p)
    biggest = max(probe.pool.slot_bytes(probe.models[r.model].model_id, r.size) for r in reqs)
    probe.close()
    out = serve([clone(r) for r in reqs], progs, arena=3 * biggest + 4096, quantum=500)
    assert len(out) == 16
    assert all(r.result is not None for r in out.values())
    admitted = sorted(r.admitted for r in out.values())
    assert admitted[-1] > admitted[0]  # later requests waited for earlier ones to finish


def test_quantum_size_does_not_change_results():
    reqs, progs = small_stream(n=10, seed=3)
    a = serve([clone(r) for r in reqs], progs, quantum=700)
    b = serve([clone(r) for r in reqs], progs, quantum=100000)
    for rid in a:
        np.testing.assert_array_equal(a[rid].result["procstat"], b[rid].result["procstat"])
        assert a[rid].result["kmc_time"] == b[rid].result["kmc_time"]


def test_srpt_evicts_and_results_do_not_change():
    """Shortest-remaining-first with eviction: two long trajectories fill the arena, then
    short requests arrive; a long one is saved to host memory, the short ones run, and the
    long one is restored later.  Every result equals the request run alone (state images
    restore bit for bit)."""
    reqs, progs = small_stream(n=40)
    tmpl = next(r for r in reqs if r.model == "c3")
    longs = [serving.Request(model="c3", size=(40, 40), rates=tmpl.rates, steps=20000, seed=3, traj_id=i,
                             rid=100 + i, arrival=0.0) for i in range(2)]
    shorts = [serving.Request(model="c3", size=(16, 16), rates=tmpl.rates, steps=600, seed=4, traj_id=10 + i,
                              rid=200 + i, arrival=0.05) for i in range(6)]
    probe = serving.Server(arena_bytes=1 << 20, max_slots=4)
    for k, p in progs.items():
        probe.add_model(k, p)
    need_long = probe.pool.slot_bytes(probe.models["c3"].model_id, (40, 40))
    need_short = probe.pool.slot_bytes(probe.models["c3"].model_id, (16, 16))
    probe.close()
    assert need_short > 4096
    srv = serving.Server(arena_bytes=2 * need_long + 1024, max_slots=64, quantum=300, policy="srpt")
    for k, p in progs.items():
        srv.add_model(k, p)
    out = {r.rid: r for r in srv.serve(longs + shorts)}
    evicted = srv.evicted
    srv.close()
    assert len(out) == len(longs) + len(shorts) and evicted > 0
    assert any(out[r.rid].evictions > 0 for r in longs)
    # the short requests finished before the long ones
    assert max(out[r.rid].done for r in shorts) < max(out[r.rid].done for r in longs)
    for r in longs + shorts[:2]:
        alone = serve([clone(r)], progs, arena=need_long + 4096, quantum=300)[r.rid]
        a, b = alone.result, out[r.rid].result
        assert a["kmc_step"] == b["kmc_step"] and a["kmc_time"] == b["kmc_time"]
        np.testing.assert_array_equal(a["procstat"], b["procstat"])
        np.testing.assert_array_equal(a["integ_rates"], b["integ_rates"])
        np.testing.assert_array_equal(a["coverage"], b["coverage"])


def test_session_continues_one_trajectory():
    """Two requests of one session (the second with new rates) end in the state of one
    trajectory run straight through with the rates changed at the same step, and the
    second request's TOF covers its own interval."""
    reqs, progs = small_stream(n=40)
    tmpl = next(r for r in reqs if r.model == "c2")
    r2 = [x * 1.5 for x in tmpl.rates]
    a = serving.Request(model="c2", size=(16, 16), rates=tmpl.rates, steps=1200, seed=9, traj_id=3, rid=1,
                        session="s1")
    b = serving.Request(model="c2", size=(16, 16), rates=r2, steps=1800, seed=9, traj_id=3, rid=2, session="s1",
                        keep=False, arrival=0.0)
    srv = serving.Server(arena_bytes=64 << 20, max_slots=16, quantum=500)
    for k, p in progs.items():
        srv.add_model(k, p)
    out = {r.rid: r for r in srv.serve([a, b])}
    assert not srv.sessions  # keep=False ended the session
    srv.close()
    # the same trajectory straight through, rates changed after 1200 steps
    pool = E.Pool(arena_bytes=64 << 20, max_slots=2)
    mid = pool.add_model(progs["c2"])
    s = pool.admit(mid, (16, 16), tmpl.rates, seed=9, rng=E.RNG_PHILOX, traj=3)
    pool.run([s], 1200)
    ps1, _ig1, t1, k1, _st = pool.results([s], progs["c2"].nproc)
    pool.set_rates(s, r2)
    pool.run([s], 1800)
    ps, ig, t, k, st = pool.results([s], progs["c2"].nproc)
    rb = out[2].result
    assert rb["kmc_step"] == k[0] == 3000 and rb["kmc_time"] == t[0]
    np.testing.assert_array_equal(rb["procstat"], ps[0])
    np.testing.assert_array_equal(rb["integ_rates"], ig[0])
    assert out[1].result["kmc_step"] == k1[0] == 1200
    assert abs(rb["interval_time"] - (t[0] - t1[0])) <= 1e-12 * t[0]
    pool.close()


def test_idle_session_moves_to_host_memory_under_pressure():
    """An idle session is saved to host memory when a new request needs its room, and
    its next request continues it bit for bit."""
    reqs, progs = small_stream(n=40)
    tmpl = next(r for r in reqs if r.model == "c3")
    probe = serving.Server(arena_bytes=1 << 20, max_slots=4)
    for k, p in progs.items():
        probe.add_model(k, p)
    need = probe.pool.slot_bytes(probe.models["c3"].model_id, (24, 24))
    probe.close()
    srv = serving.Server(arena_bytes=need + 4096, max_slots=8, quantum=400)
    for k, p in progs.items():
        srv.add_model(k, p)
    first = serving.Request(model="c3", size=(24, 24), rates=tmpl.rates, steps=800, seed=5, traj_id=1, rid=1,
                            session="x")
    other = serving.Request(model="c3", size=(24, 24), rates=tmpl.rates, steps=300, seed=6, traj_id=2, rid=2,
                            arrival=0.0)
    srv.serve([first])
    srv.serve([other])  # needs the whole arena: the idle session goes to host memory
    assert srv.sessions["x"].slot < 0 and srv.sessions["x"].image is not None and srv.evicted >= 1
    again = serving.Request(model="c3", size=(24, 24), rates=None, steps=700, seed=5, traj_id=1, rid=3,
                            session="x", keep=False)
    out = {r.rid: r for r in srv.serve([again])}
    srv.close()
    pool = E.Pool(arena_bytes=need + 4096, max_slots=2)
    mid = pool.add_model(progs["c3"])
    s = pool.admit(mid, (24, 24), tmpl.rates, seed=5, rng=E.RNG_PHILOX, traj=1)
    pool.run([s], 800)
    pool.run([s], 700)
    ps, ig, t, k, st = pool.results([s], progs["c3"].nproc)
    pool.close()
    rr = out[3].result
    assert rr["kmc_step"] == k[0] == 1500 and rr["kmc_time"] == t[0]
    np.testing.assert_array_equal(rr["procstat"], ps[0])
    np.testing.assert_array_equal(rr["integ_rates"], ig[0])


def test_sampled_request_matches_pool_sampling():
    """A request with samples > 0 returns get_std_sampled_data's averages, taken on the
    device at the batch boundaries; they equal kmc_pool_sample_run on the same
    trajectory alone."""
    reqs, progs = small_stream(n=40)
    tmpl = next(r for r in reqs if r.model == "c2")
    req = serving.Request(model="c2", size=(16, 16), rates=tmpl.rates, steps=2003, seed=4, traj_id=7, rid=1,
                          samples=4)
    other = serving.Request(model="c3", size=(12, 12), rates=next(r for r in reqs if r.model == "c3").rates,
                            steps=900, seed=4, traj_id=8, rid=2)
    srv = serving.Server(arena_bytes=64 << 20, max_slots=16, quantum=170)  # quanta cross the boundaries
    for k, p in progs.items():
        srv.add_model(k, p)
    out = {r.rid: r for r in srv.serve([req, other])}
    srv.close()
    got = out[1].result["sampled"]
    assert out[1].result["kmc_step"] == 4 * 500
    pool = E.Pool(arena_bytes=64 << 20, max_slots=2)
    mid = pool.add_model(progs["c2"])
    s = pool.admit(mid, (16, 16), tmpl.rates, seed=4, rng=E.RNG_PHILOX, traj=7)
    want = pool.sample_run([s], 4, 500)
    pool.close()
    nocc = want["occ"].shape[1]
    np.testing.assert_array_equal(got["occupation"].ravel(), want["occ"][0, :nocc])
    assert got["total_time"] == want["times"][0, 0] and got["kmc_steps"] == want["steps"][0] == 2000
