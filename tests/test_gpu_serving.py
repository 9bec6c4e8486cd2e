"""The continuous-batching server: every request's result is the same alone and in the
mix, admission waits for free arena memory, and dead-locked trajectories retire."""
import numpy as np
import pytest

from kmos_gb300 import configs, serving

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
