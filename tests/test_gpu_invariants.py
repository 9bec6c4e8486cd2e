"""Full-size workloads checked through properties that hold whatever the length of the
run: after every benchmark configuration's whole batch (2048 / 4096 / 8192 trajectories)
has run, sampled trajectories of every lattice size must have
  * avail_sites(p, :, 2) the inverse of avail_sites(p, 1..n_p, 1), zeros past n_p;
  * exactly the processes their lattice enables listed (the oracle derives those from
    the lattice alone, by touch-ups: oracle_rebuild_tables);
  * procstat summing to kmc_step and a positive, finite kmc_time.
The table checks are tests/table_invariants.py (tests/test_planted_mistakes.py shows
them catching planted mistakes).  The oracle cannot replay millions of steps of
thousands of trajectories; these checks need no replay."""
import numpy as np
import pytest

from kmos_gb300 import configs, engine as E
from table_invariants import table_violations

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("config,steps", [(3, 40000), (2, 40000), (4, 20000)])
def test_full_size_batch_invariants(config, steps):
    wl = configs.build(config, steps=steps)
    probe = E.Pool(arena_bytes=1 << 20, max_slots=1)
    mid0 = probe.add_model(wl.program)
    need = sum(probe.slot_bytes(mid0, s) for s in wl.sizes)
    probe.close()
    pool = E.Pool(arena_bytes=need + (64 << 20), max_slots=wl.n)
    mid = pool.add_model(wl.program)
    slots = []
    for i in range(0, wl.n, 1024):
        slots += pool.admit_many([mid] * len(wl.sizes[i:i + 1024]), wl.sizes[i:i + 1024], wl.rates[i:i + 1024],
                                 seeds=wl.seeds[i:i + 1024], rng=E.RNG_PHILOX, trajs=wl.trajs[i:i + 1024])
    pool.set_launch(0, 0)
    pool.run(slots, steps)
    P = wl.program.nproc
    ps, _ig, times, ksteps, status = pool.results(slots, P)
    assert set(status.tolist()) <= {0, 3}
    assert (ps.sum(axis=1) == ksteps).all()
    assert np.isfinite(times).all() and (times[ksteps > 0] > 0).all()
    # one trajectory of every lattice size, and a few more
    picks, seen = [], set()
    for i, sz in enumerate(wl.sizes):
        if sz not in seen:
            seen.add(sz)
            picks.append(i)
    picks += [1, wl.n // 2, wl.n - 1]
    for i in sorted(set(picks))[:8]:
        s = slots[i]
        as1, as2 = pool.tables(s)
        bad = table_violations(wl.program, wl.sizes[i], pool.lattice(s), as1, as2, pool.nr_of_sites(s))
        assert bad == [], (config, i, bad[:3])
    pool.close()
