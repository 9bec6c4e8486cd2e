"""The occupation-count entry point that allocates no device memory.

Some callers of this library cannot allocate device memory at the moment they need
results: a serving process whose device-memory budget is fully given to resident
trajectories, or a real-time loop where a cudaMalloc would synchronise the device.
kmc_pool_occupation_counts_static serves them from a static scratch array.
This file is collected last, so a failure here comes after every other test has run."""
import numpy as np
import pytest

from kmos_gb300 import configs, engine as E
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make_pool():
    pool = E.Pool(arena_bytes=256 << 20, max_slots=32)
    slots, wls = [], []
    for config in (2, 3, 4):
        wl = configs.build(config, n=3, steps=0, sides=[16, 32])
        mid = pool.add_model(wl.program)
        slots += pool.admit_many([mid] * wl.n, wl.sizes, wl.rates, seeds=wl.seeds, rng=E.RNG_PHILOX, trajs=wl.trajs)
        wls += [(wl, i) for i in range(wl.n)]
    return pool, slots, wls


def counters_per_slot(wl) -> int:
    """nspecies * sites per unit cell: the occupation counters of one slot."""
    return int(wl.program.words[4]) * int(wl.program.words[6])


def oracle_counts(wl, i, steps, stride):
    """Occupation counts of trajectory i after `steps` kMC steps, from the oracle's lattice."""
    o = O.Oracle(wl.program, wl.sizes[i], seed=wl.seeds[i], rng=O.RNG_PHILOX, traj=wl.trajs[i])
    o.set_rates(wl.rates[i])
    o.update_accum_rate()
    o.do_kmc_steps(steps)
    lat = o.export()["lattice"].ravel()
    ns, sp = int(wl.program.words[4]), int(wl.program.words[6])
    out = np.zeros(stride, np.int64)
    for s, spc in enumerate(lat):
        if 0 <= spc < ns:
            out[spc * sp + s % sp] += 1
    return out


def test_static_scratch_counts_equal_allocating_counts_on_two_calls():
    pool, slots, wls = make_pool()
    stride = max(counters_per_slot(wl) for wl, _ in wls)
    assert stride <= 64
    total = 0
    for steps in (500, 1500):
        pool.run(slots, steps)
        total += steps
        want = pool.occupation_counts(slots, stride)
        got = pool.occupation_counts_static(slots, stride)
        np.testing.assert_array_equal(got, want)
        # a smaller request after a larger one must not see the earlier counters
        np.testing.assert_array_equal(pool.occupation_counts_static(slots[:2], stride), want[:2])
    # and both equal the oracle's counts for a trajectory of each model
    for k in (0, 3, 6):
        wl, i = wls[k]
        np.testing.assert_array_equal(got[k], oracle_counts(wl, i, total, stride))
    pool.close()


def test_static_scratch_rejects_requests_beyond_its_size():
    pool, slots, _wls = make_pool()
    with pytest.raises(E.KMCError) as err:
        pool.occupation_counts_static(slots, 65)
    assert err.value.code == 1 and "stride" in str(err.value)
    pool.close()


def test_short_stride_is_refused_by_both_entry_points():
    """A row of `stride` counters must hold nspecies * spuck of every listed slot's
    model; a shorter stride would make rows overlap (or run past the output)."""
    pool, slots, wls = make_pool()
    need = max(counters_per_slot(wl) for wl, _ in wls)
    for fn in (pool.occupation_counts, pool.occupation_counts_static):
        with pytest.raises(E.KMCError) as err:
            fn(slots, need - 1)
        assert err.value.code == 1 and "stride" in str(err.value)
        with pytest.raises(E.KMCError):
            fn(slots, 1)
    # the pool stays usable, and an exact stride is accepted
    pool.run(slots, 100)
    np.testing.assert_array_equal(pool.occupation_counts_static(slots, need), pool.occupation_counts(slots, need))
    pool.close()
