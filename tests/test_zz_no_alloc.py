"""The occupation-count entry point that allocates no device memory.

Some callers of this library cannot allocate device memory at the moment they need
results: a serving process whose device-memory budget is fully given to resident
trajectories, or code in a stream-ordered section where a cudaMalloc would synchronise
the device.  kmc_pool_occupation_counts_static serves them from a static scratch array.
This file is collected last, so a failure here comes after every other test has run."""
import numpy as np
import pytest

from kmos_gb300 import configs, engine as E

pytestmark = pytest.mark.gpu


def make_pool():
    pool = E.Pool(arena_bytes=256 << 20, max_slots=32)
    slots = []
    for config in (2, 3, 4):
        wl = configs.build(config, n=3, steps=0, sides=[16, 32])
        mid = pool.add_model(wl.program)
        slots += pool.admit_many([mid] * wl.n, wl.sizes, wl.rates, seeds=wl.seeds, rng=E.RNG_PHILOX, trajs=wl.trajs)
    return pool, slots


def test_static_scratch_counts_equal_allocating_counts_on_two_calls():
    pool, slots = make_pool()
    stride = 8  # >= nspecies * sites per cell of every model here
    for steps in (500, 1500):
        pool.run(slots, steps)
        want = pool.occupation_counts(slots, stride)
        got = pool.occupation_counts_static(slots, stride)
        np.testing.assert_array_equal(got, want)
        # a smaller request after a larger one must not see the earlier counters
        np.testing.assert_array_equal(pool.occupation_counts_static(slots[:2], stride), want[:2])
    pool.close()


def test_static_scratch_rejects_requests_beyond_its_size():
    pool, slots = make_pool()
    with pytest.raises(E.KMCError) as err:
        pool.occupation_counts_static(slots, 65)
    assert err.value.code == 1 and "stride" in str(err.value)
    pool.close()
