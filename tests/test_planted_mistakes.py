"""The checks the GPU tests rely on, shown to catch mistakes planted in oracle
trajectories on the CPU: a lattice change without its touch-up, a swap-remove that
forgets a position entry, two list entries swapped, all caught by the invariants the
full-size GPU batches are checked with (tests/table_invariants.py); and a rate constant
slightly off shows in the comparisons the GPU parity tests make (the clock within
1e-12, the step-by-step trace)."""
import numpy as np
import pytest

from conftest import fixture_model
from kmos_gb300 import configs, program as PG
from oracle import oracle as O
from table_invariants import table_violations

CASES = [("ZGB_model", "local_smart", (12, 12)), ("pairwise_interaction", "lat_int", (16, 16))]


def stepped(name, backend, size, steps=3000):
    prog = PG.compile_model(fixture_model(name), backend)
    o = O.Oracle(prog, size, seed=7, rng=O.RNG_PHILOX, traj=3)
    o.set_rates((10.0 ** np.random.default_rng(2).uniform(-1, 2, size=prog.nproc)).tolist())
    o.update_accum_rate()
    o.do_kmc_steps(steps)
    return prog, o


@pytest.mark.parametrize("name,backend,size", CASES)
def test_invariants_hold_and_catch_planted_mistakes(name, backend, size):
    prog, o = stepped(name, backend, size)
    ex = o.export()
    assert table_violations(prog, size, ex["lattice"], ex["as1"], ex["as2"], ex["nsites"]) == []
    P = prog.nproc
    p = int(np.argmax(ex["nsites"]))
    n = int(ex["nsites"][p])
    assert n >= 2
    # two list entries swapped, positions left as they were
    as1 = ex["as1"].copy()
    as1[p, 1], as1[p, 2] = as1[p, 2], as1[p, 1]
    assert table_violations(prog, size, ex["lattice"], as1, ex["as2"], ex["nsites"])
    # a swap-remove that forgets to clear the removed site's position entry
    as1, as2, ns = ex["as1"].copy(), ex["as2"].copy(), ex["nsites"].copy()
    last = as1[p, n]
    as1[p, 1], as1[p, n] = last, 0
    as2[p, last] = 1
    ns[p] = n - 1
    assert table_violations(prog, size, ex["lattice"], as1, as2, ns)
    # a lattice change without the touch-up that keeps the tables in step
    lat = ex["lattice"].copy()
    nsp = len(fixture_model(name).species)
    s = int(np.argmax(lat == lat[0]))
    lat[s] = (lat[s] + 1) % nsp
    assert any("enables" in v for v in table_violations(prog, size, lat, ex["as1"], ex["as2"], ex["nsites"]))


@pytest.mark.parametrize("name,backend,size", CASES)
def test_planted_rate_differences_are_seen(name, backend, size):
    """One rate constant one part in a billion off shows in the clock, beyond the 1e-12
    tolerance; one part in a hundred parts two otherwise identical trajectories, so the
    step-by-step trace comparison sees it."""
    _prog, probe = stepped(name, backend, size)
    k = int(np.argmax(probe.rates() * probe.nr_of_sites()))  # a process with sites: its term counts
    for rel, seen_by in ((1e-9, "time"), (1e-2, "trace")):
        _prog, a = stepped(name, backend, size)
        _prog, b = stepped(name, backend, size)
        rates = b.rates()
        rates[k] *= 1 + rel
        b.set_rates(rates.tolist())
        b.update_accum_rate()
        ta, tb = a.trace(20000), b.trace(20000)
        if seen_by == "time":  # the same steps, but the clock is off by more than 1e-12
            assert abs(a.kmc_time - b.kmc_time) > 1e-12 * a.kmc_time
        else:
            assert not np.array_equal(ta, tb)
