"""The CPU oracle against the reference's golden vectors and published algorithms."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, fixture_model
from kmos_gb300 import program as PG, rates as R
from oracle import oracle as O


def ab_oracle(backend="local_smart"):
    m = fixture_model("AB_model")
    o = O.Oracle(PG.compile_model(m, backend), (20, 20), layer=0, seed=1, rng=O.RNG_GFORTRAN)
    rates = json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    o.set_rates(rates)
    o.update_accum_rate()
    return o


def test_rate_expressions_match_reference():
    """kmos_gb300.rates evaluates the AB model's expressions to the same doubles."""
    m = fixture_model("AB_model")
    ref = json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    assert R.model_rates(m) == ref


def test_golden_trajectory_local_smart():
    """tests/test_run/test_run.py of the reference: 10000 get_next_kmc_step +
    run_proc_nr pairs of the 20x20 AB model, seed 1, gfortran RANDOM_NUMBER stream."""
    ref = np.load(os.path.join(GOLDEN, "ab_model_ref_procs_sites.npy"))
    o = ab_oracle()
    out = []
    for _ in range(len(ref)):
        p, s = o.get_next_kmc_step()
        out.append((p, s))
        o.run_proc_nr(p, s)
    np.testing.assert_array_equal(np.array(out), ref)


def test_golden_trajectory_lat_int_prefix():
    """The reference ships the local_smart log as the lat_int golden too.  lat_int
    stores a process at the first site of its cell, local_smart at the process's
    executing coordinate (kmos/types.py:2094-2097), and lat_int re-adds every
    neighbouring process after an event (kmos/io/__init__.py:1793-1983), so the
    book-keeping order differs after the first event that touches a neighbour.  Up to
    the first AB reaction (step 155) the lat_int trajectory is the golden one; the
    reaction itself lands one cell up (the A site instead of the B site)."""
    ref = np.load(os.path.join(GOLDEN, "ab_model_ref_procs_sites.npy"))
    o = ab_oracle("lat_int")
    out = []
    for _ in range(155):
        p, s = o.get_next_kmc_step()
        out.append((p, s))
        o.run_proc_nr(p, s)
    np.testing.assert_array_equal(np.array(out[:154]), ref[:154])
    assert out[154][0] == ref[154][0] == 1
    assert out[154][1] == ref[154][1] + 20


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors of the Random123 distribution."""
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_philox_draws_in_open_interval():
    m = fixture_model("AB_model")
    o = O.Oracle(PG.compile_model(m, "local_smart"), (4, 4), rng=O.RNG_PHILOX, seed=7, traj=3)
    d = o.draws(20000)
    assert (d > 0).all() and (d < 1).all()
    assert abs(d.mean() - 0.5) < 0.01


def interval_search_literal(arr, value):
    """interval_search_real (base.mpy:1234-1338), 1-based result, 0 for dead lock."""
    left, right = 1, len(arr)
    while True:
        mid = (right + left) >> 1
        if left >= right:
            break
        if value < arr[mid - 1]:
            right = mid
        else:
            left = mid + 1
    if arr[mid - 1] == 0.0:
        while not arr[mid - 1] > 0.0:
            if mid >= len(arr):
                return 0
            mid += 1
    while mid != 1 and arr[mid - 2] >= arr[mid - 1]:
        mid -= 1
    return mid


def ballot_rule(arr, value):
    """The engine's form: min(first i with arr(i) > v, first i with arr(i) == arr(P))."""
    total = arr[-1]
    for i, a in enumerate(arr):
        if a > value or a == total:
            return i + 1
    return 0


def test_bisection_ballot_rule_equals_interval_search():
    rng = np.random.default_rng(5)
    for trial in range(20000):
        P = int(rng.integers(1, 70))
        n = rng.integers(0, 4, size=P) * (rng.random(P) < 0.6)
        r = rng.choice([0.0, 1.0, 1e6, 0.5, 3.25, 1e-9], size=P)
        arr = np.cumsum(n * r).tolist()
        if not arr[-1] > 0:
            continue
        for u in (0.0, rng.random(), rng.random(), 1.0 - 2 ** -53):
            v = u * arr[-1]
            assert interval_search_literal(arr, v) == ballot_rule(arr, v), (arr, v)


@pytest.mark.parametrize("name,backend", [("ZGB_model", "local_smart"), ("ZGB_model", "lat_int"),
                                          ("CO_oxidation_Ruo2", "local_smart"), ("CO_oxidation_Ruo2", "lat_int"),
                                          ("pairwise_interaction", "lat_int"), ("pairwise_interaction", "local_smart"),
                                          ("default_xml", "local_smart"), ("pdopd_xml", "local_smart"),
                                          ("pdopd_xml", "lat_int")])
def test_oracle_tables_stay_consistent(name, backend):
    """avail_sites(p, avail_sites(p, i, 1), 2) == i for i <= nr_of_sites(p), and the
    rest of both tables is zero, after many steps of every fixture model."""
    m = fixture_model(name)
    prog = PG.compile_model(m, backend)
    o = O.Oracle(prog, (10, 10), seed=3, rng=O.RNG_PHILOX, traj=1)
    rng = np.random.default_rng(1)
    o.set_rates(10.0 ** rng.uniform(-1, 3, size=prog.nproc))
    o.update_accum_rate()
    o.do_kmc_steps(3000)
    st = o.export()
    V = o.V
    for p in range(prog.nproc):
        n = st["nsites"][p]
        a1, a2 = st["as1"][p], st["as2"][p]
        assert (a1[n + 1:] == 0).all()
        sites = a1[1:n + 1]
        assert len(set(sites.tolist())) == n
        assert (a2[sites] == np.arange(1, n + 1)).all()
        assert np.count_nonzero(a2) == n
