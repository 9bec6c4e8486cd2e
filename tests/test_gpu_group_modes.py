"""The step kernel's launch modes against the oracle: one or two trajectories per warp
(32 or 16 lanes each), lattices and avail_sites tables in device memory or copied to
shared memory for the launch, and the solo kernel (steps on one lane) for small launches
of models with up to 8 processes.  None of them may change a result: every mode must leave
each trajectory's lattice, both avail_sites columns, nr_of_sites, procstat and step
count equal to the oracle's, and its clock and integ_rates within 1e-12 relative.

Pools mix trajectories with uneven step counts, so in the two-per-warp mode the halves
of a warp run, finish and pick up new trajectories at different times."""
import numpy as np
import pytest

from conftest import fixture_model, many_species_model, rows_model, trimer_model
from kmos_gb300 import configs, engine as E, program as PG
from oracle import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-12
# (trajectories per warp, tables on chip, solo kernel for small launches of small models)
MODES = [(1, True, True), (1, True, False), (1, False, False), (1, False, True), (2, True, False), (2, False, False)]

CASES = [("AB_model", "local_smart", (20, 20)), ("ZGB_model", "local_smart", (16, 12)),
         ("ZGB_model", "lat_int", (12, 16)), ("CO_oxidation_Ruo2", "local_smart", (10, 10)),
         ("CO_oxidation_Ruo2", "lat_int", (14, 14)), ("pairwise_interaction", "lat_int", (16, 16)),
         ("default_xml", "local_smart", (10, 10)), ("default_xml", "lat_int", (14, 14)),
         ("pdopd_xml", "lat_int", (8, 8)), ("pairwise_interaction", "lat_int", (5, 5)),
         ("ZGB_model", "lat_int", (5, 5))]


def _programs():
    out = [(name + "/" + backend, PG.compile_model(fixture_model(name), backend), size)
           for name, backend, size in CASES]
    out += [("trimer/lat_int", PG.compile_model(trimer_model(), "lat_int"), (12, 12)),
            ("trimer/local_smart", PG.compile_model(trimer_model(), "local_smart"), (12, 12)),
            ("rows/lat_int", PG.compile_model(rows_model(), "lat_int"), (16, 16)),
            ("many_species/local_smart", PG.compile_model(many_species_model(), "local_smart"), (10, 10))]
    return out


PROGRAMS = _programs()


def random_rates(P, seed):
    return (10.0 ** np.random.default_rng(seed).uniform(-1, 3, size=P)).tolist()


def check_against_oracle(pool, slot, prog, size, rates, seed, rng, steps, where):
    o = O.Oracle(prog, size, seed=seed, rng=rng, traj=seed)
    o.set_rates(rates)
    o.update_accum_rate()
    o.do_kmc_steps(steps)
    st = o.export()
    assert pool.status(slot) == 0, where
    t, k = pool.clock(slot)
    assert k == steps, where
    assert abs(t - o.kmc_time) <= RTOL * abs(o.kmc_time), where
    np.testing.assert_array_equal(pool.lattice(slot), st["lattice"], err_msg=where)
    as1, as2 = pool.tables(slot)
    np.testing.assert_array_equal(as1, st["as1"], err_msg=where)
    np.testing.assert_array_equal(as2, st["as2"], err_msg=where)
    np.testing.assert_array_equal(pool.nr_of_sites(slot), st["nsites"], err_msg=where)
    np.testing.assert_array_equal(pool.procstat(slot), st["procstat"], err_msg=where)
    np.testing.assert_allclose(pool.integ_rates(slot), st["integ"], rtol=RTOL, atol=0, err_msg=where)


@pytest.mark.parametrize("tpw,on_chip,solo", MODES)
@pytest.mark.parametrize("rng", [E.RNG_PHILOX, E.RNG_GFORTRAN])
def test_every_mode_matches_the_oracle(tpw, on_chip, solo, rng):
    pool = E.Pool(arena_bytes=256 << 20, max_slots=64)
    pool.set_trajectories_per_warp(tpw)
    pool.set_tables_on_chip(on_chip)
    pool.set_solo(solo)
    items = []
    for k, (name, prog, size) in enumerate(PROGRAMS):
        mid = pool.add_model(prog)
        for j in range(3):
            seed = 7 + 3 * k + j
            rates = random_rates(prog.nproc, seed)
            slot = pool.admit(mid, size, rates, seed=seed, rng=rng, traj=seed)
            items.append((name, prog, size, rates, seed, slot, 1500 + 733 * j))
    slots = [it[5] for it in items]
    steps = [it[6] for it in items]
    pool.run(slots, steps)
    for name, prog, size, rates, seed, slot, n in items:
        where = "%s, seed %d, %d steps, mode %s" % (name, seed, n, (tpw, on_chip, solo))
        check_against_oracle(pool, slot, prog, size, rates, seed, rng, n, where)
    pool.close()


@pytest.mark.parametrize("config", [2, 3, 4])
def test_modes_agree_on_the_benchmark_workloads(config):
    """Batches of the benchmark workloads (40 trajectories, uneven lattices for config 3)
    end bit for bit the same in every mode and launch shape, with several launches."""
    wl = configs.build(config, n=40, steps=0, sides=[16, 32])
    out = []
    for tpw, on_chip, warps in ((1, False, 0), (2, False, 0), (2, False, 4), (2, True, 0), (1, True, 2)):
        pool = E.Pool(arena_bytes=1 << 30, max_slots=64)
        pool.set_trajectories_per_warp(tpw)
        pool.set_tables_on_chip(on_chip)
        pool.set_launch(warps, 0)
        mid = pool.add_model(wl.program)
        slots = pool.admit_many([mid] * wl.n, wl.sizes, wl.rates, seeds=wl.seeds, rng=E.RNG_PHILOX, trajs=wl.trajs)
        for _ in range(2):
            pool.run(slots, 1500)
        out.append([(pool.tables(s), pool.procstat(s), pool.clock(s), pool.lattice(s)) for s in slots])
        pool.close()
    for other in out[1:]:
        for (ta, pa, ca, la), (tb, pb, cb, lb) in zip(out[0], other):
            np.testing.assert_array_equal(ta[0], tb[0])
            np.testing.assert_array_equal(ta[1], tb[1])
            np.testing.assert_array_equal(pa, pb)
            np.testing.assert_array_equal(la, lb)
            assert ca == cb
    # and the first of them against the oracle
    o = O.Oracle(wl.program, wl.sizes[0], seed=wl.seeds[0], rng=O.RNG_PHILOX, traj=wl.trajs[0])
    o.set_rates(wl.rates[0])
    o.update_accum_rate()
    o.do_kmc_steps(3000)
    np.testing.assert_array_equal(out[1][0][3], o.export()["lattice"])
    np.testing.assert_array_equal(out[1][0][1], o.export()["procstat"])


def test_single_trajectory_with_tables_on_chip_traces_like_the_oracle():
    """The plain one-trajectory drop-in of a small model (the solo kernel, lattice and
    tables in shared memory): the (process, site) of every step equals the oracle's,
    across batch boundaries of the random draws."""
    wl = configs.build(1, n=1, steps=0)
    with E.Trajectory(wl.program, wl.sizes[0], seed=wl.seeds[0], rng=E.RNG_PHILOX, traj=wl.trajs[0]) as g:
        o = O.Oracle(wl.program, wl.sizes[0], seed=wl.seeds[0], rng=O.RNG_PHILOX, traj=wl.trajs[0])
        for x in (g, o):
            x.set_rates(wl.rates[0])
            x.update_accum_rate()
        for chunk in (1, 31, 2000, 20000):
            np.testing.assert_array_equal(g.trace(chunk), o.trace(chunk))
        g.do_kmc_steps(50000)
        o.do_kmc_steps(50000)
        np.testing.assert_array_equal(g.lattice(), o.export()["lattice"])
        np.testing.assert_array_equal(g.procstat(), o.export()["procstat"])
