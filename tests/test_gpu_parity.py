"""GPU engine against the CPU oracle: bit-exact processes, sites, occupations and
tables after every sampled step; kmc_time and integ_rates within 1e-12 relative (the
device log() and glibc's log() may differ in the last place)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, fixture_model, many_species_model, rows_model, trimer_model
from kmos_gb300 import configs, engine as E, program as PG
from oracle import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-12

CASES = [("AB_model", "local_smart", (20, 20)), ("ZGB_model", "local_smart", (16, 12)),
         ("ZGB_model", "lat_int", (12, 16)), ("CO_oxidation_Ruo2", "local_smart", (10, 10)),
         ("CO_oxidation_Ruo2", "lat_int", (9, 11)), ("pairwise_interaction", "lat_int", (16, 16)),
         ("pairwise_interaction", "local_smart", (8, 8)), ("default_xml", "local_smart", (10, 10)),
         ("pdopd_xml", "local_smart", (8, 8)), ("pdopd_xml", "lat_int", (8, 8)),
         # lattices narrower than 2*reach+1: every step takes the serial interpreter
         ("pairwise_interaction", "lat_int", (5, 5)), ("ZGB_model", "local_smart", (3, 3)),
         # streams of more than 96 edits: the 4-round fast path
         ("CO_oxidation_Ruo2", "lat_int", (14, 14)), ("default_xml", "lat_int", (14, 14)),
         # the smallest lattices the fast path takes: short lists, so dels often read what
         # an earlier del of the same step moved (the replay's write log)
         ("ZGB_model", "lat_int", (5, 5)), ("CO_oxidation_Ruo2", "lat_int", (5, 5)),
         ("ZGB_model", "local_smart", (5, 5)), ("default_xml", "local_smart", (5, 5))]


def random_rates(P, seed):
    return (10.0 ** np.random.default_rng(seed).uniform(-1, 3, size=P)).tolist()


def assert_same_state(gpu, orc, P, V):
    st = orc.export()
    np.testing.assert_array_equal(gpu.lattice(), st["lattice"])
    as1, as2 = gpu.tables()
    np.testing.assert_array_equal(as1, st["as1"])
    np.testing.assert_array_equal(as2, st["as2"])
    np.testing.assert_array_equal(gpu.nr_of_sites(), st["nsites"])
    np.testing.assert_array_equal(gpu.procstat(), st["procstat"])
    np.testing.assert_allclose(gpu.integ_rates(), st["integ"], rtol=RTOL, atol=0)
    assert gpu.kmc_step == orc.kmc_step
    assert abs(gpu.kmc_time - orc.kmc_time) <= RTOL * abs(orc.kmc_time)


def test_golden_trajectory_on_gpu():
    """The reference's own golden trajectory (tests/test_run/test_run.py) through the
    C-ABI: get_next_kmc_step + run_proc_nr, gfortran stream, seed 1."""
    ref = np.load(os.path.join(GOLDEN, "ab_model_ref_procs_sites.npy"))
    m = fixture_model("AB_model")
    rates = json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    with E.Trajectory(PG.compile_model(m, "local_smart"), (20, 20), seed=1, rng=E.RNG_GFORTRAN) as t:
        t.set_rates(rates)
        t.update_accum_rate()
        out = np.zeros_like(ref)
        for i in range(len(ref)):
            p, s = t.get_next_kmc_step()
            out[i] = (p, s)
            t.run_proc_nr(p, s)
    np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("name,backend,size", CASES)
def test_initial_state(name, backend, size):
    prog = PG.compile_model(fixture_model(name), backend)
    with E.Trajectory(prog, size, seed=5) as g:
        o = O.Oracle(prog, size, seed=5)
        st = o.export()
        np.testing.assert_array_equal(g.lattice(), st["lattice"])
        as1, as2 = g.tables()
        np.testing.assert_array_equal(as1, st["as1"])
        np.testing.assert_array_equal(as2, st["as2"])


@pytest.mark.parametrize("rng", [E.RNG_GFORTRAN, E.RNG_PHILOX])
@pytest.mark.parametrize("name,backend,size", CASES)
def test_trace_matches_oracle(name, backend, size, rng):
    prog = PG.compile_model(fixture_model(name), backend)
    rates = random_rates(prog.nproc, 11)
    with E.Trajectory(prog, size, seed=17, rng=rng, traj=4) as g:
        o = O.Oracle(prog, size, seed=17, rng=rng, traj=4)
        for x in (g, o):
            x.set_rates(rates)
            x.update_accum_rate()
        for chunk in (1, 999, 9000):
            np.testing.assert_array_equal(g.trace(chunk), o.trace(chunk))
            assert_same_state(g, o, prog.nproc, o.V)
        np.testing.assert_allclose(g.accum_rates(), o.accum_rates(), rtol=0, atol=0)


@pytest.mark.parametrize("name,backend,size", [CASES[i] for i in (1, 3, 4, 5, 9)])
def test_rates_over_thirty_decades(name, backend, size):
    """Rate constants 10^U(-25, 6): many accum terms fall below half an ulp of the
    running sum (their adds change nothing, in the reference's order as here);
    accum_rates stay the oracle's bit for bit, and so do the steps."""
    prog = PG.compile_model(fixture_model(name), backend)
    rates = (10.0 ** np.random.default_rng(23).uniform(-25, 6, size=prog.nproc)).tolist()
    with E.Trajectory(prog, size, seed=29, rng=E.RNG_PHILOX, traj=1) as g:
        o = O.Oracle(prog, size, seed=29, rng=O.RNG_PHILOX, traj=1)
        for x in (g, o):
            x.set_rates(rates)
            x.update_accum_rate()
        for chunk in (1, 700, 3000):
            np.testing.assert_array_equal(g.trace(chunk), o.trace(chunk))
            np.testing.assert_array_equal(g.accum_rates(), o.accum_rates())
        assert_same_state(g, o, prog.nproc, o.V)


@pytest.mark.parametrize("which,backend,tables", [("trimer", "local_smart", True), ("trimer", "lat_int", True),
                                                  ("trimer", "lat_int", False),
                                                  ("pairwise_interaction", "lat_int", False),
                                                  ("CO_oxidation_Ruo2", "lat_int", False)])
def test_wide_conditions_and_member_scans(which, backend, tables, monkeypatch):
    """Edit forms of the fast step the fixture models alone do not reach: adds with two
    conditions (three-site processes, local_smart) and nli edits through member scans
    of the group record (models compiled without nli tables)."""
    if not tables:
        monkeypatch.setattr(PG, "NLI_TABLE_MAX", 0)
    m = trimer_model() if which == "trimer" else fixture_model(which)
    prog = PG.compile_model(m, backend)
    monkeypatch.undo()
    P = prog.nproc
    size = (14, 14) if which != "CO_oxidation_Ruo2" else (12, 12)
    for traj in range(2):
        rates = (10.0 ** np.random.default_rng(40 + traj).uniform(-1, 2, size=P)).tolist()
        with E.Trajectory(prog, size, seed=31, rng=E.RNG_PHILOX, traj=traj) as g:
            o = O.Oracle(prog, size, seed=31, rng=O.RNG_PHILOX, traj=traj)
            for x in (g, o):
                x.set_rates(rates)
                x.update_accum_rate()
            for chunk in (1, 999, 4000):
                np.testing.assert_array_equal(g.trace(chunk), o.trace(chunk))
            assert_same_state(g, o, P, o.V)


@pytest.mark.parametrize("nspecies,backend", [(16, "local_smart"), (16, "lat_int"), (29, "local_smart")])
def test_large_process_counts(nspecies, backend):
    """96 and 174 processes: the kernels with four and eight processes per lane, fast
    streams of processes past the 64th (whose list tops are not loaded ahead: their
    replay reads them from memory) and the serial interpreter for the streams over the
    on-chip limits."""
    prog = PG.compile_model(many_species_model(nspecies), backend)
    rates = (10.0 ** np.random.default_rng(5).uniform(-1, 2, size=prog.nproc)).tolist()
    with E.Trajectory(prog, (12, 12), seed=13, rng=E.RNG_PHILOX, traj=2) as g:
        o = O.Oracle(prog, (12, 12), seed=13, rng=O.RNG_PHILOX, traj=2)
        for x in (g, o):
            x.set_rates(rates)
            x.update_accum_rate()
        for chunk in (1, 999, 3000):
            np.testing.assert_array_equal(g.trace(chunk), o.trace(chunk))
        assert_same_state(g, o, prog.nproc, o.V)
        np.testing.assert_array_equal(g.accum_rates(), o.accum_rates())


@pytest.mark.parametrize("backend,size", [("local_smart", (16, 6)), ("lat_int", (32, 4))])
def test_many_dels_of_one_process(backend, size):
    """Row desorption clears eight sites at once: one process gets up to dozens of dels
    in a step, past the list tops the kernel loads ahead (the replay reads the rest from
    memory) and past its write log (once full, every read goes to memory)."""
    prog = PG.compile_model(rows_model(8), backend)
    with E.Trajectory(prog, size, seed=17, rng=E.RNG_PHILOX, traj=5) as g:
        o = O.Oracle(prog, size, seed=17, rng=O.RNG_PHILOX, traj=5)
        for x in (g, o):
            x.set_rates([20.0, 1.0, 50.0])
            x.update_accum_rate()
        for chunk in (1, 999, 5000):
            np.testing.assert_array_equal(g.trace(chunk), o.trace(chunk))
            assert_same_state(g, o, prog.nproc, o.V)


@pytest.mark.parametrize("T", [300.0, 600.0])
def test_lateral_interaction_at_one_temperature(T):
    """The config-3 model (CO, lat_int) at one temperature.  At 300 K the lattice fills
    with CO (every lateral-interaction edit of a step fires, the desorption terms are
    ~1e-16 per site); at 600 K it is sparse."""
    wl = configs.build(3, n=2, steps=0, sides=[16, 32])
    kT = configs.K_B_EV * T
    rates = [1e3] + [1e13 * np.exp(-(1.3 + 0.1 * bin(m).count("1")) / kT) for m in range(16)]
    rates = [float(r) for r in rates + [1e13 * np.exp(-0.6 / kT)] * 4]
    for i in range(wl.n):
        with E.Trajectory(wl.program, wl.sizes[i], seed=wl.seeds[i], rng=E.RNG_PHILOX, traj=wl.trajs[i]) as g:
            o = O.Oracle(wl.program, wl.sizes[i], seed=wl.seeds[i], rng=O.RNG_PHILOX, traj=wl.trajs[i])
            for x in (g, o):
                x.set_rates(rates)
                x.update_accum_rate()
            for chunk in (2000, 6000):
                np.testing.assert_array_equal(g.trace(chunk), o.trace(chunk))
                np.testing.assert_array_equal(g.accum_rates(), o.accum_rates())
            assert_same_state(g, o, wl.program.nproc, o.V)


@pytest.mark.parametrize("config", [1, 2, 3, 4])
def test_benchmark_configs_match_oracle(config):
    wl = configs.build(config, n=3, steps=5000, sides=[16, 32])
    for i in range(wl.n):
        with E.Trajectory(wl.program, wl.sizes[i], seed=wl.seeds[i], rng=E.RNG_PHILOX, traj=wl.trajs[i]) as g:
            o = O.Oracle(wl.program, wl.sizes[i], seed=wl.seeds[i], rng=O.RNG_PHILOX, traj=wl.trajs[i])
            for x in (g, o):
                x.set_rates(wl.rates[i])
                x.update_accum_rate()
            g.do_kmc_steps(wl.steps)
            o.do_kmc_steps(wl.steps)
            assert_same_state(g, o, wl.program.nproc, o.V)
            np.testing.assert_allclose(g.occupation(), o.occupation(), rtol=0, atol=0)


class PoolRun:
    """A pool with several models and uneven lattices, run in one launch."""

    def __init__(self, graph=False):
        self.wls = [configs.build(2, n=3, steps=0), configs.build(3, n=4, steps=0, sides=[16, 32, 64]),
                    configs.build(4, n=3, steps=0)]
        self.pool = E.Pool(arena_bytes=256 << 20, max_slots=64)
        self.items = []
        for wl in self.wls:
            mid = self.pool.add_model(wl.program)
            for i in range(wl.n):
                slot = self.pool.admit(mid, wl.sizes[i], wl.rates[i], seed=wl.seeds[i], rng=E.RNG_PHILOX,
                                       traj=wl.trajs[i])
                self.items.append((wl, i, slot))


def oracle_for(wl, i, steps):
    o = O.Oracle(wl.program, wl.sizes[i], seed=wl.seeds[i], rng=O.RNG_PHILOX, traj=wl.trajs[i])
    o.set_rates(wl.rates[i])
    o.update_accum_rate()
    o.do_kmc_steps(steps)
    return o


def test_pool_batch_matches_oracle():
    pr = PoolRun()
    slots = [s for _wl, _i, s in pr.items]
    steps = [1000 + 357 * k for k in range(len(slots))]  # uneven step counts
    pr.pool.run(slots, steps)
    for (wl, i, slot), n in zip(pr.items, steps):
        o = oracle_for(wl, i, n)
        st = o.export()
        assert pr.pool.status(slot) == 0
        np.testing.assert_array_equal(pr.pool.lattice(slot), st["lattice"])
        as1, as2 = pr.pool.tables(slot)
        np.testing.assert_array_equal(as1, st["as1"])
        np.testing.assert_array_equal(as2, st["as2"])
        np.testing.assert_array_equal(pr.pool.procstat(slot), st["procstat"])
        t, k = pr.pool.clock(slot)
        assert k == n and abs(t - o.kmc_time) <= RTOL * o.kmc_time


def test_same_alone_and_in_the_mix():
    """A trajectory's result does not depend on what else shares the launch."""
    pr = PoolRun()
    slots = [s for _wl, _i, s in pr.items]
    pr.pool.run(slots, 3000)
    mixed = {s: (pr.pool.procstat(s), pr.pool.clock(s)) for s in slots}
    alone = PoolRun()
    for (_wl, _i, s) in alone.items:
        alone.pool.run([s], 3000)
        ps, clk = alone.pool.procstat(s), alone.pool.clock(s)
        np.testing.assert_array_equal(ps, mixed[s][0])
        assert clk == mixed[s][1]


def test_graph_replay_equals_plain_launch():
    a, b = PoolRun(), PoolRun()
    slots = [s for _wl, _i, s in a.items]
    for _ in range(3):
        a.pool.run(slots, 700)
        b.pool.run_graph(slots, 700)
    for s in slots:
        np.testing.assert_array_equal(a.pool.procstat(s), b.pool.procstat(s))
        assert a.pool.clock(s) == b.pool.clock(s)


def test_deadlock_is_an_error_status_not_a_crash():
    """Adsorption without desorption fills the lattice; the next step finds no process
    (base.mpy:1293-1311 stops the process; here the call returns an error)."""
    m = configs.model_config1()
    prog = PG.compile_model(m, "local_smart")
    with E.Trajectory(prog, (4, 4), seed=1, rng=E.RNG_PHILOX) as t:
        t.set_rates([1.0, 0.0])
        t.update_accum_rate()
        with pytest.raises(E.KMCError) as err:
            t.do_kmc_steps(100)
        assert err.value.code == 3
        assert t.kmc_step == 16
        assert (t.lattice() == m.species_ids()["CO"]).all()


@pytest.mark.parametrize("config", [2, 3, 4])
def test_serial_and_fast_paths_agree(config):
    """The gather / replay / scatter step and the serial interpreter give the same
    tables, step by step counts and clocks."""
    wl = configs.build(config, n=6, steps=0, sides=[16, 32])
    out = []
    for fast in (False, True):
        pool = E.Pool(arena_bytes=512 << 20, max_slots=16)
        pool.set_fast_path(fast)
        mid = pool.add_model(wl.program)
        slots = pool.admit_many([mid] * wl.n, wl.sizes, wl.rates, seeds=wl.seeds, rng=E.RNG_PHILOX, trajs=wl.trajs)
        pool.run(slots, 4000)
        out.append([(pool.tables(s), pool.procstat(s), pool.clock(s))
                    for i, s in enumerate(slots)])
        pool.close()
    for (ta, pa, ca), (tb, pb, cb) in zip(*out):
        np.testing.assert_array_equal(ta[0], tb[0])
        np.testing.assert_array_equal(ta[1], tb[1])
        np.testing.assert_array_equal(pa, pb)
        assert ca == cb


@pytest.mark.parametrize("config", [2, 3, 4])
def test_launch_shape_and_table_placement_do_not_change_results(config):
    """Every launch shape the autotuner tries (one balanced block per SM, 2 or 8 warps per
    block) and both placements of the model's hot section (shared or global memory) give
    the same trajectories bit for bit; steps per launch too (one launch of 3000 steps
    against three of 1000)."""
    wl = configs.build(config, n=40, steps=0, sides=[16, 32])
    out = []
    for warps, shared, launches in ((0, True, 1), (2, True, 1), (8, False, 1), (0, False, 3), (8, True, 3)):
        pool = E.Pool(arena_bytes=1 << 30, max_slots=64)
        pool.set_launch(warps, 0)
        pool.set_table_placement(shared)
        mid = pool.add_model(wl.program)
        slots = pool.admit_many([mid] * wl.n, wl.sizes, wl.rates, seeds=wl.seeds, rng=E.RNG_PHILOX, trajs=wl.trajs)
        for _ in range(launches):
            pool.run(slots, 3000 // launches)
        out.append([(pool.tables(s), pool.procstat(s), pool.clock(s), pool.lattice(s)) for s in slots])
        pool.close()
    for other in out[1:]:
        for (ta, pa, ca, la), (tb, pb, cb, lb) in zip(out[0], other):
            np.testing.assert_array_equal(ta[0], tb[0])
            np.testing.assert_array_equal(ta[1], tb[1])
            np.testing.assert_array_equal(pa, pb)
            np.testing.assert_array_equal(la, lb)
            assert ca == cb


@pytest.mark.parametrize("backend", ["local_smart", "lat_int"])
def test_replace_species_range(backend):
    """replace_species refuses a new species outside -1..nspecies (the range state images
    and .reload files are checked against) and leaves the site as it was; the wrong old
    species is KMC_ERR_SPECIES as in the reference's stop."""
    m = fixture_model("ZGB_model")
    prog = PG.compile_model(m, backend)
    t = E.Trajectory(prog, (6, 6), seed=3)
    cur = t.get_species(1)
    ns = len(m.species)
    for bad in (ns + 1, -2, 127):
        with pytest.raises(E.KMCError) as e:
            t.replace_species(1, cur, bad)
        assert e.value.code == 1
        assert t.get_species(1) == cur
    with pytest.raises(E.KMCError) as e:
        t.replace_species(1, (cur + 1) % ns, cur)
    assert e.value.code == 2
    new = (cur + 1) % ns
    t.replace_species(1, cur, new)
    assert t.get_species(1) == new


def test_run_list_checks():
    """A slot listed twice in one run, and negative rate offsets, are refused before any
    launch."""
    prog = PG.compile_model(fixture_model("ZGB_model"), "local_smart")
    pool = E.Pool(arena_bytes=32 << 20, max_slots=4)
    mid = pool.add_model(prog)
    s = pool.admit(mid, (8, 8), [1.0] * prog.nproc, seed=1)
    with pytest.raises(E.KMCError) as e:
        pool.run([s, s], 10)
    assert e.value.code == 1
    with pytest.raises(E.KMCError) as e:
        pool.run_graph([s, s], 10)
    assert e.value.code == 1
    import ctypes
    L = E.load()
    mids = np.array([mid], np.int32)
    dims = np.array([8, 8, 1], np.int32)
    seeds = np.array([1], np.int32)
    rates = np.ones(prog.nproc)
    offs = np.array([-1], np.int32)
    out = np.zeros(1, np.int32)
    P32, PD = ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)
    rc = L.kmc_pool_admit_many(pool.h, 1, mids.ctypes.data_as(P32), dims.ctypes.data_as(P32), 0,
                               seeds.ctypes.data_as(P32), E.RNG_PHILOX, None, rates.ctypes.data_as(PD),
                               offs.ctypes.data_as(P32), out.ctypes.data_as(P32))
    assert rc == 1
    pool.run([s], 10)  # the pool still works
    pool.close()


def test_cancel_stops_a_running_batch():
    """kmc_pool_cancel from the host ends a long persistent launch within a second (the
    kernel polls the host-mapped flag every 1024 steps): the trajectories it was running
    end with the cancelled status, and the pool keeps working for new trajectories."""
    import time
    wl = configs.build(2, n=64, steps=0)
    pool = E.Pool(arena_bytes=256 << 20, max_slots=128)
    mid = pool.add_model(wl.program)
    slots = pool.admit_many([mid] * wl.n, wl.sizes, wl.rates, seeds=wl.seeds, rng=E.RNG_PHILOX, trajs=wl.trajs)
    pool.run(slots, 10_000_000, sync=False)  # about a minute if nothing stops it
    time.sleep(0.3)
    t0 = time.perf_counter()
    pool.cancel()
    pool.sync()
    assert time.perf_counter() - t0 < 2.0
    _ps, _ig, _t, steps, status = pool.results(slots, 1)
    assert (steps < 10_000_000).all()
    assert set(status.tolist()) <= {3, 8} and (status == 8).any()
    fresh = pool.admit(mid, (16, 16), wl.rates[0], seed=1)
    pool.run([fresh], 2000)
    assert pool.status(fresh) == 0 and pool.clock(fresh)[1] == 2000
    pool.close()
