"""GPU parity of the otf backend (kmc_otf_*, kmos_gb300/csrc/kmc_otf.cu) with the oracle.

* The reference's golden trajectory prefix (20x20 AB model, seed 1, gfortran stream)
  through get_next_kmc_step + run_proc_nr on the device.
* intZGB (bystander-dependent rates: base_rate * J ** nr products) and default.xml (two
  sites per cell, constant rates), batches of Philox trajectories: after every block of
  do_kmc_steps each trajectory's lattice, avail_sites, nr_of_sites, procstat, every
  list entry's rate, the process totals and accum_rates equal the oracle's bit for bit;
  kmc_time and integ_rates agree within 1e-12 relative (the device's log differs from
  the host's in the last place, which moves only the clock).
* A rate expression with exp and a multi-line aux variable: rates within 1e-15.
* trace_steps of one trajectory equals the oracle's trace.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, fixture_model
from kmos_gb300 import engine as E, otf as OTF, program as PG
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def setup_both(model, size, rates, params, ntraj, seed=7, rng=E.RNG_PHILOX, traj0=0):
    prog = PG.compile_model(model, "otf")
    b = E.OtfBatch(prog, size, ntraj=ntraj, seed=seed, rng=rng, traj0=traj0)
    b.set_rates(rates)
    b.set_user_parameters(params)
    b.recalculate_rates_matrix()
    b.update_accum_rate()
    b.update_integ_rate()
    oracles = []
    for t in range(ntraj):
        o = O.Oracle(prog, size, seed=seed, rng=rng, traj=traj0 + t)
        o.set_rates(rates)
        o.set_user_parameters(params)
        o.recalculate_rates_matrix()
        o.update_accum_rate()
        o.update_integ_rate()
        oracles.append(o)
    return prog, b, oracles


def compare(b, t, o, rate_rtol=0.0):
    g = b.state(t)
    ex = o.export()
    np.testing.assert_array_equal(g["lattice"], ex["lattice"])
    np.testing.assert_array_equal(g["nsites"], ex["nsites"])
    np.testing.assert_array_equal(g["procstat"], ex["procstat"])
    for p in range(o.P):
        n = int(ex["nsites"][p])
        np.testing.assert_array_equal(g["as1"][p, 1:n + 1], ex["as1"][p, 1:n + 1])
    np.testing.assert_array_equal(g["as2"], ex["as2"])
    rm, tot = o.rates_matrix()
    if rate_rtol == 0.0:
        np.testing.assert_array_equal(g["rates_matrix"][:, 1:], rm[:, 1:])
        np.testing.assert_array_equal(g["totals"], tot)
        np.testing.assert_array_equal(g["accum"], o.accum_rates())
    else:
        np.testing.assert_allclose(g["rates_matrix"][:, 1:], rm[:, 1:], rtol=rate_rtol, atol=0)
    assert g["kmc_step"] == o.kmc_step
    np.testing.assert_allclose(g["kmc_time"], o.kmc_time, rtol=1e-12, atol=0)
    np.testing.assert_allclose(g["integ"], o.integ_rates(), rtol=1e-12, atol=1e-300)


def test_golden_prefix_on_the_device():
    m = fixture_model("AB_model")
    rates = json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    ref = np.load(os.path.join(GOLDEN, "ab_model_ref_procs_sites.npy"))
    _prog, b, (o,) = setup_both(m, (20, 20), rates, OTF.user_parameter_values(m), 1, seed=1, rng=E.RNG_GFORTRAN)
    out = []
    for _ in range(155):
        p, s = b.get_next_kmc_step(0)
        assert (p, s) == o.get_next_kmc_step()
        out.append((p, s))
        b.run_proc_nr(p, s, 0)
        o.run_proc_nr(p, s)
    np.testing.assert_array_equal(np.array(out[:154]), ref[:154])
    assert out[154][1] == ref[154][1] + 20
    compare(b, 0, o)


INTZGB_RATES = [0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3]
INTZGB_PARAMS = [1.3, 0.7, 1.9, 1e-10, 0.5]


# 4 x 5 and 5 x 4: narrower than twice the streams' reach, so one event's ops can name
# one site twice and the replay reads old rates from the tables instead of the ones
# loaded ahead
@pytest.mark.parametrize("size,ntraj", [((16, 16), 6), ((9, 11), 3), ((4, 5), 3), ((5, 4), 2)])
def test_intzgb_batch_matches_oracle(size, ntraj):
    m = fixture_model("intZGB_otf")
    _prog, b, oracles = setup_both(m, size, INTZGB_RATES, INTZGB_PARAMS, ntraj, traj0=5)
    for block in (1, 37, 800, 1500):
        b.do_kmc_steps(block)
        for t, o in enumerate(oracles):
            o.do_kmc_steps(block)
            compare(b, t, o)
    assert b.launch_count() > 0


def test_default_xml_two_sites_per_cell():
    m = fixture_model("default_xml")
    rates = (10.0 ** np.random.default_rng(2).uniform(-1, 2, size=len(m.processes))).tolist()
    _prog, b, oracles = setup_both(m, (10, 8), rates, OTF.user_parameter_values(m), 2)
    for block in (200, 1800):
        b.do_kmc_steps(block)
        for t, o in enumerate(oracles):
            o.do_kmc_steps(block)
            compare(b, t, o)


def test_exp_rates_and_aux_variables():
    m = fixture_model("intZGB_otf")
    m.processes[0].otf_rate = "e = J_O_CO*nr_O_1nn + 0.5*J_CO_CO*nr_CO_1nn\notf_rate = base_rate*exp(-e)"
    m.processes[8].otf_rate = "base_rate*sqrt(1.0d0 + nr_O_1nn)/(1 + nr_CO_1nn)"
    _prog, b, (o,) = setup_both(m, (12, 12), INTZGB_RATES, INTZGB_PARAMS, 1)
    b.do_kmc_steps(600)
    o.do_kmc_steps(600)
    compare(b, 0, o, rate_rtol=1e-15)


def test_trace_matches_oracle():
    m = fixture_model("intZGB_otf")
    _prog, b, oracles = setup_both(m, (14, 14), INTZGB_RATES, INTZGB_PARAMS, 3)
    tr = b.trace(2, 1200)
    np.testing.assert_array_equal(tr, oracles[2].trace(1200))
    compare(b, 2, oracles[2])
    assert b.state(0)["kmc_step"] == 0   # the other trajectories did not move


def test_dropin_module_otf_build():
    """kmos_gb300.kmc_model configured for otf: the KMC_Model sequence on the GPU equals
    the oracle run the same way (gfortran stream of the seed)."""
    from kmos_gb300 import kmc_model
    m = fixture_model("intZGB_otf")
    params = dict(zip(OTF.user_parameters(m), INTZGB_PARAMS))
    base, lattice, proclist = kmc_model.configure(m, "otf")
    proclist.init((12, 10), "IntZGB", lattice.default_layer, 7, True)
    for p, r in enumerate(INTZGB_RATES, start=1):
        base.set_rate_const(p, r)
    for name, v in params.items():
        proclist.update_user_parameter(getattr(proclist, name.lower()), v)
    proclist.recalculate_rates_matrix()
    base.update_accum_rate()
    base.update_integ_rate()
    proclist.do_kmc_steps(900)
    prog = PG.compile_model(m, "otf")
    o = O.Oracle(prog, (12, 10), seed=7, rng=O.RNG_GFORTRAN)
    o.set_rates(INTZGB_RATES)
    o.set_user_parameters(INTZGB_PARAMS)
    o.recalculate_rates_matrix()
    o.update_accum_rate()
    o.update_integ_rate()
    o.do_kmc_steps(900)
    _rm, tot = o.rates_matrix()
    assert base.get_kmc_step() == 900
    np.testing.assert_allclose(base.get_kmc_time(), o.kmc_time, rtol=1e-12)
    for p in range(1, len(INTZGB_RATES) + 1):
        assert base.get_procstat(p) == o.procstat()[p - 1]
        assert base.get_rate(p) == tot[p - 1]
    np.testing.assert_array_equal(proclist.get_occupation(), o.occupation(len(m.species)))
    lattice.deallocate_system()


def test_dropin_module_otf_put_reload_and_clock(tmp_path, monkeypatch):
    """The otf build of kmos_gb300.kmc_model under kmos.run's put (lattice.replace_species,
    proclist.touchup_cell of every cell x-outermost, base.update_accum_rate;
    run/__init__.py:1243-1314, 1439-1457) equals the oracle doing the same; then
    base.save_system / reload_system into a fresh allocation continues as the original
    would, and base.set_kmc_time sets the clock."""
    from kmos_gb300 import kmc_model
    monkeypatch.chdir(tmp_path)
    m = fixture_model("intZGB_otf")
    params = dict(zip(OTF.user_parameters(m), INTZGB_PARAMS))
    size = (9, 8)

    def setup():
        base, lattice, proclist = kmc_model.configure(m, "otf")
        return base, lattice, proclist

    base, lattice, proclist = setup()
    proclist.init(size, "otfrun", lattice.default_layer, 3, True)
    for p, r in enumerate(INTZGB_RATES, start=1):
        base.set_rate_const(p, r)
    for name, v in params.items():
        proclist.update_user_parameter(getattr(proclist, name.lower()), v)
    proclist.recalculate_rates_matrix()
    base.update_accum_rate()
    base.update_integ_rate()
    proclist.do_kmc_steps(400)
    prog = PG.compile_model(m, "otf")
    o = O.Oracle(prog, size, seed=3, rng=O.RNG_GFORTRAN)
    o.set_rates(INTZGB_RATES)
    o.set_user_parameters(INTZGB_PARAMS)
    o.recalculate_rates_matrix()
    o.update_accum_rate()
    o.update_integ_rate()
    o.do_kmc_steps(400)
    # put CO at (2, 3) and O at (7, 1): model.put = _put then _adjust_database
    for (x, y), spec in (((2, 3), proclist.co), ((7, 1), proclist.o)):
        site = [x, y, 0, 1]
        old = lattice.get_species(site)
        lattice.replace_species(site, old, spec)
        o.replace_species(_lattice2nr(size, 1, x, y, 0, 1), old, spec)
        for cx in range(size[0]):
            for cy in range(size[1]):
                proclist.touchup_cell([cx, cy, 0, 0])
                o.touchup(_lattice2nr(size, 1, cx, cy, 0, 1))
        base.update_accum_rate()
        o.update_accum_rate()
    proclist.do_kmc_steps(600)
    o.do_kmc_steps(600)
    _rm, tot = o.rates_matrix()
    assert base.get_kmc_step() == 1000
    np.testing.assert_allclose(base.get_kmc_time(), o.kmc_time, rtol=1e-12)
    for p in range(1, len(INTZGB_RATES) + 1):
        assert base.get_procstat(p) == o.procstat()[p - 1]
        assert base.get_nrofsites(p) == o.nr_of_sites()[p - 1]
        assert base.get_rate(p) == tot[p - 1]
    np.testing.assert_array_equal(proclist.get_occupation(), o.occupation(len(m.species)))
    # save_system, then reload_system into a fresh allocation
    base.save_system()
    before = [base.get_procstat(p) for p in range(1, len(INTZGB_RATES) + 1)]
    proclist.do_kmc_steps(300)
    after = ([base.get_procstat(p) for p in range(1, len(INTZGB_RATES) + 1)], base.get_kmc_time())
    lattice.deallocate_system()
    base2, lattice2, proclist2 = setup()
    assert base2.reload_system("otfrun")
    assert [base2.get_procstat(p) for p in range(1, len(INTZGB_RATES) + 1)] == before
    for name, v in params.items():
        proclist2.update_user_parameter(getattr(proclist2, name.lower()), v)
    proclist2.recalculate_rates_matrix()
    base2.update_accum_rate()
    proclist2.do_kmc_steps(300)
    assert [base2.get_procstat(p) for p in range(1, len(INTZGB_RATES) + 1)] == after[0]
    assert base2.get_kmc_time() == after[1]
    base2.set_kmc_time(0.0)
    assert base2.get_kmc_time() == 0.0
    lattice2.deallocate_system()


def _states_equal(a, b, t):
    ga, gb = a.state(t), b.state(t)
    for k in ga:
        np.testing.assert_array_equal(np.asarray(ga[k]), np.asarray(gb[k]), err_msg=k)


def test_rate_tables_give_the_programs_rates():
    """Rates looked up in the per-process tables equal the rate programs' own values bit for
    bit: two batches, tables on and off, same trajectories, including a rate-constant and a
    user-parameter change between launches (the tables are refilled) and exp / sqrt / aux
    rate expressions."""
    m = fixture_model("intZGB_otf")
    m.processes[0].otf_rate = "e = J_O_CO*nr_O_1nn + 0.5*J_CO_CO*nr_CO_1nn\notf_rate = base_rate*exp(-e)"
    m.processes[8].otf_rate = "base_rate*sqrt(1.0d0 + nr_O_1nn)/(1 + nr_CO_1nn)"
    prog = PG.compile_model(m, "otf")
    batches = []
    for on in (True, False):
        b = E.OtfBatch(prog, (14, 12), ntraj=5, seed=3, traj0=2)
        b.set_rate_tables(on)
        b.set_rates(INTZGB_RATES)
        b.set_user_parameters(INTZGB_PARAMS)
        b.recalculate_rates_matrix()
        b.update_accum_rate()
        b.update_integ_rate()
        batches.append(b)
    on, off = batches
    assert on.rate_table_entries() == 25 + 1 + 4 * 256 + 2 + 2 * 49
    for block, change in ((500, None), (700, "rate"), (900, "param")):
        for b in batches:
            if change == "rate":
                b.set_rates([r * 1.7 for r in INTZGB_RATES])
                b.recalculate_rates_matrix()
            elif change == "param":
                b.set_user_parameters([p * 0.9 for p in INTZGB_PARAMS])
                b.recalculate_rates_matrix()
            b.do_kmc_steps(block)
        for t in range(5):
            _states_equal(on, off, t)


def test_constant_rate_sums_equal_summed_lists():
    """Constant-rate processes' running sums read from their tables equal the re-summed
    lists bit for bit (every state field, and so every later pick): two batches with the
    tables on and off; between launches a rate change without recalculate_rates_matrix
    (old and new rates mixed in one list, so the lists are summed from their first
    change), then recalculate_rates_matrix (tables again), a user-parameter change, and
    the picks of get_next_kmc_step and a trace."""
    m = fixture_model("intZGB_otf")
    prog = PG.compile_model(m, "otf")
    batches = []
    for on in (True, False):
        b = E.OtfBatch(prog, (20, 18), ntraj=4, seed=9, traj0=1)
        b.set_constant_rate_sums(on)
        b.set_rates(INTZGB_RATES)
        b.set_user_parameters(INTZGB_PARAMS)
        b.recalculate_rates_matrix()
        b.update_accum_rate()
        b.update_integ_rate()
        batches.append(b)
    on, off = batches
    steps = [(400, None), (300, "rate"), (300, "recalc"), (500, "param"), (200, "recalc")]
    for block, change in steps:
        for b in batches:
            if change == "rate":
                b.set_rates([r * (1.3 if p in (1, 6, 7) else 1.0) for p, r in enumerate(INTZGB_RATES)])
            elif change == "param":
                b.set_user_parameters([p * 1.1 for p in INTZGB_PARAMS])
            elif change == "recalc":
                b.recalculate_rates_matrix()
            b.do_kmc_steps(block)
        for t in range(4):
            _states_equal(on, off, t)
    assert on.get_next_kmc_step(2) == off.get_next_kmc_step(2)
    np.testing.assert_array_equal(on.trace(3, 300), off.trace(3, 300))
    _states_equal(on, off, 3)


def _lattice2nr(size, spuck, x, y, z, n):
    X, Y = size[0], size[1]
    return spuck * (x + X * (y + Y * z)) + n


def test_put_and_adjust_database_match_oracle():
    """kmos.run's put on an otf model (run/__init__.py:1243-1314, 1439-1457):
    replace_species at some sites, touchup_cell of every cell x-outermost, then
    update_accum_rate -- on the device and in the oracle, then more steps; every table,
    rate and pick equal."""
    m = fixture_model("intZGB_otf")
    size = (10, 9)
    prog, b, (o,) = setup_both(m, size, INTZGB_RATES, INTZGB_PARAMS, 1, traj0=4)
    sp = int(prog.words[6])
    b.do_kmc_steps(700)
    o.do_kmc_steps(700)
    compare(b, 0, o)
    ids = m.species_ids()
    lat = b.state(0, ["lattice"])["lattice"]
    edits = [(3, 4), (0, 0), (9, 8), (5, 5)]
    for k, (x, y) in enumerate(edits):
        site = _lattice2nr(size, sp, x, y, 0, 1)
        old = int(lat[site - 1])
        new = [ids["CO"], ids["O"], ids["empty"], ids["CO"]][k]
        b.replace_species(0, site, old, new)
        o.replace_species(site, old, new)
    cur = int(b.state(0, ["lattice"])["lattice"][0])
    with pytest.raises(E.KMCError):
        b.replace_species(0, 1, (cur + 1) % 3, cur)   # the site holds another species
    cells = [(x, y, 0) for x in range(size[0]) for y in range(size[1])]
    b.touchup_cells(0, cells)
    for (x, y, z) in cells:
        o.touchup(_lattice2nr(size, sp, x, y, z, 1))
    b.update_accum_rate()
    o.update_accum_rate()
    compare(b, 0, o)
    b.do_kmc_steps(900)
    o.do_kmc_steps(900)
    compare(b, 0, o)


def test_set_kmc_time():
    m = fixture_model("intZGB_otf")
    _prog, b, _o = setup_both(m, (8, 8), INTZGB_RATES, INTZGB_PARAMS, 2)
    b.do_kmc_steps(50)
    b.set_kmc_time(1, 123.25)
    assert b.state(1, ["clock"])["kmc_time"] == 123.25
    assert b.state(0, ["clock"])["kmc_time"] != 123.25
    b.do_kmc_steps(10)
    assert b.state(1, ["clock"])["kmc_time"] > 123.25


def test_reload_round_trip_continues_bit_for_bit(tmp_path):
    """save_system of one trajectory, reload_system into a fresh batch (the file's
    lattice, avail_sites, counters, clock, rate constants and random stream; rates_matrix
    rebuilt by recalculate_rates_matrix as kmos.run does), then both run on: every state
    field equal.  The file is the reference's layout: the oracle's reader takes it."""
    m = fixture_model("intZGB_otf")
    size = (12, 10)
    prog = PG.compile_model(m, "otf")
    a = E.OtfBatch(prog, size, ntraj=3, seed=5, rng=E.RNG_PHILOX)
    a.set_rates(INTZGB_RATES)
    a.set_user_parameters(INTZGB_PARAMS)
    a.recalculate_rates_matrix()
    a.update_accum_rate()
    a.update_integ_rate()
    a.do_kmc_steps(800)
    path = str(tmp_path / "otf.reload")
    a.save_reload(2, path, walltime=3.5)
    b = E.OtfBatch(prog, size, ntraj=1, seed=1, rng=E.RNG_PHILOX)
    b.set_user_parameters(INTZGB_PARAMS)
    assert b.load_reload(0, path) == pytest.approx(3.5)
    np.testing.assert_array_equal(b.rate_consts(), np.array(INTZGB_RATES))
    ga, gb = a.state(2), b.state(0)
    for k in ("lattice", "as1", "as2", "nsites", "procstat", "integ"):
        np.testing.assert_array_equal(ga[k], gb[k], err_msg=k)
    assert (ga["kmc_time"], ga["kmc_time_step"], ga["kmc_step"]) == (gb["kmc_time"], gb["kmc_time_step"], gb["kmc_step"])
    for x in (a, b):
        x.recalculate_rates_matrix()
        x.update_accum_rate()
    ga, gb = a.state(2), b.state(0)
    np.testing.assert_array_equal(ga["rates_matrix"], gb["rates_matrix"])
    a.do_kmc_steps(1500)
    b.do_kmc_steps(1500)
    ga, gb = a.state(2), b.state(0)
    for k in ga:
        np.testing.assert_array_equal(np.asarray(ga[k]), np.asarray(gb[k]), err_msg=k)
    from oracle import reload as R
    f = R.read_reload(path)
    assert f["nr_of_proc"] == len(m.processes) and f["volume"] == size[0] * size[1]
    saved = E.OtfBatch(prog, size, ntraj=1, seed=1, rng=E.RNG_PHILOX)
    saved.load_reload(0, path)
    g = saved.state(0)
    np.testing.assert_array_equal(f["lattice"], g["lattice"])
    np.testing.assert_array_equal(f["nr_of_sites"], g["nsites"])
    np.testing.assert_array_equal(f["procstat"], g["procstat"])
    for p in range(1, len(m.processes) + 1):
        np.testing.assert_array_equal(f["as1"][p], g["as1"][p - 1, 1:])
        np.testing.assert_array_equal(f["as2"][p], g["as2"][p - 1, 1:])
    with pytest.raises(E.KMCError):
        b.set_state(0, np.full(b.V, 99), np.zeros((b.P, b.V + 1)), np.zeros(b.P), np.zeros(b.P))
