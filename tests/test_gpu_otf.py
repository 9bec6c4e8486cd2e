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
