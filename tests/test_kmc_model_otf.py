"""The drop-in module's otf build (kmos_gb300/kmc_model.py) on the CPU: the sequence
kmos.run's KMC_Model runs for an otf model (init, set_rate_const, update_user_parameter
through proclist, recalculate_rates_matrix, update_accum_rate / update_integ_rate,
do_kmc_steps, the getters) with the engine's otf batch replaced by an oracle-backed
stand-in, so that the namespaces' argument conventions and read-outs are checked
without a GPU.  The engine's otf calls themselves are checked on the GPU
(tests/test_gpu_otf.py)."""
import numpy as np

from conftest import fixture_model
from kmos_gb300 import engine as E, kmc_model, otf as OTF, program as PG
from oracle import oracle as O


class OracleOtfBatch:
    """engine.OtfBatch's interface for one trajectory, run by the oracle (test only)."""

    def __init__(self, program, size, ntraj=1, layer=0, seed=1, rng=E.RNG_PHILOX, traj0=0):
        assert ntraj == 1
        self.o = O.Oracle(program, size, layer=layer, seed=seed, rng=rng, traj=traj0)
        self.P, self.V, self.spuck = self.o.P, self.o.V, self.o.spuck
        self.size = [int(v) for v in (list(size) + [1, 1])[:3]]

    def close(self):
        pass

    def set_rate_const(self, proc, rate):
        O.lib().oracle_set_rate_const(self.o.h, int(proc), float(rate))

    def set_user_parameter(self, k, value):
        O.lib().oracle_set_user_parameter(self.o.h, int(k), float(value))

    def recalculate_rates_matrix(self):
        self.o.recalculate_rates_matrix()

    def update_accum_rate(self):
        self.o.update_accum_rate()

    def update_integ_rate(self):
        self.o.update_integ_rate()

    def do_kmc_steps(self, n):
        self.o.do_kmc_steps(n)

    def get_next_kmc_step(self, traj=0):
        return self.o.get_next_kmc_step()

    def run_proc_nr(self, proc, site, traj=0):
        self.o.run_proc_nr(proc, site)

    def replace_species(self, traj, site, old, new):
        if self.o.get_species(site) != old:
            raise E.KMCError(2, "replace_species: the site holds another species")
        self.o.replace_species(site, old, new)

    def touchup_cells(self, traj, cells):
        X, Y = self.size[0], self.size[1]
        for x, y, z in np.asarray(cells).reshape(-1, 3):
            self.o.touchup(self.spuck * (int(x) + X * (int(y) + Y * int(z))) + 1)

    def state(self, traj=0, fields=None):
        ex = self.o.export()
        rm, tot = self.o.rates_matrix()
        return dict(lattice=ex["lattice"], as1=ex["as1"], as2=ex["as2"], nsites=ex["nsites"],
                    procstat=ex["procstat"], integ=ex["integ"], accum=self.o.accum_rates(), rates_matrix=rm,
                    totals=tot, kmc_time=self.o.kmc_time, kmc_time_step=self.o.kmc_time_step,
                    kmc_step=self.o.kmc_step)


def test_otf_dropin_sequence(monkeypatch):
    monkeypatch.setattr(E, "OtfBatch", OracleOtfBatch)
    m = fixture_model("intZGB_otf")
    rates = [0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3]
    params = {"J_CO_CO": 1.3, "J_O_CO": 0.7, "J_O_O": 1.9, "kDes": 1e-10, "yCO": 0.5}
    base, lattice, proclist = kmc_model.configure(m, "otf")
    assert proclist.backend == "otf" and kmc_model.proclist_pars.byst_co_ads == "nr_CO_1nn nr_O_1nn"
    proclist.init((12, 10), "IntZGB", lattice.default_layer, 7, True)
    for p, r in enumerate(rates, start=1):
        base.set_rate_const(p, r)
    for name, v in params.items():                      # set_rate_constants, run:2416-2427
        proclist.update_user_parameter(getattr(proclist, name.lower()), v)
    assert kmc_model.proclist_pars.get_user_parameter(proclist.j_o_co) == 0.7
    proclist.recalculate_rates_matrix()
    base.update_accum_rate()
    base.update_integ_rate()
    proclist.do_kmc_steps(800)

    prog = PG.compile_model(m, "otf")
    o = O.Oracle(prog, (12, 10), seed=7, rng=O.RNG_GFORTRAN)
    o.set_rates(rates)
    o.set_user_parameters([params[n] for n in OTF.user_parameters(m)])
    o.recalculate_rates_matrix()
    o.update_accum_rate()
    o.update_integ_rate()
    o.do_kmc_steps(800)
    rm, tot = o.rates_matrix()
    ex = o.export()
    assert base.get_kmc_step() == 800 and base.get_kmc_time() == o.kmc_time
    for p in range(1, len(rates) + 1):
        assert base.get_procstat(p) == ex["procstat"][p - 1]
        assert base.get_nrofsites(p) == ex["nsites"][p - 1]
        assert base.get_rate(p) == tot[p - 1]
        if ex["nsites"][p - 1]:
            assert base.get_rate(p, 1) == rm[p - 1, 1]
            assert base.get_avail_site(p, 1, 1) == ex["as1"][p - 1, 1]
        assert base.get_integ_rate(p) == ex["integ"][p - 1]
        assert base.get_accum_rate(p) == o.accum_rates()[p - 1]
    np.testing.assert_array_equal(proclist.get_occupation(), o.occupation(len(m.species)))
    assert lattice.get_species((3, 4, 0, 1)) == ex["lattice"][3 + 12 * 4]
    p, s = proclist.get_next_kmc_step()
    assert (p, s) == o.get_next_kmc_step()
    proclist.run_proc_nr(p, s)
    o.run_proc_nr(p, s)
    np.testing.assert_array_equal(proclist.get_occupation(), o.occupation(len(m.species)))
    # kmos.run's put (run/__init__.py:1243-1314): replace_species, then _adjust_database
    # (touchup_cell of every cell, x outermost; 1439-1457) and update_accum_rate
    import pytest
    old = lattice.get_species((0, 0, 0, 1))
    with pytest.raises(E.KMCError):
        lattice.replace_species((0, 0, 0, 1), (old + 1) % 3, 1)
    new = (old + 1) % 3
    lattice.replace_species((0, 0, 0, 1), old, new)
    o.replace_species(1, old, new)
    for x in range(12):
        for y in range(10):
            proclist.touchup_cell([x, y, 0, 0])
            o.touchup(1 + x + 12 * y)
    base.update_accum_rate()
    o.update_accum_rate()
    proclist.do_kmc_steps(300)
    o.do_kmc_steps(300)
    ex = o.export()
    assert base.get_kmc_time() == o.kmc_time
    for p in range(1, len(rates) + 1):
        assert base.get_procstat(p) == ex["procstat"][p - 1]
        assert base.get_nrofsites(p) == ex["nsites"][p - 1]
    lattice.deallocate_system()
    assert not base.is_allocated()


def test_otf_build_has_every_attribute_kmos_run_reads(tmp_path):
    """The attributes kmos.run and the CLI read (tests/golden/kmc_model_attrs.json), on an
    otf build, but the chemical-potential update (not offered) and names from docstring
    examples; and an otf export directory imports with proclist_pars."""
    import importlib
    import json
    import os
    import sys
    from conftest import GOLDEN
    from kmos_gb300 import export
    want = json.load(open(os.path.join(GOLDEN, "kmc_model_attrs.json")))
    skip = {"lattice_bridge", "site", "co", "touchup_", "update_chempot"}
    base, lattice, proclist = kmc_model.configure(fixture_model("intZGB_otf"), "otf")
    for mod, obj in {"base": base, "lattice": lattice, "proclist": proclist}.items():
        missing = [a for a in want[mod] if a not in skip and not hasattr(obj, a)]
        assert not missing, (mod, missing)
    out = os.path.join(str(tmp_path), "out")
    export.export(os.path.join(GOLDEN, "models", "intZGB_otf.json"), out, "otf")
    sys.path.insert(0, out)
    for mod in ("kmc_settings", "kmc_model"):
        sys.modules.pop(mod, None)
    try:
        drop_in = importlib.import_module("kmc_model")
        assert drop_in.proclist.backend == "otf"
        assert drop_in.proclist_pars.byst_co_ads == "nr_CO_1nn nr_O_1nn"
        assert drop_in.proclist_pars.j_o_co == drop_in.proclist.j_o_co == 2
    finally:
        sys.path.remove(out)
        for mod in ("kmc_settings", "kmc_model"):
            sys.modules.pop(mod, None)


def test_rate_functions_of_proclist_pars(monkeypatch):
    """proclist_pars.rate_<name>(nr_vars) and byst_<name>, as kmos.run's
    Model_Rate_Constants_OTF calls them (run:1868-1882): the rate for given bystander
    counts from the current rate constant and user parameters."""
    monkeypatch.setattr(E, "OtfBatch", OracleOtfBatch)
    m = fixture_model("intZGB_otf")
    base, lattice, proclist = kmc_model.configure(m, "otf")
    pars = kmc_model.proclist_pars
    proclist.init((6, 6), "IntZGB", lattice.default_layer, 1, True)
    base.set_rate_const(proclist.co_ads, 0.25)
    for name, v in {"J_CO_CO": 1.3, "J_O_CO": 0.7}.items():
        proclist.update_user_parameter(getattr(proclist, name.lower()), v)
    nr_vars = pars.byst_co_ads.split()            # ['nr_CO_1nn', 'nr_O_1nn']
    counts = np.zeros(len(nr_vars), int)
    counts[nr_vars.index("nr_CO_1nn")], counts[nr_vars.index("nr_O_1nn")] = 2, 1
    want = (0.25 * OTF.powi(0.7, 1, OTF.K_F64)) * OTF.powi(1.3, 2, OTF.K_F64)
    assert pars.rate_co_ads(counts) == want
    assert pars.rate_co_des() == 0.0 and pars.byst_co_des == ""
    lattice.deallocate_system()


def test_chemical_potentials(monkeypatch):
    """mu_* in an otf_rate: the generator's chempots array, set by update_chempot
    (io:2740-2790), here the entries after the user parameters.  Every CO_ads entry's
    rate after recalculate_rates_matrix is base_rate * exp(-mu_CO * nr_CO_1nn) of its cell."""
    import math
    monkeypatch.setattr(E, "OtfBatch", OracleOtfBatch)
    m = fixture_model("intZGB_otf")
    m.processes[0].otf_rate = "base_rate*exp(-mu_CO*nr_CO_1nn)"
    assert OTF.chempot_names(m) == ["mu_CO"]
    assert int(PG.compile_model(m, "otf").words[23]) == len(m.parameters) + 1
    base, lattice, proclist = kmc_model.configure(m, "otf")
    pars = kmc_model.proclist_pars
    proclist.init((8, 8), "IntZGB", lattice.default_layer, 3, True)
    rates = [0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3]
    for p, r in enumerate(rates, start=1):
        base.set_rate_const(p, r)
    pars.update_chempot(pars.mu_co, 0.35)
    assert pars.chempots[0] == 0.35
    proclist.recalculate_rates_matrix()
    proclist.do_kmc_steps(300)        # every event keeps the touched rates current
    st = kmc_model._state.traj.b.state(0)
    lat = st["lattice"]
    co = proclist.co
    n = base.get_nrofsites(proclist.co_ads)
    assert n > 0
    for i in range(1, n + 1):
        site = base.get_avail_site(proclist.co_ads, i, 1)
        x, y = (site - 1) % 8, (site - 1) // 8
        nco = sum(lat[((x + dx) % 8) + 8 * ((y + dy) % 8)] == co for dx, dy in ((1, 0), (0, 1), (-1, 0), (0, -1)))
        assert base.get_rate(proclist.co_ads, i) == 0.4 * math.exp(-(0.35 * nco))
    lattice.deallocate_system()


def test_mu_names_are_chemical_potentials_even_when_a_parameter_has_the_name(monkeypatch):
    """The reference's _parse_otf_rate (io:3086-3090) tests ``mu_`` before the user
    parameters, so a parameter named mu_CO never shadows the chemical potential: the
    rate reads chempots, not the parameter's value."""
    import math
    from kmos_gb300 import model as M
    monkeypatch.setattr(E, "OtfBatch", OracleOtfBatch)
    m = fixture_model("intZGB_otf")
    m.parameters.append(M.Parameter(name="mu_CO", value="9.0"))
    m.processes[0].otf_rate = "base_rate*exp(-mu_CO*nr_CO_1nn)"
    assert OTF.chempot_names(m) == ["mu_CO"]
    base, lattice, proclist = kmc_model.configure(m, "otf")
    pars = kmc_model.proclist_pars
    proclist.init((8, 8), "IntZGB", lattice.default_layer, 3, True)
    for p, r in enumerate([0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3], start=1):
        base.set_rate_const(p, r)
    pars.update_chempot(pars.mu_co, 0.35)
    proclist.recalculate_rates_matrix()
    proclist.do_kmc_steps(300)
    lat = kmc_model._state.traj.b.state(0)["lattice"]
    n = base.get_nrofsites(proclist.co_ads)
    assert n > 0
    for i in range(1, n + 1):
        site = base.get_avail_site(proclist.co_ads, i, 1)
        x, y = (site - 1) % 8, (site - 1) // 8
        nco = sum(lat[((x + dx) % 8) + 8 * ((y + dy) % 8)] == proclist.co
                  for dx, dy in ((1, 0), (0, 1), (-1, 0), (0, -1)))
        assert base.get_rate(proclist.co_ads, i) == 0.4 * math.exp(-(0.35 * nco))
    lattice.deallocate_system()


def test_an_expression_that_does_not_tokenize_is_refused():
    """As the reference raises on a tokenize error (io:3080-3085), so does the compiler."""
    import pytest
    m = fixture_model("intZGB_otf")
    m.processes[0].otf_rate = "base_rate*exp(-(mu_CO*nr_CO_1nn)"
    with pytest.raises(OTF.ExprError):
        OTF.chempot_names(m)
    with pytest.raises(OTF.ExprError):
        PG.compile_model(m, "otf")
