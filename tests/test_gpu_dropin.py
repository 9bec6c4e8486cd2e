"""The f2py-compatible drop-in driven the way kmos.run.KMC_Model drives kmc_model
(kmos/run/__init__.py: reset 243-339, set_rate_constants 2369-2437, run_proc_nr
1357-1363, do_steps 416-432, get_atoms 680-850)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from kmos_gb300 import kmc_model, model as M, rates as R
from oracle import oracle as O
from kmos_gb300 import program as PG

pytestmark = pytest.mark.gpu


def reset(name, size=20, seed=1, backend="local_smart"):
    m = M.load_json(os.path.join(GOLDEN, "models", name + ".json"))
    base, lattice, proclist = kmc_model.configure(m, backend)
    proclist.init(np.array([size] * int(lattice.model_dimension)), "kmc_model", lattice.default_layer, seed, True)
    params = {p.name: {"value": p.value} for p in m.parameters}
    for proc in sorted(p.name for p in m.processes):  # set_rate_constants: sorted names
        expr = [p for p in m.processes if p.name == proc][0].rate_constant
        base.set_rate_const(getattr(proclist, proc.lower()), R.evaluate_rate_expression(expr, params))
    base.update_accum_rate()
    base.update_integ_rate()
    return m, base, lattice, proclist


def test_golden_trajectory_through_the_drop_in():
    ref = np.load(os.path.join(GOLDEN, "ab_model_ref_procs_sites.npy"))
    _m, base, lattice, proclist = reset("AB_model")
    out = []
    for _ in range(len(ref)):
        proc, site = proclist.get_next_kmc_step()
        out.append((proc, site))
        if base.get_avail_site(proc, site, 2):  # KMC_Model.run_proc_nr
            proclist.run_proc_nr(proc, site)
    lattice.deallocate_system()
    np.testing.assert_array_equal(np.array(out), ref)


@pytest.mark.parametrize("name,backend", [("ZGB_model", "local_smart"), ("pairwise_interaction", "lat_int"),
                                          ("default_xml", "local_smart")])
def test_do_steps_and_tof_readout_match_the_oracle(name, backend):
    m, base, lattice, proclist = reset(name, size=16, seed=3, backend=backend)
    rates = [base.get_rate(i) for i in range(1, proclist.nr_of_proc + 1)]
    o = O.Oracle(PG.compile_model(m, backend), (16, 16), seed=3)
    o.set_rates(rates)
    o.update_accum_rate()
    t0, k0 = base.get_kmc_time(), base.get_kmc_step()
    ps0 = np.array([base.get_procstat(i) for i in range(1, proclist.nr_of_proc + 1)])
    proclist.do_kmc_steps(20000)
    o.do_kmc_steps(20000)
    dt = base.get_kmc_time() - t0
    assert base.get_kmc_step() - k0 == 20000 == o.kmc_step
    assert abs(base.get_kmc_time() - o.kmc_time) <= 1e-12 * o.kmc_time
    ps = np.array([base.get_procstat(i) for i in range(1, proclist.nr_of_proc + 1)])
    np.testing.assert_array_equal(ps, o.procstat())
    tof = (ps - ps0) / dt / (16 * 16)  # get_atoms: procstat deltas per unit time and cell
    np.testing.assert_allclose(tof, (o.procstat() - ps0) / o.kmc_time / 256, rtol=1e-11)
    integ = np.array([base.get_integ_rate(i) for i in range(1, proclist.nr_of_proc + 1)])
    np.testing.assert_allclose(integ, o.integ_rates(), rtol=1e-12)
    np.testing.assert_array_equal(proclist.get_occupation()[:m.species_ids().__len__()],
                                  o.occupation(len(m.species)))
    sites = [lattice.calculate_nr2lattice(s) for s in (1, 7, 100)]
    assert [lattice.calculate_lattice2nr(x) for x in sites] == [1, 7, 100]
    assert [lattice.get_species(x) for x in sites] == [o.get_species(s) for s in (1, 7, 100)]
    lattice.deallocate_system()


@pytest.mark.parametrize("name,backend", [("ZGB_model", "local_smart"), ("ZGB_model", "lat_int"),
                                          ("CO_oxidation_Ruo2", "local_smart")])
def test_put_and_adjust_database(name, backend):
    """kmos.run's put (lattice.replace_species, then _adjust_database: a touch-up of every
    site -- every cell for lat_int -- in order, then update_accum_rate;
    kmos/run/__init__.py:1243-1314, 1439-1457) through the drop-in module, whose queued
    touch-ups run as one launch, against the oracle making the same calls one by one."""
    m, base, lattice, proclist = reset(name, size=10, seed=4, backend=backend)
    prog = PG.compile_model(m, backend)
    P = prog.nproc
    o = O.Oracle(prog, (10, 10), layer=lattice.default_layer, seed=4, rng=O.RNG_GFORTRAN)
    o.set_rates([base.get_rate(p) for p in range(1, P + 1)])
    o.update_accum_rate()
    proclist.do_kmc_steps(400)
    o.do_kmc_steps(400)
    rng = np.random.default_rng(9)
    X, Y, spuck = 10, 10, int(lattice.spuck)
    nspecies = len(m.species)
    for _ in range(12):  # put
        x, y, n = int(rng.integers(0, X)), int(rng.integers(0, Y)), int(rng.integers(1, spuck + 1))
        new = int(rng.integers(0, nspecies))
        old = lattice.get_species([x, y, 0, n])
        lattice.replace_species([x, y, 0, n], old, new)
        o.replace_species(lattice.calculate_lattice2nr([x, y, 0, n]), old, new)
    touch = sorted(a for a in dir(proclist) if a.startswith("touchup_"))
    for x in range(X):  # _adjust_database
        for y in range(Y):
            if backend == "lat_int":
                proclist.touchup_cell([x, y, 0, 0])
                o.touchup(lattice.calculate_lattice2nr([x, y, 0, 1]))
            else:
                for n in range(spuck):
                    getattr(proclist, touch[n])([x, y, 0, n + 1])
                    o.touchup(lattice.calculate_lattice2nr([x, y, 0, n + 1]))
    base.update_accum_rate()
    o.update_accum_rate()
    ex = o.export()
    for p in range(1, P + 1):
        n_p = base.get_nrofsites(p)
        assert n_p == ex["nsites"][p - 1]
        assert [base.get_avail_site(p, i, 1) for i in range(1, n_p + 1)] == list(ex["as1"][p - 1, 1:n_p + 1])
        assert base.get_accum_rate(p) == o.accum_rates()[p - 1]
    proclist.do_kmc_steps(3000)
    o.do_kmc_steps(3000)
    ex = o.export()
    assert base.get_kmc_step() == o.kmc_step
    assert [base.get_nrofsites(p) for p in range(1, P + 1)] == list(ex["nsites"])
    assert [lattice.get_species(lattice.calculate_nr2lattice(s)) for s in range(1, o.V + 1)] == list(ex["lattice"])
    lattice.deallocate_system()
