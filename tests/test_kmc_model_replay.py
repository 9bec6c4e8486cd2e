"""The reference's kmos.run.KMC_Model over the drop-in module, replayed on the CPU.

tests/golden/kmc_model_run.json holds every call the reference's own KMC_Model code
(kmos/run/__init__.py: reset, do_steps, get_atoms, get_std_sampled_data, run_proc_nr,
put / _adjust_database, deallocate) made on kmc_model's base / lattice / proclist, with
the results the drop-in returned (tests/golden/make_kmc_model_run.py).  Here the log is
replayed on a fresh drop-in whose engine is the oracle, which checks the replay itself
and the drop-in's own arithmetic (lattice mapping, constants, argument conventions);
tests/test_gpu_kmc_model_run.py replays it on the GPU engine."""
import json
import os

import pytest

import dropin_replay as DR
from conftest import GOLDEN, fixture_model
from kmos_gb300 import engine as E, kmc_model

CASES = json.load(open(os.path.join(GOLDEN, "kmc_model_run.json")))


@pytest.mark.parametrize("case", CASES, ids=[c["model"] + "-" + c["backend"] for c in CASES])
def test_replay_on_the_oracle_engine(case, monkeypatch):
    monkeypatch.setattr(E, "Trajectory", DR.OracleTrajectory)
    base, lattice, proclist = kmc_model.configure(fixture_model(case["model"]), case["backend"])
    DR.replay(case["log"], {"base": base, "lattice": lattice, "proclist": proclist})
    assert not base.is_allocated()  # the log ends with KMC_Model.deallocate


def test_the_log_covers_the_kmc_model_calls():
    """The recorded sequences reach the engine through every kind of call KMC_Model makes
    on this path."""
    calls = {(e["ns"], e["attr"]) for c in CASES for e in c["log"] if e["op"] == "call"}
    for want in [("proclist", "init"), ("base", "set_rate_const"), ("base", "update_accum_rate"),
                 ("base", "update_integ_rate"), ("proclist", "do_kmc_steps"), ("base", "get_kmc_time"),
                 ("base", "get_kmc_step"), ("base", "get_procstat"), ("base", "get_integ_rate"),
                 ("proclist", "get_occupation"), ("base", "get_kmc_time_step"), ("proclist", "get_next_kmc_step"),
                 ("base", "get_avail_site"), ("proclist", "run_proc_nr"), ("lattice", "get_species"),
                 ("lattice", "replace_species"), ("proclist", "touchup_cell"), ("lattice", "deallocate_system"),
                 ("base", "is_allocated")]:
        assert want in calls, want
