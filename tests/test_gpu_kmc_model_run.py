"""The reference's kmos.run.KMC_Model over the drop-in module, on the GB300.

tests/golden/kmc_model_run.json holds every call the reference's own KMC_Model code
(kmos/run/__init__.py: reset 243-339 with set_rate_constants 2369-2437, do_steps 416-432,
get_atoms 680-850, get_std_sampled_data 865-966, run_proc_nr / get_next_kmc_step
1357-1367, put / _adjust_database 1288-1314 and 1439-1457, deallocate 388-414) made on
kmc_model's base / lattice / proclist, recorded with the oracle as the engine
(tests/golden/make_kmc_model_run.py).  Replayed here on the GPU engine, every result must
be the one the reference's code received: integers, tables and occupations exactly,
kmc_time, kmc_time_step and integ_rates within 1e-12 relative."""
import json
import os

import pytest

import dropin_replay as DR
from conftest import GOLDEN, fixture_model
from kmos_gb300 import kmc_model

pytestmark = pytest.mark.gpu
CASES = json.load(open(os.path.join(GOLDEN, "kmc_model_run.json")))


@pytest.mark.parametrize("case", CASES, ids=[c["model"] + "-" + c["backend"] for c in CASES])
def test_replay_on_the_gpu_engine(case):
    base, lattice, proclist = kmc_model.configure(fixture_model(case["model"]), case["backend"])
    DR.replay(case["log"], {"base": base, "lattice": lattice, "proclist": proclist})
    assert not base.is_allocated()
