"""The get_std_sampled_data restatement (oracle/sampling.py) against the reference's
own code: tests/golden/sampling.json holds what kmos.run.KMC_Model.get_std_sampled_data
(kmos/run/__init__.py:865-966) returned on oracle trajectories (make_sampling_golden.py)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, fixture_model
from kmos_gb300 import program as PG, rates as R, sampling as S
from oracle import oracle as O, sampling as OS

CASES = json.load(open(os.path.join(GOLDEN, "sampling.json")))


def case_rates(model, name):
    if name == "AB_model":
        return json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    return [float(r) for r in R.model_rates(model)]


def oracle_case(c):
    m = fixture_model(c["model"])
    prog = PG.compile_model(m, c["backend"])
    o = O.Oracle(prog, c["size"], seed=c["seed"], rng=c["rng"], traj=c["traj"])
    o.set_rates(case_rates(m, c["model"]))
    o.update_accum_rate()
    o.do_kmc_steps(c["warmup_steps"])
    return m, o


@pytest.mark.parametrize("i", range(len(CASES)), ids=[c["model"] + "-" + c["tof_method"] for c in CASES])
def test_restatement_matches_reference_code(i):
    c = CASES[i]
    m, o = oracle_case(c)
    names, mat = OS.tof_matrix(m)
    params = [float({p.name: p.value for p in m.parameters}[k]) for k in S.param_names(m)]
    trk = OS.Trackers(len(m.processes), len(names))
    cells = int(np.prod(c["size"]))
    got = OS.std_sampled_data(o, trk, mat, cells, len(m.species), c["samples"], c["sample_size"],
                              c["tof_method"], params)
    np.testing.assert_array_equal(got, np.array(c["values"]))


@pytest.mark.parametrize("i", range(0, len(CASES), 2), ids=[c["model"] for c in CASES[::2]])
def test_header_matches_reference(i):
    c = CASES[i]
    assert S.std_header(fixture_model(c["model"])) == c["header"]
