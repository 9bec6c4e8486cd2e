"""Independent random streams give statistically equal results: the engine on Philox
streams against the oracle on the gfortran stream (the reference's own generator), same
model and parameters, compared through get_std_sampled_data's estimators (time-weighted
coverages, TOF from procstat).  Each quantity's trajectory means must agree within 3
standard errors of their difference.  Seeds are fixed, so the outcome is deterministic."""
import numpy as np
import pytest

from kmos_gb300 import configs, engine as E, sampling as S
from oracle import oracle as O, sampling as OS

pytestmark = pytest.mark.gpu


def test_tof_and_coverage_agree_within_3_se():
    m = configs.model_config2()
    y = 0.48
    rates = [y] + [(1 - y) / 4] * 4 + [1e6] * 4
    prog = configs.compile_model(m, "local_smart")
    size, warm, samples, sample_size = (20, 20, 1), 20000, 10, 20000
    names, mat = S.tof_matrix(m)
    nocc = len(m.species) * m.spuck

    pool = E.Pool(arena_bytes=256 << 20, max_slots=256)
    mid = pool.add_model(prog)
    n_gpu = 128
    slots = pool.admit_many([mid] * n_gpu, [size] * n_gpu, [rates] * n_gpu, seeds=[77] * n_gpu,
                            rng=E.RNG_PHILOX, trajs=list(range(n_gpu)))
    pool.run(slots, warm)
    gpu = S.get_std_sampled_data(pool, slots, m, samples, sample_size, tof_method="procrates")
    status = pool.results(slots, 1)[4]
    pool.close()
    assert (status == 0).all(), "a trajectory poisoned; the comparison assumes the reactive regime"

    rows = []
    for seed in range(1, 33):
        o = O.Oracle(prog, size, seed=seed, rng=O.RNG_GFORTRAN)
        o.set_rates(rates)
        o.update_accum_rate()
        o.do_kmc_steps(warm)
        trk = OS.Trackers(len(m.processes), len(names))
        rows.append(OS.std_sampled_data(o, trk, mat, 400, len(m.species), samples, sample_size, "procrates"))
    ora = np.array(rows)

    # columns: tof (1), coverages (species sorted by name), total_time, simulated_time, steps
    species = sorted(m.species)
    cols = {"tof": 0}
    cols.update({"cov_" + sp: 1 + i for i, sp in enumerate(species)})
    for name, c in cols.items():
        a, b = gpu[:, c], ora[:, c]
        se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
        assert abs(a.mean() - b.mean()) <= 3 * se, (name, a.mean(), b.mean(), se)
    assert gpu[:, 0].mean() > 0  # the reactive regime: CO2 is made
