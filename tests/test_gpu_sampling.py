"""On-device sampling (kmc_pool_sample_*, kmos_gb300.sampling.get_std_sampled_data)
against get_std_sampled_data (kmos/run/__init__.py:865-966): the reference's own code's
outputs on oracle trajectories (tests/golden/sampling.json) and the oracle's
restatement (oracle/sampling.py) on a batch of mixed trajectories.

Tolerances: kMC step counts exact; times, TOFs and occupation means within 1e-12
relative (the device log() and glibc's log() may differ in the last place, and the TOF
is formed from the total differences instead of per-batch terms)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, fixture_model
from kmos_gb300 import engine as E, program as PG, rates as R, sampling as S
from oracle import oracle as O, sampling as OS

pytestmark = pytest.mark.gpu
RTOL = 1e-12
CASES = json.load(open(os.path.join(GOLDEN, "sampling.json")))


def case_rates(model, name):
    if name == "AB_model":
        return json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    return [float(r) for r in R.model_rates(model)]


def close(got, want):
    got, want = np.asarray(got, float), np.asarray(want, float)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=RTOL, atol=1e-300)


@pytest.mark.parametrize("i", range(len(CASES)), ids=[c["model"] + "-" + c["tof_method"] for c in CASES])
def test_matches_reference_code(i):
    c = CASES[i]
    m = fixture_model(c["model"])
    prog = PG.compile_model(m, c["backend"])
    pool = E.Pool(arena_bytes=1 << 26, max_slots=4)
    mid = pool.add_model(prog)
    s = pool.admit(mid, c["size"], case_rates(m, c["model"]), seed=c["seed"], rng=c["rng"], traj=c["traj"])
    pool.run([s], c["warmup_steps"])
    got = S.get_std_sampled_data(pool, [s], m, c["samples"], c["sample_size"], tof_method=c["tof_method"])
    close(got[0], c["values"])
    assert got[0][-1] == c["values"][-1]
    d = S.get_std_sampled_data(pool, [s], m, 2, 100, tof_method=c["tof_method"], output="dict")[0]
    assert list(d) == c["header"][1:].split()
    pool.close()


def test_batch_matches_restatement():
    """64 trajectories of three models in one pool, sampled together; each checked
    against the restatement run on its own oracle trajectory."""
    specs = [("pairwise_interaction", "lat_int"), ("CO_oxidation_Ruo2", "local_smart"), ("ZGB_model", "lat_int")]
    models = [fixture_model(n) for n, _ in specs]
    progs = [PG.compile_model(m, b) for m, (_, b) in zip(models, specs)]
    pool = E.Pool(arena_bytes=1 << 28, max_slots=128)
    mids = [pool.add_model(p) for p in progs]
    rng = np.random.default_rng(8)
    items = []
    for j in range(64):
        k = j % 3
        size = (int(rng.integers(6, 20)), int(rng.integers(6, 20)))
        rates = (10.0 ** rng.uniform(-1, 2, size=progs[k].nproc)).tolist()
        s = pool.admit(mids[k], size, rates, seed=40 + j, rng=E.RNG_PHILOX, traj=j)
        items.append((k, s, size, rates, 40 + j, j))
    slots = [s for _, s, *_ in items]
    pool.run(slots, 300)
    samples, sample_size = 4, 2002
    out = pool.sample_run(slots, samples, int(sample_size / samples))
    for idx, (k, s, size, rates, seed, traj) in enumerate(items):
        if idx % 4:
            continue  # every fourth trajectory against the oracle
        m = models[k]
        o = O.Oracle(progs[k], size, seed=seed, rng=O.RNG_PHILOX, traj=traj)
        o.set_rates(rates)
        o.update_accum_rate()
        o.do_kmc_steps(300)
        names, mat = OS.tof_matrix(m)
        trk = OS.Trackers(len(m.processes), len(names))
        p0, i0 = o.procstat(), o.integ_rates()
        want = OS.std_sampled_data(o, trk, mat, size[0] * size[1], len(m.species), samples, sample_size, "integ")
        nocc = len(m.species) * m.spuck
        ntof = len(names)
        close(out["occ"][idx][:nocc], want[ntof:ntof + nocc])
        close(out["times"][idx], want[-3:-1])
        assert out["steps"][idx] == want[-1]
        assert out["status"][idx] == 0
        np.testing.assert_array_equal(out["dprocstat"][idx][:len(m.processes)], o.procstat() - p0)
        np.testing.assert_allclose(out["dinteg"][idx][:len(m.processes)], o.integ_rates() - i0, rtol=0,
                                   atol=RTOL * np.abs(o.integ_rates()).max())
    pool.close()


def test_manual_sampling_equals_sample_run():
    prog = PG.compile_model(fixture_model("CO_oxidation_Ruo2"), "local_smart")
    pools = []
    for _ in range(2):
        pool = E.Pool(arena_bytes=1 << 27, max_slots=16)
        mid = pool.add_model(prog)
        slots = [pool.admit(mid, (8 + j, 9), (10.0 ** np.linspace(-1, 2, prog.nproc)).tolist(), seed=3, traj=j)
                 for j in range(8)]
        pools.append((pool, slots))
    (a, sa), (b, sb) = pools
    ra = a.sample_run(sa, 3, 700)
    b.sample_begin(sb)
    for _ in range(3):
        b.run(sb, 700, sync=False)
        b.sample(sb)
    rb = b.sample_end(sb)
    for key in ra:
        np.testing.assert_array_equal(ra[key], rb[key])
    with pytest.raises(E.KMCError):
        b.sample(sb)  # the records were freed by sample_end
    free0 = a.free_bytes()[0]
    a.sample_begin(sa)
    assert a.free_bytes()[0] < free0
    a.release(sa[0])  # a released slot gives its record back too
    a.sample_end(sa[1:])
    a.close()
    b.close()
