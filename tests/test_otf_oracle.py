"""The oracle's otf backend (oracle/kmc_oracle.c, backend 2).

* The reference's golden trajectory (tests/test_run: 20x20 AB model, seed 1, gfortran
  stream; the reference ships the local_smart log as the otf golden too): the otf pick
  -- the process from the per-process totals, then the entry from the running sum of the
  chosen list -- gives the golden (process, site) pairs up to the first AB reaction.  As
  for lat_int, otf stores a process at its cell's first site, local_smart at its
  executing coordinate, so the reaction at step 155 lands one cell up.
* Long intZGB runs keep the otf invariants: every list holds exactly the (process, cell)
  pairs whose conditions hold on the lattice, every entry's rate is gr_<process> of the
  current lattice (each bystander change was followed by its rate update), and the
  process totals are the left-to-right sums of the lists.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, fixture_model
from kmos_gb300 import otf as OTF, program as PG
from oracle import oracle as O


def otf_oracle(model, size, rates, params=None, **kw):
    prog = PG.compile_model(model, "otf")
    o = O.Oracle(prog, size, **kw)
    o.set_rates(rates)
    o.set_user_parameters(params if params is not None else OTF.user_parameter_values(model))
    o.recalculate_rates_matrix()
    o.update_accum_rate()
    o.update_integ_rate()
    return prog, o


def test_golden_trajectory_otf_prefix():
    m = fixture_model("AB_model")
    rates = json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    ref = np.load(os.path.join(GOLDEN, "ab_model_ref_procs_sites.npy"))
    _prog, o = otf_oracle(m, (20, 20), rates, seed=1, rng=O.RNG_GFORTRAN)
    out = []
    for _ in range(155):
        p, s = o.get_next_kmc_step()
        out.append((p, s))
        o.run_proc_nr(p, s)
    np.testing.assert_array_equal(np.array(out[:154]), ref[:154])
    assert out[154][0] == ref[154][0] == 1
    assert out[154][1] == ref[154][1] + 20


def fresh_rate(prog, model, o, p, site, lat):
    """gr_<p> at the cell of ``site``, from the lattice, in Python."""
    w = prog.words
    r = int(w[int(w[22]) + p - 1])
    nb, nv = int(w[r]), int(w[r + 1])
    X, Y = o.size[0], o.size[1]
    c = (site - 1) // o.spuck
    bx, by = c % X, c // X
    nr, pos = [0] * nv, r + 4
    for _ in range(nb):
        dx, dy, _dz, n = PG.unpack_coord(int(w[pos]))
        s = o.spuck * (((bx + dx) % X) + X * ((by + dy) % Y)) + n
        npairs = int(w[pos + 1])
        for j in range(npairs):
            if lat[s - 1] == int(w[pos + 2 + 2 * j]):
                nr[int(w[pos + 3 + 2 * j])] += 1
        pos += 2 + 2 * npairs
    return OTF.evaluate(w[pos:], o.rates()[p - 1], o._userpar, nr)


@pytest.mark.parametrize("seed", [3, 4])
def test_intzgb_invariants(seed):
    m = fixture_model("intZGB_otf")
    rates = [0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3]
    params = [1.3, 0.7, 1.9, 1e-10, 0.5]      # J_CO_CO, J_O_CO, J_O_O, kDes, yCO
    prog, o = otf_oracle(m, (12, 10), rates, params, seed=seed, rng=O.RNG_PHILOX, traj=1)
    o._userpar = params
    for block in range(4):
        o.do_kmc_steps(700)
        ex = o.export()
        lat = ex["lattice"]
        rm, tot = o.rates_matrix()
        ns = ex["nsites"]
        # tables: the enabled (process, cell) pairs, from a rebuild of the same lattice
        ref = O.Oracle(prog, (12, 10), seed=1)
        rb = ref.rebuild_tables(lat)
        for p in range(1, o.P + 1):
            mine = set(ex["as1"][p - 1, 1:1 + ns[p - 1]].tolist())
            assert mine == set(rb["as1"][p - 1, 1:1 + rb["nsites"][p - 1]].tolist())
            for i in range(1, ns[p - 1] + 1):
                site = int(ex["as1"][p - 1, i])
                assert rm[p - 1, i] == fresh_rate(prog, m, o, p, site, lat), (block, p, i)
        o.update_accum_rate()
        rm, tot = o.rates_matrix()
        for p in range(o.P):
            s = 0.0
            for i in range(1, ns[p] + 1):
                s = s + rm[p, i]
            assert tot[p] == s
        acc = [float(tot[0])]
        for p in range(1, o.P):
            acc.append(acc[-1] + float(tot[p]))
        assert o.accum_rates().tolist() == acc
    assert o.kmc_step == 2800


def test_otf_and_local_smart_are_the_same_kinetics():
    """Without bystanders every otf entry's rate is its rate constant, so otf and
    local_smart sample the same Markov chain (different book-keeping, different draws
    per event): the AB model's time-averaged coverages from 8 trajectories of each agree
    within 4 standard errors."""
    m = fixture_model("AB_model")
    rates = json.load(open(os.path.join(GOLDEN, "ab_model_rates.json")))["rates"]
    cov = {}
    for backend in ("otf", "local_smart"):
        prog = PG.compile_model(m, backend)
        vals = []
        for t in range(8):
            o = O.Oracle(prog, (12, 12), seed=21, rng=O.RNG_PHILOX, traj=t)
            o.set_rates(rates)
            if backend == "otf":
                o.set_user_parameters(OTF.user_parameter_values(m))
                o.recalculate_rates_matrix()
            o.update_accum_rate()
            o.do_kmc_steps(3000)               # relax
            acc, tsum = 0.0, 0.0
            for _ in range(60):
                t0 = o.kmc_time
                o.do_kmc_steps(100)
                occ = o.occupation(len(m.species))
                acc += occ[:, 0] * (o.kmc_time - t0)
                tsum += o.kmc_time - t0
            vals.append(acc / tsum)
        cov[backend] = np.array(vals)
    a, b = cov["otf"], cov["local_smart"]
    se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b)) + 1e-12
    assert np.all(np.abs(a.mean(0) - b.mean(0)) < 4 * se), (a.mean(0), b.mean(0), se)
