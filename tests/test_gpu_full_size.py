"""The 2048-trajectory lat_int workload (uneven square lattices, side 16..256, T in
[300, 600] K) at its full lattice sizes and full run length, bit for bit against the
oracle.

From the workload's own trajectories, the coldest and the hottest of side 128 and of
side 256 run their 1e6 kMC steps through the pool's batched fast path (one launch for the
four, as the batch runs them).  At checkpoints along the run the lattice, both
avail_sites columns, nr_of_sites and procstat must equal the oracle's exactly, kmc_step
too; kmc_time and integ_rates within 1e-12 relative.  The large cold lattices are where
the lateral-interaction streams are longest and the tables largest
(base_lat_int.mpy:243-311, kmos/io/__init__.py:1793-1983)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from kmos_gb300 import configs, engine as E
from oracle import oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-12
CHECKPOINTS = [1000, 100_000, 500_000, 1_000_000]


def pick(wl):
    """The coldest and the hottest trajectory of side 128 and of side 256."""
    side, T = np.asarray(wl.notes["side"]), np.asarray(wl.notes["T"])
    out = []
    for s in (128, 256):
        idx = np.where(side == s)[0]
        out += [int(idx[np.argmin(T[idx])]), int(idx[np.argmax(T[idx])])]
    return out


def oracle_states(wl, i):
    """The oracle's state of trajectory i at every checkpoint (the C oracle releases the
    GIL, so trajectories run in parallel threads)."""
    o = O.Oracle(wl.program, wl.sizes[i], seed=wl.seeds[i], rng=O.RNG_PHILOX, traj=wl.trajs[i])
    o.set_rates(wl.rates[i])
    o.update_accum_rate()
    states, done = [], 0
    for c in CHECKPOINTS:
        o.do_kmc_steps(c - done)
        done = c
        st = o.export()
        st["kmc_time"], st["kmc_step"] = o.kmc_time, o.kmc_step
        states.append(st)
    return states


def test_full_size_lattices_over_the_full_run():
    wl = configs.build(3)
    picks = pick(wl)
    with ThreadPoolExecutor(len(picks)) as ex:
        want = list(ex.map(lambda i: oracle_states(wl, i), picks))
    probe = E.Pool(arena_bytes=1 << 20, max_slots=1)
    pmid = probe.add_model(wl.program)
    need = sum(probe.slot_bytes(pmid, wl.sizes[i]) for i in picks)
    probe.close()
    pool = E.Pool(arena_bytes=need + (16 << 20), max_slots=len(picks))
    mid = pool.add_model(wl.program)
    slots = [pool.admit(mid, wl.sizes[i], wl.rates[i], seed=wl.seeds[i], rng=E.RNG_PHILOX, traj=wl.trajs[i])
             for i in picks]
    done = 0
    for c, chk in enumerate(CHECKPOINTS):
        pool.run(slots, chk - done)
        done = chk
        for k, slot in enumerate(slots):
            st = want[k][c]
            where = "trajectory %d (side %d, T %.0f K) at step %d" % (
                picks[k], wl.sizes[picks[k]][0], wl.notes["T"][picks[k]], chk)
            assert pool.status(slot) == 0, where
            t, step = pool.clock(slot)
            assert step == st["kmc_step"] == chk, where
            assert abs(t - st["kmc_time"]) <= RTOL * abs(st["kmc_time"]), where
            np.testing.assert_array_equal(pool.lattice(slot), st["lattice"], err_msg=where)
            as1, as2 = pool.tables(slot)
            np.testing.assert_array_equal(as1, st["as1"], err_msg=where)
            np.testing.assert_array_equal(as2, st["as2"], err_msg=where)
            np.testing.assert_array_equal(pool.nr_of_sites(slot), st["nsites"], err_msg=where)
            np.testing.assert_array_equal(pool.procstat(slot), st["procstat"], err_msg=where)
            np.testing.assert_allclose(pool.integ_rates(slot), st["integ"], rtol=RTOL, atol=0, err_msg=where)
    pool.close()
