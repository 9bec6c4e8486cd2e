"""Saving and restoring trajectories on the GPU.

* Binary state images (kmc_pool_save_state / kmc_pool_restore_state): a trajectory
  saved, released and restored into another slot continues bit for bit like one that
  never left the device; images are validated before they reach the device.
* .reload files (base.save_system / reload_system, base.mpy:363-578): the engine's file
  equals the oracle's writer (oracle/reload.py) on the same state, line for line; a
  file with the engine's "#gb300" lines resumes the trajectory exactly; a file in the
  reference's bare layout loads its lattice, tables and counters.
"""
import os

import numpy as np
import pytest

from conftest import fixture_model
from kmos_gb300 import engine as E, kmc_model, program as PG
from oracle import oracle as O, reload as RL

pytestmark = pytest.mark.gpu

MODELS = [("pairwise_interaction", "lat_int", (16, 16)), ("CO_oxidation_Ruo2", "local_smart", (10, 10)),
          ("ZGB_model", "lat_int", (12, 16)), ("default_xml", "local_smart", (10, 10))]


def rates_for(P, seed):
    return (10.0 ** np.random.default_rng(seed).uniform(-1, 3, size=P)).tolist()


def _pool_with(programs, n_each, arena=1 << 28):
    pool = E.Pool(arena_bytes=arena, max_slots=256)
    mids = [pool.add_model(p) for p in programs]
    slots = []
    for k, (p, mid) in enumerate(zip(programs, mids)):
        for j in range(n_each):
            slots.append(pool.admit(mid, MODELS[k][2], rates_for(p.nproc, 10 * k + j), seed=5 + k,
                                    rng=E.RNG_PHILOX, traj=j))
    return pool, mids, slots


def _state(pool, s):
    P = pool.nproc(pool.slot_model[s])
    ps, ig, t, k, st = pool.results([s], P)
    as1, as2 = pool.tables(s)
    return ps[0], ig[0], t[0], k[0], st[0], pool.lattice(s), as1, as2


def test_pool_restore_continues_bit_exact():
    progs = [PG.compile_model(fixture_model(n), b) for n, b, _ in MODELS]
    a, mids_a, slots_a = _pool_with(progs, 3)
    b, mids_b, slots_b = _pool_with(progs, 3)
    a.run(slots_a, 1500)
    b.run(slots_b, 1500)
    images = [(a.slot_model[s], a.save_state(s)) for s in slots_a]
    for s in slots_a:
        a.release(s)
    filler = a.admit(mids_a[0], (8, 8), rates_for(progs[0].nproc, 99), seed=1)  # restored slots move
    restored = [a.restore_state(m, img) for m, img in images]
    assert sorted(restored) != sorted(slots_a)
    a.run(restored, 2500)
    b.run(slots_b, 2500)
    for r, s in zip(restored, slots_b):
        for x, y in zip(_state(a, r), _state(b, s)):
            np.testing.assert_array_equal(x, y)
    a.release(filler)
    a.close()
    b.close()


def test_image_is_compact_and_validated():
    prog = PG.compile_model(fixture_model("pairwise_interaction"), "lat_int")
    pool = E.Pool(arena_bytes=1 << 27, max_slots=8)
    mid = pool.add_model(prog)
    s = pool.admit(mid, (64, 64), rates_for(prog.nproc, 1), seed=2)
    pool.run([s], 4000)
    img = pool.save_state(s)
    assert len(img) * 10 < pool.slot_bytes(mid, (64, 64))
    V = 64 * 64
    bad = bytearray(img)
    bad[-4:] = int(V + 7).to_bytes(4, "little", signed=True)  # last avail_sites entry off the lattice
    with pytest.raises(E.KMCError) as e:
        pool.restore_state(mid, bytes(bad))
    assert e.value.code == 4
    with pytest.raises(E.KMCError) as e:
        pool.restore_state(mid, img[:-8])
    assert e.value.code == 1
    other = pool.add_model(PG.compile_model(fixture_model("ZGB_model"), "lat_int"))
    with pytest.raises(E.KMCError) as e:
        pool.restore_state(other, img)
    assert e.value.code == 1
    s2 = pool.restore_state(mid, img)  # the untouched image still loads
    for x, y in zip(_state(pool, s), _state(pool, s2)):
        np.testing.assert_array_equal(x, y)
    pool.close()


@pytest.mark.parametrize("name,backend,size", MODELS)
def test_handle_state_round_trip(name, backend, size):
    prog = PG.compile_model(fixture_model(name), backend)
    with E.Trajectory(prog, size, seed=9, rng=E.RNG_GFORTRAN) as g:
        g.set_rates(rates_for(prog.nproc, 3))
        g.update_accum_rate()
        g.do_kmc_steps(2000)
        img = g.save_state()
        t1 = g.trace(3000)
        end1 = (g.kmc_time, g.procstat(), g.integ_rates())
        g.load_state(img)
        t2 = g.trace(3000)
        np.testing.assert_array_equal(t1, t2)
        assert g.kmc_time == end1[0]
        np.testing.assert_array_equal(g.procstat(), end1[1])
        np.testing.assert_array_equal(g.integ_rates(), end1[2])


def _lines(path):
    with open(path) as f:
        return [ln.rstrip("\n") for ln in f if not ln.startswith("#gb300")]


@pytest.mark.parametrize("name,backend,size", MODELS)
def test_reload_file_matches_oracle_writer(name, backend, size, tmp_path):
    prog = PG.compile_model(fixture_model(name), backend)
    rates = rates_for(prog.nproc, 4)
    with E.Trajectory(prog, size, seed=13, rng=E.RNG_GFORTRAN) as g:
        o = O.Oracle(prog, size, seed=13, rng=O.RNG_GFORTRAN)
        for x in (g, o):
            x.set_rates(rates)
            x.update_accum_rate()
            x.do_kmc_steps(2500)
        pg, po = str(tmp_path / "gpu.reload"), str(tmp_path / "oracle.reload")
        g.save_reload(pg)
        RL.write_oracle_reload(po, o, walltime=g.walltime)
        lg, lo = _lines(pg), _lines(po)
        assert len(lg) == len(lo)
        for a, b in zip(lg, lo):
            if a.startswith(" kmc_time") or a.startswith(" walltime"):
                continue
            assert a == b
        tg, to = float(lg[2].split()[1]), float(lo[2].split()[1])
        assert abs(tg - to) <= 1e-12 * abs(to)


@pytest.mark.parametrize("name,backend,size", MODELS[:2])
def test_reload_resumes_exactly(name, backend, size, tmp_path):
    prog = PG.compile_model(fixture_model(name), backend)
    path = str(tmp_path / "run.reload")
    with E.Trajectory(prog, size, seed=21, rng=E.RNG_PHILOX, traj=3) as g:
        g.set_rates(rates_for(prog.nproc, 5))
        g.update_accum_rate()
        g.do_kmc_steps(1800)
        g.save_reload(path)
        P, V, dims = E.reload_info(path)
        assert (P, V, dims) == (prog.nproc, g.V, list(g.size))
        with E.Trajectory(prog, dims, seed=77, rng=E.RNG_GFORTRAN) as h:
            h.load_reload(path)
            np.testing.assert_array_equal(h.trace(2000), g.trace(2000))
            assert h.kmc_time == g.kmc_time and h.kmc_step == g.kmc_step
            np.testing.assert_array_equal(h.integ_rates(), g.integ_rates())
            np.testing.assert_array_equal(h.lattice(), g.lattice())


def test_reload_reference_layout(tmp_path):
    """A file in the reference's bare layout (no "#gb300" lines) restores lattice,
    tables, counters and rates (to the 8 digits ES14.7 keeps); integ_rates restart at
    zero as the reference's reload leaves them."""
    name, backend, size = MODELS[1]
    prog = PG.compile_model(fixture_model(name), backend)
    o = O.Oracle(prog, size, seed=2, rng=O.RNG_PHILOX, traj=0)
    o.set_rates(rates_for(prog.nproc, 6))
    o.update_accum_rate()
    o.do_kmc_steps(3000)
    path = str(tmp_path / "ref.reload")
    RL.write_oracle_reload(path, o)
    assert E.reload_info(path)[2] is None
    ex = o.export()
    with E.Trajectory(prog, size, seed=1) as g:
        g.load_reload(path)
        np.testing.assert_array_equal(g.lattice(), ex["lattice"])
        as1, as2 = g.tables()
        np.testing.assert_array_equal(as1, ex["as1"])
        np.testing.assert_array_equal(as2, ex["as2"])
        np.testing.assert_array_equal(g.nr_of_sites(), ex["nsites"])
        np.testing.assert_array_equal(g.procstat(), ex["procstat"])
        assert g.kmc_step == o.kmc_step
        np.testing.assert_allclose(g.rates(), o.rates(), rtol=1e-7)
        assert not g.integ_rates().any()
        g.do_kmc_steps(500)  # the restored tables step on
    # a file whose two avail_sites columns disagree is refused
    lines = open(path).read().split("\n")
    k = next(i for i, ln in enumerate(lines) if ln.startswith("avail_sites_back"))
    toks = lines[k].split()
    j = next(i for i in range(2, len(toks)) if toks[i] != "0")
    toks[j] = str(int(toks[j]) + 1)
    lines[k] = " ".join(toks)
    bad = str(tmp_path / "bad.reload")
    open(bad, "w").write("\n".join(lines))
    with E.Trajectory(prog, size, seed=1) as g:
        with pytest.raises(E.KMCError) as e:
            g.load_reload(bad)
        assert e.value.code == 4


def test_dropin_save_and_reload_system(tmp_path):
    """base.save_system / base.reload_system through the f2py-compatible module."""
    m = fixture_model("ZGB_model")
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        base, lattice, proclist = kmc_model.configure(m, "local_smart")
        proclist.init([12, 12], "zgb_run", lattice.default_layer, 3, True)
        for p in range(1, proclist.nr_of_proc + 1):
            base.set_rate_const(p, 1.0 + p)
        base.update_accum_rate()
        proclist.do_kmc_steps(1500)
        lat = [base.get_species(i) for i in range(1, 145)]
        t, k = base.get_kmc_time(), base.get_kmc_step()
        base.save_system()
        assert os.path.exists("zgb_run.reload")
        nxt = [proclist.get_next_kmc_step() for _ in range(1)]
        lattice.deallocate_system()
        assert base.reload_system("nothing_here") is False
        assert base.reload_system("zgb_run") is True
        assert [base.get_species(i) for i in range(1, 145)] == lat
        assert base.get_kmc_time() == t and base.get_kmc_step() == k
        assert [proclist.get_next_kmc_step()] == nxt
        lattice.deallocate_system()
    finally:
        os.chdir(cwd)


@pytest.mark.parametrize("name,backend,size", [MODELS[0], MODELS[1]])
def test_oracle_written_image_continues_like_the_oracle(name, backend, size):
    """An image written from an oracle trajectory by a writer that shares no code with the
    engine (oracle/image.py) restores into a pool and steps on exactly as the oracle
    does."""
    from oracle import image as IM
    prog = PG.compile_model(fixture_model(name), backend)
    o = O.Oracle(prog, size, seed=7, rng=O.RNG_PHILOX, traj=3)
    o.set_rates(rates_for(prog.nproc, 8))
    o.update_accum_rate()
    o.do_kmc_steps(2000)
    img = IM.write_image(prog, o, size, seed=7, traj=3)
    pool = E.Pool(arena_bytes=1 << 27, max_slots=4)
    mid = pool.add_model(prog)
    s = pool.restore_state(mid, img)
    pool.run([s], 3000)
    o.do_kmc_steps(3000)
    ex = o.export()
    np.testing.assert_array_equal(pool.lattice(s), ex["lattice"])
    as1, as2 = pool.tables(s)
    np.testing.assert_array_equal(as1, ex["as1"])
    np.testing.assert_array_equal(as2, ex["as2"])
    ps, ig, t, k, st = pool.results([s], prog.nproc)
    np.testing.assert_array_equal(ps[0][:prog.nproc], ex["procstat"])
    assert k[0] == o.kmc_step and st[0] == 0
    assert abs(t[0] - o.kmc_time) <= 1e-12 * abs(o.kmc_time)
    pool.close()
