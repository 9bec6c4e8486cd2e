"""The oracle's .reload writer and reader (oracle/reload.py) on the CPU: Fortran edit
descriptors of base.mpy:528-575 on known values, and a write / read round trip of an
oracle trajectory's state."""
import numpy as np
import pytest

from conftest import fixture_model
from kmos_gb300 import program as PG
from oracle import oracle as O, reload as RL


def test_edit_descriptors():
    assert RL.es(1.0, 22, 15) == " 1.000000000000000E+00"
    assert RL.es(0.0, 22, 15) == " 0.000000000000000E+00"
    assert RL.es(-2.5e-7, 22, 15) == "-2.500000000000000E-07"
    assert RL.es(1e13, 14, 7) == " 1.0000000E+13"
    assert RL.es(123456789.0, 14, 7) == " 1.2345679E+08"
    assert RL.es(1.5e-120, 14, 7) == " 1.5000000-120"
    assert RL.es(3.0e200, 14, 7) == " 3.0000000+200"
    assert RL.es(0.0, 13, 7) == "0.0000000E+00"
    assert RL.es(-1.0, 13, 7) == "*************"
    assert RL.iw(-1, 9) == "       -1"
    assert RL.iw(12345, 22) == " " * 17 + "12345"
    assert RL.iw(10 ** 9, 9) == "*" * 9
    assert RL._real("1.5000000-120") == 1.5e-120
    assert RL._real("2.0D+03") == 2000.0


def test_round_trip(tmp_path):
    prog = PG.compile_model(fixture_model("CO_oxidation_Ruo2"), "local_smart")
    o = O.Oracle(prog, (6, 5), seed=3, rng=O.RNG_PHILOX, traj=1)
    o.set_rates(np.linspace(1.0, 50.0, prog.nproc))
    o.update_accum_rate()
    o.do_kmc_steps(3000)
    path = str(tmp_path / "t.reload")
    RL.write_oracle_reload(path, o, walltime=1.25)
    r = RL.read_reload(path)
    ex = o.export()
    assert r["nr_of_proc"] == prog.nproc and r["volume"] == o.V and r["kmc_step"] == o.kmc_step
    assert abs(r["kmc_time"] - o.kmc_time) <= 1e-15 * o.kmc_time and r["walltime"] == 1.25
    np.testing.assert_array_equal(r["lattice"], ex["lattice"])
    np.testing.assert_array_equal(r["procstat"], ex["procstat"])
    np.testing.assert_array_equal(r["nr_of_sites"], ex["nsites"])
    np.testing.assert_allclose(r["rates"], o.rates(), rtol=1e-7)
    for p in range(prog.nproc):
        np.testing.assert_array_equal(r["as1"][p + 1], ex["as1"][p][1:])
        np.testing.assert_array_equal(r["as2"][p + 1], ex["as2"][p][1:])


def test_native_reader_takes_the_oracle_writers_file(tmp_path):
    """The library's .reload reader (kmos_gb300/csrc/kmc_reload.h, shared by the lattice
    and otf backends; kmc_reload_info needs no device) parses the oracle's independently
    written file: nr_of_proc and volume, no system-size line (the reference's own files
    have none), and the #gb300 system_size line when one is added; a file without the
    counts, or with an unreadable count, is refused."""
    from kmos_gb300 import engine as E
    prog = PG.compile_model(fixture_model("CO_oxidation_Ruo2"), "local_smart")
    o = O.Oracle(prog, (6, 5), seed=3, rng=O.RNG_PHILOX, traj=1)
    o.set_rates(np.linspace(1.0, 50.0, prog.nproc))
    o.update_accum_rate()
    o.do_kmc_steps(500)
    path = str(tmp_path / "t.reload")
    RL.write_oracle_reload(path, o, walltime=0.5)
    assert E.reload_info(path) == (prog.nproc, o.V, None)
    text = open(path).read()
    with open(path, "w") as f:
        f.write("#gb300 system_size 6 5 1\n" + text)
    assert E.reload_info(path) == (prog.nproc, o.V, [6, 5, 1])
    bad = str(tmp_path / "bad.reload")
    with open(bad, "w") as f:
        f.write("\n".join(l for l in text.splitlines() if not l.strip().startswith("nr_of_proc")) + "\n")
    with pytest.raises(E.KMCError):
        E.reload_info(bad)
    with open(bad, "w") as f:
        f.write(text.replace("nr_of_proc", "nr_of_proc x", 1))
    with pytest.raises(E.KMCError):
        E.reload_info(bad)
    with pytest.raises(E.KMCError):
        E.reload_info(str(tmp_path / "missing.reload"))
