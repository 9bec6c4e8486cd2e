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


def _oracle_file(tmp_path, name, backend, size, steps=400):
    prog = PG.compile_model(fixture_model(name), backend)
    o = O.Oracle(prog, size, seed=5, rng=O.RNG_PHILOX, traj=2)
    if backend == "otf":
        from kmos_gb300 import otf as OTF
        o.set_user_parameters(OTF.user_parameter_values(fixture_model(name)))
    o.set_rates(np.linspace(1.0, 20.0, prog.nproc))
    if backend == "otf":
        o.recalculate_rates_matrix()
    o.update_accum_rate()
    o.do_kmc_steps(steps)
    path = str(tmp_path / ("%s_%s.reload" % (name, backend)))
    RL.write_oracle_reload(path, o, walltime=0.25)
    return prog, o, path


def _edit(path, out, fn):
    lines = open(path).read().splitlines()
    with open(out, "w") as f:
        f.write("\n".join(fn(lines)) + "\n")
    return out


@pytest.mark.parametrize("name, backend, size", [("CO_oxidation_Ruo2", "local_smart", (6, 5)),
                                                 ("pdopd_xml", "lat_int", (5, 4)),
                                                 ("intZGB_otf", "otf", (6, 6))])
def test_native_check_of_reload_files(tmp_path, name, backend, size):
    """kmc_check_reload (no device) makes the checks the lattice and otf loaders make
    before anything reaches the GPU: the oracle's file passes; a wrong system size, a
    species out of range, a missing vector, a nr_of_sites or avail_sites entry that
    disagrees with the other column, and a "#gb300 rng" line of an unknown stream, of an
    all-zero gfortran state or that does not read are refused."""
    from kmos_gb300 import engine as E
    prog, o, path = _oracle_file(tmp_path, name, backend, size)
    E.check_reload(prog, size, path)
    nsp = len(fixture_model(name).species)
    bad = str(tmp_path / "bad.reload")

    def refused(fn, code):
        _edit(path, bad, fn)
        with pytest.raises(E.KMCError) as e:
            E.check_reload(prog, size, bad)
        assert e.value.code == code, str(e.value)

    with pytest.raises(E.KMCError) as e:
        E.check_reload(prog, (size[0] + 1, size[1]), path)
    assert e.value.code == 1

    def lattice_species(lines):
        return [" ".join(["lattice", str(nsp + 1)] + l.split()[2:]) if l.split()[:1] == ["lattice"] else l
                for l in lines]
    refused(lattice_species, 1)
    refused(lambda lines: [l for l in lines if l.split()[:1] != ["lattice"]], 1)

    ex = o.export()
    q = int(np.argmax(ex["nsites"]))       # a process with entries
    assert ex["nsites"][q] >= 2

    def more_sites(lines):
        out = []
        for l in lines:
            t = l.split()
            if t[:1] == ["nr_of_sites"]:
                t[1 + q] = str(int(t[1 + q]) + 1)
                l = " ".join(t)
            out.append(l)
        return out
    refused(more_sites, 4)

    def swap_entries(lines):
        out = []
        for l in lines:
            t = l.split()
            if t[:2] == ["avail_sites", str(q + 1)]:
                t[2], t[3] = t[3], t[2]
                l = " ".join(t)
            out.append(l)
        return out
    refused(swap_entries, 4)

    for line in ("#gb300 rng 7 1 2 3 4 5 6", "#gb300 rng 0 1 2 0 0 0 0", "#gb300 rng 1 1 2 x 4 5 6",
                 "#gb300 rng 1 1 -2 3 4 5 6", "#gb300 rng 1 1 2 3 4 5"):
        refused(lambda lines, line=line: lines + [line], 1)
    _edit(path, bad, lambda lines: lines + ["#gb300 rng 1 3 1 5 0 0 0"])
    E.check_reload(prog, size, bad)
    with pytest.raises(E.KMCError) as e:
        E.check_reload(np.array([7, 1, 0, 1, 1, 1, 1], np.int32), size, path)
    assert e.value.code == 5


def test_native_reload_check_survives_random_corruption(tmp_path):
    """Random edits of a valid file (lines dropped or duplicated, tokens replaced by
    random integers or text, the file cut at a random byte) never crash the native reader;
    each is accepted or refused with KMC_ERR_ARG / KMC_ERR_TABLE."""
    from kmos_gb300 import engine as E
    prog, o, path = _oracle_file(tmp_path, "CO_oxidation_Ruo2", "local_smart", (6, 5))
    text = open(path).read()
    lines = text.splitlines()
    rng = np.random.default_rng(17)
    bad = str(tmp_path / "fuzz.reload")
    codes = {}
    for trial in range(300):
        kind = trial % 4
        cur = list(lines)
        if kind == 0:
            del cur[int(rng.integers(len(cur)))]
            body = "\n".join(cur) + "\n"
        elif kind == 1:
            i = int(rng.integers(len(cur)))
            cur.insert(i, cur[i])
            body = "\n".join(cur) + "\n"
        elif kind == 2:
            i = int(rng.integers(len(cur)))
            t = cur[i].split()
            if len(t) > 1:
                j = int(rng.integers(1, len(t)))
                t[j] = str(rng.choice(["-1", "0", "1", "2", "-7", "x", "1e3", "99999999999", str(o.V), str(o.V + 1)]))
                cur[i] = " ".join(t)
            body = "\n".join(cur) + "\n"
        else:
            body = text[:int(rng.integers(len(text)))]
        with open(bad, "w") as f:
            f.write(body)
        try:
            E.check_reload(prog, (6, 5), bad)
            code = 0
        except E.KMCError as e:
            code = e.code
        codes[code] = codes.get(code, 0) + 1
    assert set(codes) <= {0, 1, 4}, codes
    assert codes.get(1, 0) + codes.get(4, 0) > 150, codes
