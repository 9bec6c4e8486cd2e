"""The otf backend's program against the reference's own golden otf exports
(tests/golden/ops/*_otf.json, made by tests/golden/make_otf_golden.py from
tests/export_test/reference_export_intZGB_otf and reference_export_otf): the op order of
every run_proc_<name> (guarded dels, replaces, rate updates, adds with their select-case
conditions), the cell touch-up, and every gr_<name> function -- which bystander species
count towards which nr variable, and the rate expression, compiled from the generated
Fortran's own text, giving the same rate program as the model's otf_rate.  Plus the
expression semantics: Fortran typing and libgcc's integer powering."""
import json
import math
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, fixture_model
from kmos_gb300 import otf as OTF, program as PG

CASES = [("intZGB_otf", "intZGB_otf_otf.json"), ("default_xml", "default_xml_otf.json")]


def norm(op):
    if op[0] == "add":
        return ["add", int(op[1]), list(op[2]), sorted([list(c), int(m)] for c, m in op[3])]
    return [op[0]] + [list(x) if isinstance(x, (tuple, list)) else int(x) for x in op[1:]]


@pytest.mark.parametrize("name,gold", CASES)
def test_otf_op_order_matches_generated_fortran(name, gold):
    g = json.load(open(os.path.join(GOLDEN, "ops", gold)))
    prog = PG.compile_model(fixture_model(name), "otf")
    assert set(int(p) for p in g["procs"]) == set(range(1, prog.nproc + 1))
    for p, ops in g["procs"].items():
        assert [norm(o) for o in prog.proc_stream(int(p))] == [norm(o) for o in ops], "process %s" % p
    assert [norm(o) for o in prog.touchup_stream(0)] == [norm(o) for o in g["touchups"]["1"]]


def records(prog):
    w = prog.words
    off = int(w[22])
    out = {}
    for p in range(1, prog.nproc + 1):
        r = int(w[off + p - 1])
        nb, nv, nc = int(w[r]), int(w[r + 1]), int(w[r + 2])
        pos, byst = r + 4, []
        for _ in range(nb):
            coord, npairs = PG.unpack_coord(int(w[pos])), int(w[pos + 1])
            pairs = [[int(w[pos + 2 + 2 * j]), int(w[pos + 3 + 2 * j])] for j in range(npairs)]
            byst.append([list(coord), pairs])
            pos += 2 + 2 * npairs
        out[p] = (nv, byst, [int(x) for x in w[pos:pos + nc]])
        if p < prog.nproc:
            assert pos + nc <= int(w[off + p])
    return out


@pytest.mark.parametrize("name,gold", CASES)
def test_rate_functions_match_generated_fortran(name, gold):
    g = json.load(open(os.path.join(GOLDEN, "ops", gold)))
    model = fixture_model(name)
    prog = PG.compile_model(model, "otf")
    recs = records(prog)
    for p, ref in g["rates"].items():
        nv, byst, code = recs[int(p)]
        assert byst == ref["bystanders"], "process %s" % p
        proc = model.processes[int(p) - 1]
        names = OTF.nr_var_names(proc)
        assert len(names) == nv
        # the generated Fortran's rate expression, read back into otf_rate syntax
        text = ref["expr"].replace("&", " ")
        text = re.sub(r"rates\s*\(\s*\w+\s*\)", "base_rate", text)
        text = re.sub(r"userpar\s*\(\s*(\w+)\s*\)", r"\1", text)
        text = re.sub(r"nr_vars\s*\(\s*(\d+)\s*\)", lambda m: names[int(m.group(1)) - 1], text)
        from kmos_gb300.model import Process
        twin = Process(proc.name, proc.rate_constant, bystanders=proc.bystanders, otf_rate=text)
        assert OTF.compile_rate(model, twin)[1] == code, "process %s: %s" % (p, text)


def run(expr, base=2.0, par=None, nr=None, model=None):
    from kmos_gb300.model import Bystander, Coord, Parameter, Process
    model = model or fixture_model("intZGB_otf")
    proc = Process("p", "1", bystanders=[Bystander(("O", "CO"), Coord("default", (1, 0, 0), "square"), "f")],
                   otf_rate=expr)
    _names, code, _d = OTF.compile_rate(model, proc)
    par = par if par is not None else [1.5, 0.75, 3.0, 1e-10, 0.5]
    return OTF.evaluate(code, base, par, nr or [2, 3])


def test_expression_semantics():
    # integer arithmetic stays integer (truncating division) until it meets a real
    assert run("7/2") == 3.0 and run("-7/2") == -3.0 and run("7/2.0") == 3.5
    # a real literal is single precision: 0.1 is the float32 value widened
    assert run("0.1") == float(np.float32(0.1)) and run("0.1d0") == 0.1
    assert run("base_rate*0.1") == 2.0 * float(np.float32(0.1))
    # real ** integer by libgcc's binary powering, the reciprocal for negative powers
    x = 1.1
    assert run("J_CO_CO**nr_CO_f", par=[x, 0, 0, 0, 0], nr=[5, 0]) == x * ((x * x) * (x * x))
    assert run("J_CO_CO**(-nr_CO_f)", par=[x, 0, 0, 0, 0], nr=[3, 0]) == 1.0 / (x * (x * x))
    assert run("J_CO_CO**0", par=[x, 0, 0, 0, 0]) == 1.0
    # integer ** integer
    assert run("2**nr_O_f", nr=[0, 10]) == 1024.0
    # Fortran precedence: unary minus below **, ** right-associative
    assert run("-2.0d0**2") == -4.0 and run("2**3**2") == 512.0
    # multi-line expressions with auxiliary (real(8)) variables
    assert run("a = base_rate*3\notf_rate = a/2") == 3.0
    # unit constants are the single-precision literal of their %.10e value
    assert run("kboltzmann") == float(np.float32(float("%.10e" % 1.3806488e-23)))
    assert math.isclose(run("exp(-J_O_CO)"), math.exp(-0.75), rel_tol=0, abs_tol=0)


def test_intzgb_rates_equal_the_formula():
    model = fixture_model("intZGB_otf")
    prog = PG.compile_model(model, "otf")
    recs = records(prog)
    assert OTF.user_parameters(model) == ["J_CO_CO", "J_O_CO", "J_O_O", "kDes", "yCO"]
    assert OTF.user_parameter_values(model) == [1.0, 1.0, 1.0, 1e-10, 0.5]
    par = [1.3, 0.7, 1.9, 1e-10, 0.5]
    rng = np.random.default_rng(0)
    for _ in range(50):
        nco, no = (int(v) for v in rng.integers(0, 5, 2))
        # CO_ads: base * J_O_CO**nr_O_1nn * J_CO_CO**nr_CO_1nn, nr_vars sorted (CO, O)
        got = OTF.evaluate(recs[1][2], 0.25, par, [nco, no])
        want = (0.25 * OTF.powi(0.7, no, OTF.K_F64)) * OTF.powi(1.3, nco, OTF.K_F64)
        assert got == want


def fuzz_otf(seed: int, trials: int):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from kmos_gb300 import engine as E
    progs = [PG.compile_model(fixture_model(n), "otf") for n in ("intZGB_otf", "default_xml", "AB_model")]
    rng = np.random.default_rng(seed)
    accepted = refused = 0
    for trial in range(trials):
        w = np.array(progs[trial % len(progs)].words, dtype=np.int32)
        for _ in range(int(rng.integers(1, 4))):
            i = int(rng.integers(0, len(w)))
            how = int(rng.integers(0, 4))
            if how == 0:
                w[i] = int(rng.integers(-2**31, 2**31, dtype=np.int64))
            elif how == 1:
                w[i] = (int(w[i]) + int(rng.integers(-4, 5)) + 2**31) % 2**32 - 2**31
            elif how == 2:
                w[i] = np.uint32((int(w[i]) & 0xFFFFFFFF) ^ (1 << int(rng.integers(0, 32)))).view(np.int32)
            else:
                w[i] = -int(rng.integers(1, 8))
        try:
            E.check_otf_program(w)
            accepted += 1
        except E.KMCError as e:
            if e.code != 5:
                raise SystemExit("refused with status %d" % e.code)
            refused += 1
    return accepted, refused


@pytest.mark.parametrize("seed", [1, 2])
def test_malformed_otf_programs_never_crash_the_check(seed):
    """kmc_otf_check_program (run by kmc_otf_create) on randomly corrupted otf programs:
    refused with KMC_ERR_PROGRAM or accepted, never a crash (child process)."""
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    code = ("import sys; sys.path[:0] = [%r, %r]; import test_otf_program as T; print(*T.fuzz_otf(%d, 2000))"
            % (here, os.path.dirname(here), seed))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=here)
    assert r.returncode == 0, r.stderr[-2000:]
    accepted, refused = map(int, r.stdout.split()[-2:])
    assert refused > 0 and accepted + refused == 2000


def test_otf_check_refuses_what_the_device_cannot_run():
    """kmc_otf_check_program refuses, with KMC_ERR_PROGRAM: a rate program deeper than
    the device stack, one reading an nr variable or user parameter that does not exist,
    an unknown instruction, a touch-up strip inside a process stream, a local_smart
    program."""
    from kmos_gb300 import engine as E
    from kmos_gb300.model import Bystander, Coord, Process
    m = fixture_model("intZGB_otf")
    E.check_otf_program(PG.compile_model(m, "otf"))

    def refused(words):
        with pytest.raises(E.KMCError) as e:
            E.check_otf_program(words)
        assert e.value.code == 5

    deep = "+".join(["(base_rate*J_O_O"] * 17) + ")" * 17
    m2 = fixture_model("intZGB_otf")
    m2.processes[1].otf_rate = deep
    with pytest.raises(OTF.ExprError):
        PG.compile_model(m2, "otf")              # the compiler refuses it first
    prog = PG.compile_model(m, "otf")
    w = np.array(prog.words, dtype=np.int32)
    r = int(w[int(w[22])])                      # rate record of process 1 (CO_ads)
    nb = int(w[r])
    pos = r + 4
    for _ in range(nb):
        pos += 2 + 2 * int(w[pos + 1])
    code0 = pos                                  # first instruction: PUSH_BASE
    for bad in (OTF.ins(OTF.I_PUSH_NR, 0, 9), OTF.ins(OTF.I_PUSH_PAR, 0, 5), 99):
        v = w.copy()
        v[code0] = bad
        refused(v)
    v = w.copy()
    v[int(w[int(w[10])])] = PG.op_header(PG.OP_STRIP)   # first op of process 1
    refused(v)
    refused(PG.compile_model(m, "local_smart").words)


def test_ini_bystanders_and_otf_rate_read_like_the_xml():
    """The .ini form kmos writes for otf models (kmos/types.py:418-428: ``bystanders =
    ['O', 'CO']@default.(1, 0, 0)|1nn + ...``, ``otf_rate = ...``) reads back into the same
    processes as the .xml; the JSON form keeps bystanders and otf_rate."""
    from kmos_gb300 import model as M
    xml = fixture_model("intZGB_otf")
    lines = ["[Meta]", "model_name = IntZGB", "model_dimension = 2", "",
             "[SpeciesList]", "default_species = empty", ""]
    for sp in xml.species:
        lines += ["[Species %s]" % sp, "representation = ", ""]
    lines += ["[Lattice]", "cell_size = 1.0 1.0 1.0", "default_layer = square", "",
              "[Layer square]", "site default = (0.5, 0.5, 0.5); default_species; ", ""]
    for p in xml.parameters:
        lines += ["[Parameter %s]" % p.name, "value = %s" % p.value, "adjustable = False", "min = 0.0",
                  "max = 0.0", "scale = linear", ""]

    def sh(species, c):
        off = tuple(c.offset)
        return "%s@%s%s" % (species, c.name, ".%s" % (off,) if any(off) else "")

    for p in xml.processes:
        lines += ["[Process %s]" % p.name, "rate_constant = %s" % p.rate_constant,
                  "enabled = True",
                  "conditions = " + " + ".join(sh(c.species, c.coord) for c in p.conditions),
                  "actions = " + " + ".join(sh(a.species, a.coord) for a in p.actions)]
        if p.bystanders:
            lines.append("bystanders = " + " + ".join("%s|%s" % (sh(list(b.allowed_species), b.coord), b.flag)
                                                      for b in p.bystanders))
        lines.append("otf_rate = %s" % p.otf_rate)
        lines.append("")
    ini = M.load_ini("\n".join(lines))
    assert [p.name for p in ini.processes] == [p.name for p in xml.processes]
    for a, b in zip(ini.processes, xml.processes):
        assert a.bystanders == b.bystanders and a.otf_rate == b.otf_rate
        assert a.conditions == b.conditions and a.actions == b.actions
    assert (PG.compile_model(ini, "otf").words == PG.compile_model(xml, "otf").words).all()
    back = M.from_dict(M.to_dict(xml))
    assert [(p.bystanders, p.otf_rate) for p in back.processes] == [(p.bystanders, p.otf_rate) for p in xml.processes]
