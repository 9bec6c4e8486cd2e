"""The op program against the op order of the Fortran the reference's code generator
writes (tests/golden/ops/*.json, made by tests/golden/make_golden.py from that
generator's output for every fixture model and both backends).

local_smart: per process, the inlined put/take/create/annihilate routines of
run_proc_nr -- replaces, guarded dels and adds (each add with the conditions of the
select-case path leading to it) -- and every touch-up.  lat_int: per process, the del
list, the lattice writes and the add list of its run_proc_<group>, and every nli function
evaluated on every species assignment of its coordinates."""
import glob
import json
import os

import pytest

from conftest import GOLDEN, fixture_model
from kmos_gb300 import program as PG

FILES = sorted(glob.glob(os.path.join(GOLDEN, "ops", "*.json")))


def norm(op):
    kind = op[0]
    if kind == "add":
        return ["add", op[1], list(op[2]), sorted([list(c), int(m)] for c, m in op[3])]
    return [kind] + [list(x) if isinstance(x, (tuple, list)) else int(x) for x in op[1:]]


def load(path):
    name = os.path.basename(path)[:-5]
    model, backend = name.rsplit("_", 1) if not name.endswith("local_smart") else (name[:-12], "local_smart")
    if name.endswith("lat_int"):
        model, backend = name[:-8], "lat_int"
    return model, backend, json.load(open(path))


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-5] for f in FILES])
def test_process_op_order_matches_generated_fortran(path):
    model, backend, gold = load(path)
    prog = PG.compile_model(fixture_model(model), backend)
    assert set(int(p) for p in gold["procs"]) == set(range(1, prog.nproc + 1))
    for p, ops in gold["procs"].items():
        mine = [norm(op) for op in prog.proc_stream(int(p))]
        want = [norm(op) for op in ops]
        assert mine == want, "process %s of %s/%s" % (p, model, backend)


@pytest.mark.parametrize("path", [f for f in FILES if f.endswith("local_smart.json")],
                         ids=[os.path.basename(f)[:-5] for f in FILES if f.endswith("local_smart.json")])
def test_touchup_order_matches_generated_fortran(path):
    model, backend, gold = load(path)
    prog = PG.compile_model(fixture_model(model), backend)
    for n, ops in gold["touchups"].items():
        mine = []
        for op in prog.touchup_stream(int(n) - 1):
            if op[0] == "strip":  # touchup_<site> first dels every process that is there
                mine += [["gdel", p, list(op[1])] for p in range(1, prog.nproc + 1)]
            else:
                mine.append(norm(op))
        assert mine == [norm(op) for op in ops], "touch-up of site %s" % n


@pytest.mark.parametrize("path", [f for f in FILES if f.endswith("lat_int.json")],
                         ids=[os.path.basename(f)[:-5] for f in FILES if f.endswith("lat_int.json")])
def test_nli_functions_match_generated_fortran(path):
    model, backend, gold = load(path)
    prog = PG.compile_model(fixture_model(model), backend)
    w = prog.words
    off_groups = int(w[12])
    assert int(w[8]) == len(gold["groups"])
    for g, tab in gold["nli"].items():
        rec = int(w[off_groups + int(g)])
        M, K = int(w[rec]), int(w[rec + 1])
        coords = [tuple(PG.unpack_coord(int(c))) for c in w[rec + 2:rec + 2 + K]]
        gcoords = [tuple(c) for c in tab["coords"]]
        assert set(coords) <= set(gcoords) or not gcoords
        members = [(int(w[rec + 2 + K + m * (1 + K)]), [int(x) & 0xFFFFFFFF for x in
                    w[rec + 3 + K + m * (1 + K):rec + 3 + K + m * (1 + K) + K]]) for m in range(M)]
        for combo, want in zip(tab["combos"], tab["values"]):
            at = dict(zip(gcoords, combo))
            got = 0
            for proc, masks in members:
                if all((mk >> (31 if at[c] < 0 else at[c])) & 1 for c, mk in zip(coords, masks)):
                    got = proc
            assert got == want, (g, combo)
