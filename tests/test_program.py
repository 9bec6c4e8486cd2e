"""The op-program compiler: numbering rules, op order and structural invariants."""
import numpy as np
import pytest

from conftest import fixture_model
from kmos_gb300 import model as M, program as PG

MODELS = ["AB_model", "ZGB_model", "CO_oxidation_Ruo2", "pairwise_interaction", "default_xml", "pdopd_xml"]


@pytest.mark.parametrize("name", MODELS)
@pytest.mark.parametrize("backend", ["local_smart", "lat_int"])
def test_compiles_and_decodes(name, backend):
    m = fixture_model(name)
    prog = PG.compile_model(m, backend)
    w = prog.words
    assert w[0] == PG.MAGIC and w[15] == len(w)
    for p in range(1, prog.nproc + 1):
        ops = prog.proc_stream(p)
        assert ops, (name, p)
        kinds = {op[0] for op in ops}
        assert kinds <= {"replace", "gdel", "add", "li_del", "li_add"}


def test_numbering_rules():
    m = fixture_model("AB_model")
    assert m.species_ids() == {"A": 0, "B": 1, "empty": 2}  # sorted names
    assert list(m.process_ids())[:2] == ["AB_react_down", "AB_react_left"]  # file order
    assert m.null_species() == -1


def test_executing_coordinate_uses_string_sort_key():
    """AB_react_down acts on a.(0,0,0) and a.(0,-1,0); as *strings*
    'default_a_0_-1_0' < 'default_a_0_0_0', so the process runs from the lower site."""
    m = fixture_model("AB_model")
    p = m.processes[0]
    assert p.executing_coord().offset == (0, -1, 0)


def test_ab_put_routine_op_order():
    """put_A_default_a of the generated AB proclist.f90 (kmos/io/__init__.py:2219-2409):
    replace, guarded dels of A_adsorption and B_adsorption, then add A_desorption and
    the four AB_react adds in if-tree order."""
    m = fixture_model("AB_model")
    prog = PG.compile_model(m, "local_smart")
    ops = prog.proc_stream(5)  # A_adsorption -> put_A_default_a(lsite)
    assert ops[0][0] == "replace"
    assert [o[:2] for o in ops[1:3]] == [("gdel", 5), ("gdel", 7)]
    adds = [(o[1], o[2][:3]) for o in ops[3:]]
    assert adds == [(6, (0, 0, 0)), (1, (0, -1, 0)), (2, (-1, 0, 0)), (3, (0, 0, 0)), (4, (0, 0, 0))]


def test_lat_int_groups_of_pairwise_model():
    m = fixture_model("pairwise_interaction")
    groups = PG.ProgramBuilder(m, "lat_int").lat_int_groups()
    sizes = [len(mem) for _g, mem in groups]
    assert sum(sizes) == len(m.processes)
    assert max(sizes) == 16  # the desorption processes differ only in bystanders


def test_iftree_most_common_tie_break():
    items = [((((0, 1, 0, 1), "A"), ((1, 0, 0, 1), "B")), PG.AddItem((), 1, (0, 0, 0, 1))),
             ((((1, 0, 0, 1), "B"),), PG.AddItem((), 2, (0, 0, 0, 1)))]
    items = [(c, PG.AddItem(c, leaf.proc, leaf.target)) for c, leaf in items]
    order = [leaf.proc for leaf in PG.flatten_iftree(items)]
    assert order == [2, 1]  # (1,0,0,1) is asked twice and goes to the top of the tree


def test_json_round_trip():
    for name in MODELS:
        m = fixture_model(name)
        assert M.to_dict(M.from_dict(M.to_dict(m))) == M.to_dict(m)
