"""Generates the golden fixtures under tests/golden/ from the reference checkout.

Run with KMOS_REFERENCE set to a checkout of mhoffman/kmos;
the committed outputs are what the tests read, so the tests never need the reference.

Outputs
  models/<name>.json          reference test models, read by the reference's own
                              Project importers (kmos/types.py) and stored in this
                              package's JSON model form.
  ab_model_rates.json         rate constants of tests/test_run/AB_model.ini as kmos's
                              evaluate_rate_expression computes them.
  ab_model_ref_procs_sites.npy  the 10000 (proc, site) pairs of the reference's golden
                              trajectory tests/test_run/_tmp_export_local_smart/
                              ref_procs_sites_local_smart.log (identical for lat_int and otf).
  ops/<model>_<backend>.json  the op order of the Fortran the reference's generator writes
                              for each fixture model (fortran_ops.py reads it): per process
                              the inlined op list, the touch-ups, and every nli function's
                              value on every species assignment of its coordinates.  The
                              .ini models are exported here with the reference generator;
                              for default.xml and pdopd.xml (the reference's XML reader needs
                              lxml, absent here) the generated code the reference ships as
                              its own golden export (tests/export_test/reference_*) is used.
"""
import ast
import json
import re
import os
import sys
import types
from unittest import mock

import numpy as np

REF = os.environ.get("KMOS_REFERENCE")
if not REF:
    raise SystemExit("set KMOS_REFERENCE to a checkout of mhoffman/kmos")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

MODELS = {
    "AB_model": "tests/test_run/AB_model.ini",
    "ZGB_model": "tests/ini_test/ZGB_model.ini",
    "CO_oxidation_Ruo2": "tests/ini_test/CO_oxidation_Ruo2.ini",
    "pairwise_interaction": "tests/ini_test/pairwise_interaction.ini",
    "default_xml": "tests/export_test/default.xml",
    "pdopd_xml": "tests/export_test/pdopd.xml",
}

# IUPAC masses as carried by ASE for the elements these models use
MASSES = {"H": 1.008, "C": 12.011, "N": 14.007, "O": 15.999, "Pd": 106.42}


def import_reference():
    """Imports the reference's kmos package with its optional heavy dependencies
    (ase, janaf tables) replaced by small stand-ins."""
    jd = types.ModuleType("janaf_data")
    jd.__path__ = ["/nonexistent_janaf"]
    sys.modules["janaf_data"] = jd
    ase = mock.MagicMock()
    symbols = types.ModuleType("ase.symbols")
    import re

    def string2symbols(s):
        out = []
        for sym, cnt in re.findall(r"([A-Z][a-z]?)(\d*)", s):
            out += [sym] * (int(cnt) if cnt else 1)
        return out

    symbols.string2symbols = string2symbols
    data = types.ModuleType("ase.data")
    names = sorted(MASSES)
    data.atomic_numbers = {s: i for i, s in enumerate(names)}
    data.atomic_masses = [MASSES[s] for s in names]
    sys.modules.update({"ase": ase, "ase.symbols": symbols, "ase.data": data, "ase.atoms": ase.atoms})
    sys.path.insert(0, REF)
    import kmos
    import kmos.types
    return kmos


def export_reference(kmos, path, backend, out_dir):
    import kmos.io
    pt = kmos.types.Project()
    pt.import_file(path)
    os.makedirs(out_dir, exist_ok=True)
    try:
        kmos.io.export_source(pt, out_dir, code_generator=backend)
    except Exception as e:  # write_settings evaluates rates it cannot; the sources are written
        print("  export:", repr(e)[:80])


SHIPPED = {("default_xml", "local_smart"): "tests/export_test/reference_export",
           ("default_xml", "lat_int"): "tests/export_test/reference_export_lat_int",
           ("pdopd_xml", "local_smart"): "tests/export_test/reference_pdopd_local_smart",
           ("pdopd_xml", "lat_int"): "tests/export_test/reference_pdopd_lat_int"}


def _jsonable(ops):
    out = []
    for op in ops:
        if op[0] == "add":
            out.append(["add", op[1], list(op[2]), sorted([list(c), m] for c, m in op[3])])
        else:
            out.append([op[0]] + [list(x) if isinstance(x, tuple) else x for x in op[1:]])
    return out


def write_op_goldens(kmos):
    import itertools
    import tempfile
    sys.path.insert(0, HERE)
    import fortran_ops as F

    os.makedirs(os.path.join(HERE, "ops"), exist_ok=True)
    rng = np.random.default_rng(0)
    for name, rel in MODELS.items():
        for backend in ("local_smart", "lat_int"):
            if (name, backend) in SHIPPED:
                d = os.path.join(REF, SHIPPED[(name, backend)])
            elif rel.endswith(".ini"):
                d = tempfile.mkdtemp(prefix="kmos_export_")
                export_reference(kmos, os.path.join(REF, rel), backend, d)
            else:
                continue
            out = {"backend": backend}
            if backend == "local_smart":
                procs, touch, const = F.local_smart_ops(d)
                out["touchups"] = {str(n): _jsonable(ops) for n, ops in touch.items()}
            else:
                procs, nlis, groups, const = F.lat_int_ops(d)
                out["groups"] = groups
                tables = {}
                species = sorted(v for k, v in const.items() if False)
                for g, tree in nlis.items():
                    coords = F.tree_coords(tree)
                    ids = sorted({v for v in _species_ids(d, F)})
                    combos = list(itertools.product(ids, repeat=len(coords)))
                    if len(combos) > 20000:
                        combos = [tuple(int(x) for x in rng.choice(ids, size=len(coords))) for _ in range(20000)]
                    vals = [F.eval_nli(tree, lambda c, a=dict(zip(coords, cb)): a[c]) for cb in combos]
                    tables[str(g)] = {"coords": [list(c) for c in coords], "combos": [list(c) for c in combos],
                                      "values": vals}
                out["nli"] = tables
            out["procs"] = {str(p): _jsonable(ops) for p, ops in procs.items()}
            with open(os.path.join(HERE, "ops", "%s_%s.json" % (name, backend)), "w") as fh:
                json.dump(out, fh, separators=(",", ":"))
            print("ops", name, backend, len(procs), "processes")


def _species_ids(directory, F):
    import glob
    for f in glob.glob(os.path.join(directory, "proclist*.f90")):
        text = open(f).read()
        m = re.search(r"nr_of_species\s*=\s*(\d+)", text)
        if m:
            return range(int(m.group(1)))
    raise ValueError("no species count in %s" % directory)


def main():
    kmos = import_reference()
    write_op_goldens(kmos)
    from kmos_gb300 import model as M

    os.makedirs(os.path.join(HERE, "models"), exist_ok=True)
    for name, rel in MODELS.items():
        path = os.path.join(REF, rel)
        if rel.endswith(".ini"):
            # the reference's own importer, cross-checked against this package's reader
            pt = kmos.types.Project()
            pt.import_file(path)
            m = M.from_project(pt)
            mine = M.load(path)
            assert M.to_dict(mine)["processes"] == M.to_dict(m)["processes"], name
        else:
            # the reference's XML importer needs lxml, which is absent: use this
            # package's reader of the same layout (kmos/types.py:915-1159)
            m = M.load(path)
        M.save_json(m, os.path.join(HERE, "models", name + ".json"))
        print("model", name, len(m.processes), "processes")

    # AB model rates, evaluated by the reference's own evaluate_rate_expression
    pt = kmos.types.Project()
    pt.import_file(os.path.join(REF, MODELS["AB_model"]))
    params = {p.name: {"value": p.value} for p in pt.parameter_list}
    rates = [kmos.evaluate_rate_expression(p.rate_constant, params) for p in pt.process_list]
    with open(os.path.join(HERE, "ab_model_rates.json"), "w") as fh:
        json.dump({"rates": rates, "processes": [p.name for p in pt.process_list]}, fh, indent=1)

    log = os.path.join(REF, "tests/test_run/_tmp_export_local_smart/ref_procs_sites_local_smart.log")
    pairs = np.array(ast.literal_eval(open(log).read()), dtype=np.int32)
    np.save(os.path.join(HERE, "ab_model_ref_procs_sites.npy"), pairs)
    print("golden log", pairs.shape)


if __name__ == "__main__":
    main()
