"""Generates the golden fixtures under tests/golden/ from the reference checkout.

Run in a container that has mhoffman/kmos at KMOS_REFERENCE (default /root/reference);
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
"""
import ast
import json
import os
import sys
import types
from unittest import mock

import numpy as np

REF = os.environ.get("KMOS_REFERENCE", "/root/reference")
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


def main():
    kmos = import_reference()
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
