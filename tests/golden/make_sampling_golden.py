"""Generates tests/golden/sampling.json: the reference's own get_std_sampled_data code
run on oracle trajectories.

The reference's kmos.run module (kmos/run/__init__.py) is imported with a stand-in
``kmc_model`` whose base / lattice / proclist getters read an oracle trajectory (the
CPU restatement of the compiled step loop) and a stand-in ``kmc_settings``.  Then
KMC_Model.get_std_sampled_data and KMC_Model.get_atoms run unmodified on that state.
The committed JSON pins oracle/sampling.py (the oracle for the engine's on-device
sampling) to the reference's Python arithmetic.

Run with KMOS_REFERENCE set to a checkout of mhoffman/kmos:
    python tests/golden/make_sampling_golden.py
"""
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import import_reference  # noqa: E402

from kmos_gb300 import model as M, program as PG, rates as R  # noqa: E402
from oracle import oracle as O  # noqa: E402

# (fixture model, backend, system size, rng, seed, traj, samples, sample_size)
CASES = [
    ("AB_model", "local_smart", (20, 20), O.RNG_GFORTRAN, 1, 0, 5, 2000),
    ("pairwise_interaction", "lat_int", (16, 16), O.RNG_PHILOX, 3, 2, 4, 3001),
    ("CO_oxidation_Ruo2", "local_smart", (10, 10), O.RNG_PHILOX, 7, 5, 6, 1200),
    ("ZGB_model", "lat_int", (12, 12), O.RNG_PHILOX, 11, 1, 3, 900),
]


def case_rates(model, name):
    if name == "AB_model":
        return json.load(open(os.path.join(HERE, "ab_model_rates.json")))["rates"]
    return [float(r) for r in R.model_rates(model)]


def fake_modules(model, orc):
    """kmc_model (base, lattice, proclist) and kmc_settings backed by ``orc``."""
    base = types.SimpleNamespace(
        get_kmc_time=lambda: orc.kmc_time,
        get_kmc_step=lambda: orc.kmc_step,
        get_kmc_time_step=lambda: orc.kmc_time_step,
        get_procstat=lambda p: int(orc.procstat()[p - 1]),
        get_integ_rate=lambda p: float(orc.integ_rates()[p - 1]),
        set_kmc_time=lambda t: None,
    )
    proclist = types.SimpleNamespace(
        nr_of_proc=len(model.processes),
        get_occupation=lambda: orc.occupation(len(model.species)),
        do_kmc_steps=lambda n: orc.do_kmc_steps(int(n)),  # f2py truncates a float count
    )
    lattice = types.SimpleNamespace()
    km = types.ModuleType("kmc_model")
    km.base, km.lattice, km.proclist = base, lattice, proclist
    settings = types.ModuleType("kmc_settings")
    settings.parameters = {p.name: {"value": p.value, "adjustable": p.adjustable} for p in model.parameters}
    settings.tof_count = {p.name: dict(p.tof_count) for p in model.processes if p.tof_count}
    settings.representations = {s: "" for s in model.species}
    settings.site_names = ["%s_%s" % (layer, site.name) for layer, site in model.site_list()]
    return km, settings


def run_case(kmos_pkg, name, backend, size, rng, seed, traj, samples, sample_size, tof_method):
    model = M.load_json(os.path.join(HERE, "models", name + ".json"))
    prog = PG.compile_model(model, backend)
    orc = O.Oracle(prog, size, seed=seed, rng=rng, traj=traj)
    orc.set_rates(case_rates(model, name))
    orc.update_accum_rate()
    orc.do_kmc_steps(500)  # start from a running state
    km, settings = fake_modules(model, orc)
    sys.modules["kmc_model"] = km
    sys.modules["kmc_settings"] = settings
    if "ase.io" not in sys.modules:  # kmos.run imports ase.io.write for geometry output only
        aseio = types.ModuleType("ase.io")
        aseio.write = lambda *a, **k: None
        sys.modules["ase.io"] = aseio
    for mod in [m for m in sys.modules if m == "kmos.run" or m.startswith("kmos.run.")]:
        del sys.modules[mod]
    import kmos.run as run
    obj = run.KMC_Model.__new__(run.KMC_Model)
    obj.base, obj.proclist, obj.settings = km.base, km.proclist, settings
    obj.size = np.array(list(size) + [1] * (3 - len(size)))
    # KMC_Model.__init__ (run/__init__.py:261-273)
    obj.tofs = tofs = run.get_tof_names()
    obj.tof_matrix = np.zeros((len(tofs), km.proclist.nr_of_proc))
    for process, tof_count in sorted(settings.tof_count.items()):
        process_nr = model.process_ids()[process]
        for tof, tof_factor in tof_count.items():
            obj.tof_matrix[tofs.index(tof), process_nr - 1] += tof_factor
    obj.procstat = np.zeros((km.proclist.nr_of_proc), dtype=np.int64)
    obj.integ_rates = np.zeros((km.proclist.nr_of_proc,))
    obj.time = 0.0
    obj.steps = 0
    out = run.KMC_Model.get_std_sampled_data(obj, samples, sample_size, tof_method=tof_method, output="dict")
    header = obj.get_std_header()
    return {"model": name, "backend": backend, "size": list(size), "rng": rng, "seed": seed, "traj": traj,
            "warmup_steps": 500, "samples": samples, "sample_size": sample_size, "tof_method": tof_method,
            "header": header, "values": [float(out[k]) for k in header[1:].split()]}


def main():
    kmos_pkg = import_reference()
    cases = []
    for c in CASES:
        for method in ("integ", "procrates"):
            cases.append(run_case(kmos_pkg, *c, tof_method=method))
            print(c[0], method, cases[-1]["values"][-3:])
    with open(os.path.join(HERE, "sampling.json"), "w") as f:
        json.dump(cases, f, indent=1)


if __name__ == "__main__":
    main()
