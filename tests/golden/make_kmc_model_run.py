"""Generates tests/golden/kmc_model_run.json: the reference's own kmos.run.KMC_Model
driving this package's drop-in module (kmos_gb300.kmc_model) unchanged.

For each case the model is exported with kmos_gb300.export (kmc_model.py, which
configures the drop-in, and kmc_settings.py), and the reference's kmos.run
(kmos/run/__init__.py) is imported from KMOS_REFERENCE with ase stubbed (kmos.run imports
it for geometry output only).  Then, through KMC_Model's public methods:
  KMC_Model(size, random_seed) -- reset: proclist.init, set_rate_constants,
      base.update_accum_rate / update_integ_rate (run:155-339, 2369-2437);
  do_steps (416-432); get_atoms(geometry=False) (680-850);
  get_std_sampled_data with tof_method "integ" and "procrates" (865-966);
  get_next_kmc_step + run_proc_nr (1357-1367); put + _adjust_database (1288-1314,
      1439-1457); do_steps again; deallocate (388-414).
The drop-in's engine is the oracle here (tests/dropin_replay.py: OracleTrajectory), so
nothing needs a GPU.  Every access the reference's code makes to the module's base /
lattice / proclist is recorded with its arguments and result; the fixture holds that log
and KMC_Model's outputs.  tests/test_gpu_kmc_model_run.py replays the log on the GPU
drop-in; tests/test_kmc_model_replay.py replays it on the oracle-backed one.

Run with KMOS_REFERENCE set to a checkout of mhoffman/kmos:
    python tests/golden/make_kmc_model_run.py
"""
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, HERE)

from make_golden import import_reference  # noqa: E402

import dropin_replay as DR  # noqa: E402
from kmos_gb300 import engine as E, export, kmc_model  # noqa: E402

# (fixture model, backend, system size, random seed, steps, samples, sample size, put site, put species)
# (models whose rate constants need no JANAF chemical potentials, absent here)
CASES = [
    ("AB_model", "local_smart", (20, 20), 1, 3000, 4, 4000, (3, 4, 0, 1), "A"),
    ("default_xml", "lat_int", (10, 10), 3, 3000, 4, 4000, (5, 2, 0, 2), "CO"),
    ("ZGB_model", "local_smart", (16, 16), 7, 2000, 3, 3000, (1, 1, 0, 1), "CO"),
]


def run_case(name, backend, size, seed, steps, samples, sample_size, put_site, put_species):
    log = []
    with tempfile.TemporaryDirectory() as tmp:
        export.export(os.path.join(HERE, "models", name + ".json"), tmp, backend)
        sys.path.insert(0, tmp)
        for mod in ("kmc_model", "kmc_settings"):
            sys.modules.pop(mod, None)
        import kmc_settings  # noqa: F401  (the exported settings)
        import kmc_model as exported
        km = types.ModuleType("kmc_model")
        km.base = DR.Recorder("base", exported.base, log)
        km.lattice = DR.Recorder("lattice", exported.lattice, log)
        km.proclist = DR.Recorder("proclist", exported.proclist, log)
        sys.modules["kmc_model"] = km
        for mod in [m for m in sys.modules if m == "kmos.run" or m.startswith("kmos.run.")]:
            del sys.modules[mod]
        import kmos.run as run
        model = run.KMC_Model(size=size, print_rates=False, banner=False, random_seed=seed)
        model.do_steps(steps)
        atoms = model.get_atoms(geometry=False)
        out = {"atoms": {k: DR.enc(getattr(atoms, k)) for k in
                         ("kmc_time", "kmc_step", "occupation", "procstat", "integ_rates", "tof_data", "tof_integ")}}
        for method in ("integ", "procrates"):
            data = model.get_std_sampled_data(samples, sample_size, tof_method=method, output="dict")
            out["std_" + method] = {k: float(v) for k, v in data.items()}
        events = []
        for _ in range(40):
            proc, site = model.get_next_kmc_step()
            events.append([int(proc), int(site), bool(model.run_proc_nr(proc, site))])
        out["events"] = events
        species = getattr(model.proclist, put_species.lower())
        model.put(list(put_site), species)
        model.do_steps(steps)
        out["after_put"] = {"kmc_step": int(model.base.get_kmc_step()),
                            "occupation": DR.enc(np.array(model.proclist.get_occupation()))}
        model.deallocate()
        sys.path.remove(tmp)
        for mod in ("kmc_model", "kmc_settings"):
            sys.modules.pop(mod, None)
    return {"model": name, "backend": backend, "size": list(size), "seed": seed, "outputs": out, "log": log}


def main():
    import_reference()
    if "ase.io" not in sys.modules:  # kmos.run imports ase.io.write for geometry output only
        aseio = types.ModuleType("ase.io")
        aseio.write = lambda *a, **k: None
        sys.modules["ase.io"] = aseio
    E.Trajectory = DR.OracleTrajectory  # the oracle as the drop-in's engine
    cases = []
    for c in CASES:
        cases.append(run_case(*c))
        kmc_model.__dict__.pop("_state", None)
        print(c[0], c[1], len(cases[-1]["log"]), "calls",
              cases[-1]["outputs"]["std_integ"].get("kmc_steps"))
    with open(os.path.join(HERE, "kmc_model_run.json"), "w") as f:
        json.dump(cases, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
