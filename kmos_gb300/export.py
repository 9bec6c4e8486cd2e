"""Writes a model directory that ``kmos.run`` can run on the GB300 engine.

``kmos export`` writes Fortran sources plus ``kmc_settings.py`` (kmos/io/__init__.py:
3725-3845) and builds them into ``kmc_model`` with f2py.  This writes, instead of the
Fortran and the f2py build, a ``kmc_model.py`` that configures the engine's drop-in
(``kmos_gb300.kmc_model``) for the model, and a ``kmc_settings.py`` with the fields
``kmos.run`` reads: parameters, rate_constants, tof_count, site_names, representations,
lattice_representation, species_tags, simulation_size, random_seed, setup_model.

    python -m kmos_gb300.export model.ini out_dir [local_smart|lat_int|otf]

An otf export's ``kmc_model`` also has ``proclist_pars`` (kmos.run imports it when present).
"""
from __future__ import annotations

import json
import os
import sys

from .model import load, to_dict


def export(model_path: str, out_dir: str, backend: str = "local_smart") -> None:
    m = load(model_path)
    d = to_dict(m)
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, "kmc_model.py"), "w") as fh:
        fh.write('"""f2py-compatible kmc_model running on the GB300 engine (model %s, %s)."""\n'
                 % (m.name, backend))
        fh.write("import kmc_settings as _settings\n")
        fh.write("from kmos_gb300.kmc_model import configure as _configure\n\n")
        fh.write("base, lattice, proclist = _configure(_settings.model_json, _settings.backend)\n")
        if backend == "otf":
            fh.write("from kmos_gb300.kmc_model import proclist_pars  # noqa: E402\n")
    out = []
    out.append("model_name = %r\n" % m.name)
    out.append("simulation_size = 20\nrandom_seed = 1\nbackend = %r\n\n" % backend)
    out.append("def setup_model(model):\n    pass\n\n")
    out.append("parameters = {\n")
    for p in m.parameters:
        out.append('    %r:{"value":%r, "adjustable":%r, "min":%r, "max":%r,"scale":%r},\n'
                   % (p.name, str(p.value), p.adjustable, str(p.min), str(p.max), p.scale))
    out.append("    }\n\nrate_constants = {\n")
    for p in m.processes:
        out.append("    %r:(%r, %r),\n" % (p.name, p.rate_constant, p.enabled))
    out.append("    }\n\n")
    out.append("site_names = %r\n" % ["%s_%s" % (l, s.name) for l, s in m.site_list()])
    out.append("representations = {\n")
    for sp in sorted(m.species):
        out.append('    %r:"""%s""",\n' % (sp, m.representations.get(sp, "").strip()))
    out.append('    }\n\nlattice_representation = """"""\n\nspecies_tags = {\n')
    for sp in sorted(m.species):
        out.append('    %r:"""""",\n' % sp)
    out.append("    }\n\ntof_count = {\n")
    for p in m.processes:
        if p.tof_count is not None:
            out.append("    %r:%r,\n" % (p.name, p.tof_count))
    out.append("    }\n\n")
    out.append("model_json = %r\n" % (d,))
    with open(os.path.join(out_dir, "kmc_settings.py"), "w") as fh:
        fh.write("".join(out))


if __name__ == "__main__":
    export(sys.argv[1], sys.argv[2], sys.argv[3] if len(sys.argv) > 3 else "local_smart")
