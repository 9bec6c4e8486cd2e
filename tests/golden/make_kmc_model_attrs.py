"""Writes kmc_model_attrs.json: the attributes of the f2py module's base / lattice /
proclist objects that kmos.run and the kmos CLI read (every ``base.X``, ``lattice.X``,
``proclist.X`` and ``self.base.X`` ... in their source), the list the drop-in module
(kmos_gb300.kmc_model) must provide.

Run with KMOS_REFERENCE set to a checkout of mhoffman/kmos:
    python tests/golden/make_kmc_model_attrs.py
"""
import json
import os
import re

REF = os.environ.get("KMOS_REFERENCE")
if not REF:
    raise SystemExit("set KMOS_REFERENCE to a checkout of mhoffman/kmos")
FILES = ["kmos/run/__init__.py", "kmos/cli.py"]
HERE = os.path.dirname(os.path.abspath(__file__))

attrs = {"base": set(), "lattice": set(), "proclist": set()}
for rel in FILES:
    src = open(os.path.join(REF, rel)).read()
    for mod, name in re.findall(r"\b(?:self\.)?(base|lattice|proclist)\.([A-Za-z_][A-Za-z_0-9]*)", src):
        attrs[mod].add(name)
out = {k: sorted(v) for k, v in attrs.items()}
out["sources"] = FILES
json.dump(out, open(os.path.join(HERE, "kmc_model_attrs.json"), "w"), indent=1)
print({k: len(v) for k, v in attrs.items()})
