"""Generates the otf-backend golden fixtures from the reference checkout.

Run with KMOS_REFERENCE set to a checkout of mhoffman/kmos;
the tests read only the committed outputs.

Outputs
  models/intZGB_otf.json    tests/export_test/intZGB_otf.xml (bystanders and otf_rate
                            expressions), read with kmos_gb300.model.load_xml since the
                            reference's XML reader needs lxml, absent here.
  ops/intZGB_otf_otf.json   op order of the reference's own golden otf exports
  ops/default_xml_otf.json  (tests/export_test/reference_export_intZGB_otf and
                            reference_export_otf, the latter default.xml), read by
                            fortran_ops.otf_ops: per process the dels, replaces, rate
                            updates and adds of run_proc_<name>, the touch-up of a cell,
                            and every gr_<name> function's bystander counting and rate
                            expression.
"""
import json
import os
import sys

REF = os.environ.get("KMOS_REFERENCE")
if not REF:
    raise SystemExit("set KMOS_REFERENCE to a checkout of mhoffman/kmos")
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import fortran_ops as F  # noqa: E402
from kmos_gb300 import model as M  # noqa: E402


def jsonable(ops):
    return [[op[0]] + [list(x) if isinstance(x, tuple) else x for x in op[1:]] for op in ops]


def main():
    m = M.load_xml(os.path.join(REF, "tests/export_test/intZGB_otf.xml"))
    M.save_json(m, os.path.join(HERE, "models", "intZGB_otf.json"))
    for name, d in (("intZGB_otf", "reference_export_intZGB_otf"), ("default_xml", "reference_export_otf")):
        g = F.otf_ops(os.path.join(REF, "tests/export_test", d))
        out = {"procs": {str(p): jsonable(ops) for p, ops in sorted(g["procs"].items())},
               "touchups": {k: jsonable(v) for k, v in g["touchups"].items()},
               "rates": {str(p): r for p, r in sorted(g["rates"].items())}}
        with open(os.path.join(HERE, "ops", "%s_otf.json" % name), "w") as fh:
            json.dump(out, fh, indent=0)


if __name__ == "__main__":
    main()
