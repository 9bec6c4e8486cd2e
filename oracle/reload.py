"""kmos ``.reload`` files, restated for the oracle.

TEST INFRASTRUCTURE ONLY: tests/ use this module to check the engine's
``kmc_save_reload`` / ``kmc_load_reload`` against an independent writer and reader of
the same layout.  The product never imports it.

Layout (mhoffman/kmos, kmos/fortran_src/base.mpy):
  save_system   base.mpy:489-575 -- a comment line, ``#Scalar variables``, then
                kmc_time (a,ES22.15), walltime (a,ES13.7), kmc_step (a,I22), nr_of_proc
                and volume (list-directed), ``#Vector variables``, procstat (a,P*I21),
                nr_of_sites (a,P*I9), rates (a,P*ES14.7), lattice (a,V*I9), then one
                line per process of avail_sites(p,:,1) and of avail_sites(p,:,2), each
                (a,(V+1)*I9) with the process number first.
  reload_system base.mpy:363-486 -- label-directed list reads; lines starting with
                ``#`` are skipped.
Edit descriptors follow the Fortran standard: ESw.d writes one non-zero digit before
the point and d after, exponent ``E+dd`` for |e| <= 99 and ``+ddd`` (no letter) for
|e| <= 999, right-justified; a field that does not fit is w asterisks.  List-directed
default-integer output (gfortran) is a blank then the value right-justified in 12.
"""
from __future__ import annotations

import numpy as np


def es(v: float, w: int, d: int) -> str:
    """Fortran ESw.d."""
    v = float(v)
    if v != v:
        s = "NaN"
    elif v in (float("inf"), float("-inf")):
        s = "Infinity" if v > 0 else "-Infinity"
        if len(s) > w:
            s = "Inf" if v > 0 else "-Inf"
    else:
        mant, _, ex = ("{:.%dE}" % d).format(v).partition("E")
        e = int(ex)
        if -99 <= e <= 99:
            s = "%sE%s%02d" % (mant, "-" if e < 0 else "+", abs(e))
        else:
            s = "%s%s%03d" % (mant, "-" if e < 0 else "+", abs(e))
    return "*" * w if len(s) > w else s.rjust(w)


def iw(v: int, w: int) -> str:
    """Fortran Iw."""
    s = str(int(v))
    return "*" * w if len(s) > w else s.rjust(w)


def write_reload(path: str, kmc_time: float, walltime: float, kmc_step: int, procstat, nsites, rates, lattice,
                 as1, as2):
    """save_system's file; as1 / as2 are [P][V+1] with index 0 unused (avail_sites(p, i, 1 / 2))."""
    P, V = len(nsites), len(lattice)
    out = ["#Reload file written by kmos. Do not edit manually!", "#Scalar variables",
           " kmc_time  " + es(kmc_time, 22, 15), " walltime   " + es(walltime, 13, 7),
           " kmc_step " + iw(kmc_step, 22), " nr_of_proc " + iw(P, 12), " volume " + iw(V, 12),
           "#Vector variables",
           "procstat " + "".join(iw(x, 21) for x in procstat),
           "nr_of_sites " + "".join(iw(x, 9) for x in nsites),
           "rates " + "".join(es(x, 14, 7) for x in rates),
           "lattice " + "".join(iw(x, 9) for x in lattice)]
    for p in range(P):
        out.append("avail_sites " + iw(p + 1, 9) + "".join(iw(x, 9) for x in as1[p][1:]))
    for p in range(P):
        out.append("avail_sites_back " + iw(p + 1, 9) + "".join(iw(x, 9) for x in as2[p][1:]))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def write_oracle_reload(path: str, o, walltime: float = 0.0):
    """save_system for an oracle trajectory."""
    ex = o.export()
    write_reload(path, o.kmc_time, walltime, o.kmc_step, ex["procstat"], ex["nsites"], o.rates(), ex["lattice"],
                 ex["as1"], ex["as2"])


def _real(tok: str) -> float:
    t = tok.replace("D", "E").replace("d", "E")
    if "E" not in t.upper():
        for k in range(1, len(t)):
            if t[k] in "+-" and (t[k - 1].isdigit() or t[k - 1] == "."):
                t = t[:k] + "E" + t[k:]
                break
    return float(t)


def read_reload(path: str) -> dict:
    """reload_system's two passes over the labels it knows; other lines are ignored."""
    r = {"as1": {}, "as2": {}}
    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok or tok[0].startswith("#"):
                continue
            label, rest = tok[0], tok[1:]
            if label in ("nr_of_proc", "volume", "kmc_step"):
                r[label] = int(rest[0])
            elif label in ("kmc_time", "walltime"):
                r[label] = _real(rest[0])
            elif label in ("lattice", "nr_of_sites", "procstat"):
                r[label] = np.array([int(x) for x in rest], dtype=np.int64)
            elif label == "rates":
                r[label] = np.array([_real(x) for x in rest])
            elif label in ("avail_sites", "avail_sites_back"):
                r["as1" if label == "avail_sites" else "as2"][int(rest[0])] = np.array([int(x) for x in rest[1:]],
                                                                                         dtype=np.int64)
    return r
