"""Properties of a trajectory's state that hold however long it ran (used on the GPU's
full-size batches, and checked on planted mistakes on the CPU)."""
import numpy as np

from oracle import oracle as O


def table_violations(program, size, lattice, as1, as2, nsites):
    """Violations (strings) of: avail_sites(p, :, 2) the inverse of avail_sites(p,
    1..n_p, 1) with zeros past n_p, and the listed processes exactly those the lattice
    enables (derived from the lattice alone by the oracle's touch-ups)."""
    out = []
    P = len(nsites)
    for p in range(P):
        n = int(nsites[p])
        listed = as1[p][1:n + 1]
        if not ((listed >= 1).all() and (as1[p][n + 1:] == 0).all()):
            out.append("process %d: list entries out of range or past its length" % (p + 1))
            continue
        if not (as2[p][listed] == np.arange(1, n + 1)).all() or int((as2[p][1:] != 0).sum()) != n:
            out.append("process %d: positions are not the inverse of the list" % (p + 1))
    rb = O.Oracle(program, size, seed=1).rebuild_tables(lattice)
    for p in range(P):
        got = set(as1[p][1:int(nsites[p]) + 1].tolist())
        want = set(rb["as1"][p][1:int(rb["nsites"][p]) + 1].tolist())
        if got != want:
            out.append("process %d: lists %d sites, the lattice enables %d" % (p + 1, len(got), len(want)))
    return out
