"""The fast step's semantics on the CPU: every process's resolved fast stream
(kmos_gb300/program.py), evaluated the way the step kernel evaluates it -- all
conditions on the slot values from before the step, then the edits that fire applied in
program order, then the final species of the replaced slots -- must leave the lattice,
both avail_sites columns and nr_of_sites exactly as the oracle's serial interpretation
of the op program (run_proc_nr, the reference's put/take and lat_int order) leaves them.

Checked on many steps of oracle trajectories of every fixture model under both backends,
the three-site model, and models compiled without nli tables (member scans).  The GPU
parity tests check the kernel itself; this pins the stream encoding independently of it.
"""
import numpy as np
import pytest

from conftest import fixture_model, trimer_model
from kmos_gb300 import program as PG
from oracle import oracle as O


def s8(v):
    return v - 256 if v >= 128 else v


def in_mask(species, mask):
    return ((mask & 0xFFFFFFFF) >> (31 if species < 0 else species)) & 1


def emulate(words, ex, proc, site, dims):
    """The fast step of (proc, site) applied to copies of the exported state; None when
    the process has no fast stream."""
    w = [int(x) for x in words]
    ns_species, spuck = w[4], w[6]
    hot = w[w[21]:w[21] + w[20]]
    off = hot[proc - 1]
    if off == 0:
        return None
    X, Y, Z = dims
    nlat, nchk, nwr, w3 = hot[off:off + 4]
    nedit, nq = w3 & 0xFFFF, (w3 >> 16) & 0xF
    coords = hot[off + 4:off + 4 + nlat]
    wr = hot[off + 4 + nlat + 2 * nchk:off + 4 + nlat + 2 * nchk + 2 * nwr]
    rec = off + ((4 + nlat + 2 * nchk + 2 * nwr + 3) & ~3)
    c = (site - 1) // spuck
    bx, by, bz = c % X, (c // X) % Y, c // (X * Y)
    lat = ex["lattice"].copy()
    as1, as2, ns = ex["as1"].copy(), ex["as2"].copy(), ex["nsites"].copy()
    latsite, latv = [], []
    for cw in coords:
        u = cw & 0xFFFFFFFF
        x = (bx + s8(u & 0xFF)) % X
        y = (by + s8((u >> 8) & 0xFF)) % Y
        z = (bz + s8((u >> 16) & 0xFF)) % Z
        s = spuck * (x + X * (y + Y * z)) + (u >> 24)
        latsite.append(s)
        latv.append(int(lat[s - 1]))

    def code(v):
        return ns_species if v < 0 or v > ns_species else v

    def ref_value(r):
        return latv[r] if r >= 0 else -r - 2

    fired = []  # (kind, process, site) in program order, all decided on pre-step values
    for k in range(nedit):
        q0 = hot[rec + 4 * k:rec + 4 * k + 4]
        h = q0[0] & 0xFFFFFFFF
        op, cnt, arg = h & 0xFF, (h >> 8) & 0xFF, h >> 16
        target = latsite[q0[1]]
        if op >= 6:
            refs = [hot[rec + 4 * ((1 + j // 4) * nedit + k) + j % 4] for j in range(4 * nq)]
            p = hot[q0[2] + sum(code(latv[r & 0xFF]) * (r >> 8) for r in refs)]
            if p:
                fired.append(("del" if op == 6 else "add", p, target))
        elif op == 2:
            fired.append(("gdel", arg, target))
        elif op == 3:
            if cnt <= 1:
                on = cnt == 0 or in_mask(latv[q0[2]], q0[3])
            else:
                e = off + q0[2]
                on = all(in_mask(ref_value(hot[e + 2 + j]), hot[e + 2 + cnt + j]) for j in range(cnt))
            if on:
                fired.append(("add", arg, target))
        else:
            e = off + q0[2]
            roff, refs = hot[e + 3], hot[e + 4:e + 4 + cnt]
            M, K = hot[roff], hot[roff + 1]
            vals = [ref_value(r) for r in refs]
            p = 0
            for m in range(M):
                mem = hot[roff + 2 + K + m * (1 + K):roff + 2 + K + (m + 1) * (1 + K)]
                if all(in_mask(v, mem[1 + j]) for j, v in enumerate(vals)):
                    p = mem[0]
            if p:
                fired.append(("del" if op == 4 else "add", p, target))
    for kind, p, s in fired:  # add_proc / del_proc (base.mpy:211-302), program order
        q = p - 1
        n = ns[q]
        if kind == "add":
            as1[q, n + 1] = s
            as2[q, s] = n + 1
            ns[q] = n + 1
            continue
        m = as2[q, s]
        if m == 0:
            assert kind == "gdel", "an nli del of an absent entry"
            continue
        last = as1[q, n]
        if m < n:
            as1[q, m] = last
            as2[q, last] = m
            as1[q, n] = 0
        else:
            as1[q, m] = 0
        as2[q, s] = 0
        ns[q] = n - 1
    for j in range(nwr):
        lat[latsite[wr[2 * j]] - 1] = wr[2 * j + 1]
    return lat, as1, as2, ns


CASES = [("AB_model", "local_smart", (20, 20), True), ("ZGB_model", "local_smart", (16, 12), True),
         ("ZGB_model", "lat_int", (12, 16), True), ("CO_oxidation_Ruo2", "local_smart", (10, 10), True),
         ("CO_oxidation_Ruo2", "lat_int", (14, 14), True), ("pairwise_interaction", "lat_int", (16, 16), True),
         ("pairwise_interaction", "local_smart", (8, 8), True), ("default_xml", "local_smart", (10, 10), True),
         ("pdopd_xml", "local_smart", (8, 8), True), ("pdopd_xml", "lat_int", (8, 8), True),
         ("trimer", "local_smart", (14, 14), True), ("trimer", "lat_int", (14, 14), True),
         ("trimer", "lat_int", (14, 14), False), ("pairwise_interaction", "lat_int", (16, 16), False)]


@pytest.mark.parametrize("name,backend,size,tables", CASES)
def test_fast_stream_equals_serial_interpretation(name, backend, size, tables, monkeypatch):
    if not tables:
        monkeypatch.setattr(PG, "NLI_TABLE_MAX", 0)
    prog = PG.compile_model(trimer_model() if name == "trimer" else fixture_model(name), backend)
    monkeypatch.undo()
    rates = (10.0 ** np.random.default_rng(3).uniform(-1, 2, size=prog.nproc)).tolist()
    o = O.Oracle(prog, size, seed=11, rng=O.RNG_PHILOX, traj=1)
    o.set_rates(rates)
    o.update_accum_rate()
    dims = (size[0], size[1], 1)
    checked = 0
    for block in range(12):
        o.do_kmc_steps(150)
        for _ in range(8):
            proc, site = o.get_next_kmc_step()
            got = emulate(prog.words, o.export(), proc, site, dims)
            o.run_proc_nr(proc, site)
            if got is None:
                continue
            ex = o.export()
            np.testing.assert_array_equal(got[0], ex["lattice"])
            np.testing.assert_array_equal(got[1], ex["as1"])
            np.testing.assert_array_equal(got[2], ex["as2"])
            np.testing.assert_array_equal(got[3], ex["nsites"])
            checked += 1
    assert checked > 40
