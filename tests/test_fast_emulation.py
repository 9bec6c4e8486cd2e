"""The fast step's semantics on the CPU: every process's resolved fast stream
(kmos_gb300/program.py), evaluated the way the step kernel evaluates it -- all
conditions on the slot values from before the step, then the edits that fire applied in
program order, then the final species of the replaced slots -- must leave the lattice,
both avail_sites columns and nr_of_sites exactly as the oracle's serial interpretation
of the op program (run_proc_nr, the reference's put/take and lat_int order) leaves them.

Checked on many steps of oracle trajectories of every fixture model under both backends,
the three-site model, and models compiled without nli tables (member scans).  The edits
are applied twice: directly, and the way the kernel's replay applies them (lane-private
write log, values loaded before the replay, the entries it leaves out of the log), so
that the argument that no read needs an unlogged entry is checked too.  The GPU parity
tests check the kernel itself; this pins the stream encoding and the replay's reads
independently of it.
"""
import numpy as np
import pytest

from conftest import fixture_model, many_species_model, rows_model, trimer_model
from kmos_gb300 import program as PG
from oracle import oracle as O


def s8(v):
    return v - 256 if v >= 128 else v


def in_mask(species, mask):
    return ((mask & 0xFFFFFFFF) >> (31 if species < 0 else species)) & 1


def emulate(words, ex, proc, site, dims, replay=False):
    """The fast step of (proc, site) applied to copies of the exported state; None when
    the process has no fast stream.  replay: apply the edits the way the kernel's
    replay does (write log, values loaded before the replay) instead of directly."""
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
    if replay:
        replay_like_the_kernel(fired, as1, as2, ns, dels_first=bool((w3 >> 20) & 1))
    else:
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


LOG_MAX, TAIL_MAX, TAIL_PROCS = 16, 6, 64  # the kernel's (kmc_device.cuh)


def replay_like_the_kernel(fired, as1, as2, ns, dels_first):
    """The step kernel's replay (replay_process): each process on its own, reads of a
    del's position and of the list top from the lane's write log (newest first), else
    from the values loaded before the replay (the position of every del's site, the
    top TAIL_MAX list entries), else from memory, which every write reaches; the
    vacated top entries are never logged, and in a dels-first stream neither are the
    cleared positions nor the adds.  A read that needed an entry left out of the log
    would see a value from before the step, and the tables would come out wrong."""
    pre1, pre2, n0s = as1.copy(), as2.copy(), ns.copy()
    for p in sorted({p for _k, p, _s in fired}):
        q = p - 1
        edits = [(k, s) for k, pp, s in fired if pp == p]
        ndel = sum(1 for k, _s in edits if k != "add")
        n0 = n0s[q]
        tail = {n0 - j: pre1[q, n0 - j] for j in range(min(ndel, TAIL_MAX)) if n0 - j >= 1} if q < TAIL_PROCS else {}
        log, logok, n = [], True, n0

        def put(table, index, val, logged=True):
            nonlocal logok
            (as2 if table else as1)[q, index] = val
            if logged and logok:
                if len(log) < LOG_MAX:
                    log.append(((table, index), val))
                else:
                    logok = False

        def lookup(table, index):
            for key, val in reversed(log):
                if key == (table, index):
                    return val
            return None

        for kind, s in edits:
            if kind == "add":
                n += 1
                put(0, n, s, not dels_first)
                put(1, s, n, not dels_first)
                continue
            if not logok:
                m = as2[q, s]
            else:
                m = lookup(1, s)
                m = pre2[q, s] if m is None else m
            if m == 0:
                assert kind == "gdel", "an nli del of an absent entry"
                continue
            if m < n:
                if not logok:
                    last = as1[q, n]
                else:
                    last = lookup(0, n)
                    if last is None and q < TAIL_PROCS and n0 - n < TAIL_MAX and n <= n0:
                        assert n in tail, "the kernel would read a list entry it did not load"
                        last = tail[n]
                    elif last is None:
                        last = as1[q, n]
                put(0, m, last)
                put(0, n, 0, False)
                put(1, last, m)
            else:
                put(0, m, 0, False)
            put(1, s, 0, not dels_first)
            n -= 1
        ns[q] = n


CASES = [("AB_model", "local_smart", (20, 20), True), ("ZGB_model", "local_smart", (16, 12), True),
         ("ZGB_model", "lat_int", (12, 16), True), ("CO_oxidation_Ruo2", "local_smart", (10, 10), True),
         ("CO_oxidation_Ruo2", "lat_int", (14, 14), True), ("pairwise_interaction", "lat_int", (16, 16), True),
         ("pairwise_interaction", "local_smart", (8, 8), True), ("default_xml", "local_smart", (10, 10), True),
         ("pdopd_xml", "local_smart", (8, 8), True), ("pdopd_xml", "lat_int", (8, 8), True),
         ("trimer", "local_smart", (14, 14), True), ("trimer", "lat_int", (14, 14), True),
         ("trimer", "lat_int", (14, 14), False), ("pairwise_interaction", "lat_int", (16, 16), False),
         # the smallest lattices the fast path takes: short lists, so a del often reads an
         # entry an earlier del of the same step moved (the replay's write log is used)
         ("ZGB_model", "lat_int", (5, 5), True), ("CO_oxidation_Ruo2", "lat_int", (5, 5), True),
         ("ZGB_model", "local_smart", (5, 5), True), ("default_xml", "local_smart", (5, 5), True),
         # 96 processes: fast streams of processes past the 64th, whose list tops the
         # kernel does not load ahead
         ("many_species", "local_smart", (8, 8), True),
         # row desorption: dozens of dels of one process in one step, more than the list
         # tops loaded ahead and than the replay log holds
         ("rows", "local_smart", (16, 6), True), ("rows", "lat_int", (32, 4), True)]


@pytest.mark.parametrize("name,backend,size,tables", CASES)
def test_fast_stream_equals_serial_interpretation(name, backend, size, tables, monkeypatch):
    if not tables:
        monkeypatch.setattr(PG, "NLI_TABLE_MAX", 0)
    model = {"trimer": trimer_model, "many_species": many_species_model,
             "rows": rows_model}.get(name, lambda: fixture_model(name))()
    prog = PG.compile_model(model, backend)
    monkeypatch.undo()
    reach = int(prog.words[19])
    assert size[0] > 2 * (reach & 0xFF) and size[1] > 2 * ((reach >> 8) & 0xFF)  # the fast path's lattices
    rates = (10.0 ** np.random.default_rng(3).uniform(-1, 2, size=prog.nproc)).tolist()
    if name == "rows":
        rates = [20.0, 1.0, 50.0]  # rows fill up and leave often
    o = O.Oracle(prog, size, seed=11, rng=O.RNG_PHILOX, traj=1)
    o.set_rates(rates)
    o.update_accum_rate()
    dims = (size[0], size[1], 1)
    checked = 0
    for block in range(12):
        o.do_kmc_steps(150)
        for _ in range(8):
            proc, site = o.get_next_kmc_step()
            before = o.export()
            got = emulate(prog.words, before, proc, site, dims)
            got_replay = emulate(prog.words, before, proc, site, dims, replay=True)
            o.run_proc_nr(proc, site)
            if got is None:
                continue
            ex = o.export()
            for g in (got, got_replay):
                np.testing.assert_array_equal(g[0], ex["lattice"])
                np.testing.assert_array_equal(g[1], ex["as1"])
                np.testing.assert_array_equal(g[2], ex["as2"])
                np.testing.assert_array_equal(g[3], ex["nsites"])
            checked += 1
    assert checked > 40
