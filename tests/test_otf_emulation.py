"""The otf step kernel's two shortcuts, emulated on the CPU against the oracle.

1. Event replay (run_event in kmos_gb300/csrc/kmc_otf.cu): the lattice writes first, then
   every table op's avail_sites(p, site, 2) and every add condition and rate taken
   from the state before the table ops (positions) and the final lattice (conditions,
   rates); the replay uses a loaded position only while no earlier op of the event has
   deleted or added an entry of that process, and skips the rate of an update whose
   entry was absent before the event.  Emulated step by step on oracle trajectories, it
   must leave avail_sites, nr_of_sites and every entry's rate exactly as the oracle's
   serial run_proc_nr does.
2. Running sums: each list re-summed only from the first entry the event changed (the
   smallest position an add, a del or an update wrote) must equal the oracle's full
   left-to-right re-sum of update_accum_rate, bit for bit.
"""
import numpy as np
import pytest

from conftest import fixture_model
from kmos_gb300 import otf as OTF, program as PG
from oracle import oracle as O

OP_REPLACE, OP_GDEL, OP_ADD, OP_UPDATE = 1, 2, 3, 7


def in_mask(sp, mask):
    return ((int(mask) & 0xFFFFFFFF) >> (31 if sp < 0 else sp)) & 1


class Emu:
    def __init__(self, prog, size, params, o):
        self.w = [int(x) for x in prog.words]
        self.X, self.Y = size
        self.spuck = self.w[6]
        self.P = self.w[3]
        self.params = params
        self.o = o

    def site(self, bx, by, cw):
        u = cw & 0xFFFFFFFF
        dx, dy = [(v - 256 if v >= 128 else v) for v in (u & 0xFF, (u >> 8) & 0xFF)]
        return self.spuck * (((bx + dx) % self.X) + self.X * ((by + dy) % self.Y)) + (u >> 24), bx + dx, by + dy

    def rate(self, lat, p, cx, cy):
        w = self.w
        r = w[w[22] + p - 1]
        nb, nv = w[r], w[r + 1]
        nr, pos = [0] * nv, r + 4
        for _ in range(nb):
            s, _x, _y = self.site(cx, cy, w[pos])
            for j in range(w[pos + 1]):
                if lat[s - 1] == w[pos + 2 + 2 * j]:
                    nr[w[pos + 3 + 2 * j]] += 1
            pos += 2 + 2 * w[pos + 1]
        return OTF.evaluate(w[pos:], self.o.rates()[p - 1], self.params, nr)

    def event(self, proc, site, st):
        """run_event on copies of the exported state; returns (lat, as1, as2, ns, rm, dirty)."""
        w = self.w
        lat = st["lattice"].copy()
        as1, as2, ns, rm = st["as1"].copy(), st["as2"].copy(), st["nsites"].copy(), st["rm"].copy()
        dirty = [10 ** 9] * self.P
        c = (site - 1) // self.spuck
        bx, by = c % self.X, c // self.X
        ops, p = [], w[w[10] + proc - 1]
        while True:   # phase 1: lattice writes, table ops listed
            h = w[p] & 0xFFFFFFFF
            op, cnt, arg = h & 0xFF, (h >> 8) & 0xFF, h >> 16
            if op == 0:
                break
            if op == OP_REPLACE:
                s, _x, _y = self.site(bx, by, w[p + 1])
                assert in_mask(lat[s - 1], w[p + 2])
                lat[s - 1] = w[p + 3]
                p += 4
                continue
            ops.append(p)
            p += 2 + 2 * cnt if op == OP_ADD else 2
        pre = []      # phase 2: positions before the event, conditions and rates after the writes
        for p in ops:
            h = w[p] & 0xFFFFFFFF
            op, cnt, arg = h & 0xFF, (h >> 8) & 0xFF, h >> 16
            s, cx, cy = self.site(bx, by, w[p + 1])
            m0 = int(as2[arg - 1, s])
            ok = op == OP_ADD or (op == OP_UPDATE and m0 != 0)
            if op == OP_ADD:
                ok = all(in_mask(lat[self.site(bx, by, w[p + 2 + 2 * j])[0] - 1], w[p + 3 + 2 * j])
                         for j in range(cnt))
            pre.append((m0, ok, self.rate(lat, arg, cx, cy) if ok else 0.0))
        moved = set()
        for p, (m0, ok, rate) in zip(ops, pre):   # phase 3: the replay
            h = w[p] & 0xFFFFFFFF
            op, arg = h & 0xFF, h >> 16
            q = arg - 1
            s, _cx, _cy = self.site(bx, by, w[p + 1])
            m = m0 if q not in moved else int(as2[q, s])
            if q not in moved:
                assert m == as2[q, s], "a loaded position went stale"
            if op == OP_GDEL:
                if m:
                    n = ns[q]
                    if m < n:
                        last = as1[q, n]
                        as1[q, m], as1[q, n] = last, 0
                        rm[q, m], rm[q, n] = rm[q, n], 0.0
                        as2[q, last] = m
                    else:
                        as1[q, m], rm[q, m] = 0, 0.0
                    as2[q, s] = 0
                    ns[q] = n - 1
                    dirty[q] = min(dirty[q], m)
                    moved.add(q)
            elif op == OP_ADD:
                if ok:
                    assert m == 0
                    n = ns[q] + 1
                    ns[q] = n
                    as1[q, n], as2[q, s], rm[q, n] = s, n, rate
                    dirty[q] = min(dirty[q], n)
                    moved.add(q)
            else:
                if m:
                    assert ok, "an update of an entry that was absent before the event"
                    rm[q, m] = rate
                    dirty[q] = min(dirty[q], m)
        return lat, as1, as2, ns, rm, dirty


CASES = [("intZGB_otf", (12, 10), [0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3], [1.3, 0.7, 1.9, 1e-10, 0.5]),
         ("default_xml", (8, 6), None, None), ("AB_model", (10, 10), None, None)]


@pytest.mark.parametrize("name,size,rates,params", CASES)
def test_event_replay_and_running_sums(name, size, rates, params):
    m = fixture_model(name)
    prog = PG.compile_model(m, "otf")
    rates = rates or (10.0 ** np.random.default_rng(5).uniform(-1, 2, size=len(m.processes))).tolist()
    params = params if params is not None else OTF.user_parameter_values(m)
    o = O.Oracle(prog, size, seed=9, rng=O.RNG_PHILOX, traj=2)
    o.set_rates(rates)
    o.set_user_parameters(params)
    o.recalculate_rates_matrix()
    o.update_accum_rate()
    emu = Emu(prog, size, params, o)
    checked = 0
    for block in range(10):
        o.do_kmc_steps(137)
        for _ in range(6):
            proc, site = o.get_next_kmc_step()
            ex = o.export()
            rm, _tot = o.rates_matrix()
            st = dict(ex, rm=rm)
            lat, as1, as2, ns, rm2, dirty = emu.event(proc, site, st)
            o.run_proc_nr(proc, site)
            ex2 = o.export()
            rm_o, _ = o.rates_matrix()
            np.testing.assert_array_equal(lat, ex2["lattice"])
            np.testing.assert_array_equal(as1, ex2["as1"])
            np.testing.assert_array_equal(as2, ex2["as2"])
            np.testing.assert_array_equal(ns, ex2["nsites"])
            np.testing.assert_array_equal(rm2, rm_o)
            # running sums from the first changed entry on == the full re-sum
            o.update_accum_rate()
            _r, full = o.rates_matrix()
            for q in range(o.P):
                n = int(ns[q])
                s = 0.0
                pm = []
                for i in range(1, n + 1):
                    s = s + rm2[q, i]
                    pm.append(s)
                lo = dirty[q]
                # entries before the first changed one keep their old running sums
                old = []
                s = 0.0
                for i in range(1, int(ex["nsites"][q]) + 1):
                    s = s + st["rm"][q, i]
                    old.append(s)
                for i in range(1, min(lo, n + 1)):
                    assert pm[i - 1] == old[i - 1], (q, i, lo)
                assert (pm[-1] if n else 0.0) == full[q]
            checked += 1
    assert checked == 60


def test_constant_rate_running_sums_are_one_table():
    """The identity behind the otf kernel's constant-rate sums (otf_uniform_kernel): for
    every process whose rate program reads no bystander count, after
    recalculate_rates_matrix and any number of steps every entry of its list holds the same
    rate c, and the oracle's total of the list (update_accum_rate's left-to-right sum) is
    F(n), F(i) = F(i-1) + c from F(0) = 0 -- the same for every trajectory.  Checked on the
    oracle's intZGB trajectories, including through a rate change followed by
    recalculate_rates_matrix."""
    m = fixture_model("intZGB_otf")
    prog = PG.compile_model(m, "otf")
    w = np.asarray(prog.words)
    off_rate = int(w[22])
    const = [p for p in range(int(w[3])) if int(w[int(w[off_rate + p]) + 1]) == 0]
    assert len(const) == 3   # CO and the two O2 desorption directions
    rates = [0.4, 0.05, 0.1, 0.1, 0.1, 0.1, 0.02, 0.02, 0.3, 0.3]
    params = [1.3, 0.7, 1.9, 1e-10, 0.5]
    for traj in (0, 3):
        o = O.Oracle(prog, (24, 20), seed=11, rng=O.RNG_PHILOX, traj=traj)
        o.set_rates(rates)
        o.set_user_parameters(params)
        o.recalculate_rates_matrix()
        o.update_accum_rate()
        for block, change in ((3000, False), (2000, True), (2000, False)):
            if change:
                o.set_rates([r * 1.7 for r in rates])
                o.recalculate_rates_matrix()
            o.do_kmc_steps(block)
            o.update_accum_rate()
            rm, tot = o.rates_matrix()
            ns = o.export()["nsites"]
            for p in const:
                n = int(ns[p])
                row = rm[p, 1:n + 1]
                if n == 0:
                    assert tot[p] == 0.0
                    continue
                c = row[0]
                assert (row == c).all()
                f = 0.0
                for _ in range(n):
                    f = f + c
                assert tot[p] == f


def _bisect(arr, size, value):
    """interval_search_real as kmc_otf.cu's interval_search runs it (lane 0)."""
    left, right = 1, size
    while True:
        mid = (right + left) >> 1
        if left >= right:
            break
        if value < arr[mid]:
            right = mid
        else:
            left = mid + 1
    if arr[mid] == 0.0:
        while True:
            if arr[mid] > 0.0:
                break
            if mid >= size:
                return 0
            mid += 1
    while mid != 1 and arr[mid - 1] >= arr[mid]:
        mid -= 1
    return mid


def _warp_search(arr, size, value):
    """kmc_otf.cu's interval_search_warp, the 32 lanes emulated."""
    lo, hi = 1, size
    while lo < hi:
        step = (hi - lo + 32) >> 5
        t = [(lo + lane * step >= hi) or (value < arr[lo + lane * step]) for lane in range(32)]
        if not any(t):
            lo += 31 * step + 1
            continue
        j = t.index(True)
        if j == 0:
            hi = lo
            break
        pj = lo + j * step
        lo = lo + (j - 1) * step + 1
        hi = min(pj, hi)
    mid = lo
    if arr[mid] == 0.0:
        while True:
            if arr[mid] > 0.0:
                break
            if mid >= size:
                return 0
            mid += 1
    while mid != 1 and arr[mid - 1] >= arr[mid]:
        mid -= 1
    return mid


def test_warp_entry_search_equals_the_bisection():
    """The otf kernel's warp-parallel entry search returns the bisection's index on running
    sums of non-negative rates: random lists of every size class around the 32-way round
    boundaries, with zeros, plateaus, one positive entry, constant rates, and values at 0,
    inside, at and past the total."""
    rng = np.random.default_rng(1)
    for _ in range(3000):
        size = int(rng.choice([1, 2, 3, 31, 32, 33, 63, 64, 65, 1023, 1024, 1025, 1057, 5000]))
        kind = int(rng.integers(0, 4))
        if kind == 0:
            r = rng.uniform(0, 1, size)
        elif kind == 1:
            r = rng.choice([0.0, 0.5, 1.0], size)
        elif kind == 2:
            r = np.zeros(size)
            r[rng.integers(0, size)] = 1.0
        else:
            r = np.full(size, 0.02)
        arr = np.concatenate([[0.0], np.cumsum(r)])
        tot = arr[size]
        for value in (rng.uniform(0, tot) if tot > 0 else 0.0, 0.0, tot, rng.uniform(0, 2 * tot + 1)):
            assert _warp_search(arr, size, value) == _bisect(arr, size, value)
