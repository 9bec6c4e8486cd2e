"""Fast streams (the step kernel's gather / evaluate / replay form of a process stream)
and the engine's program check, on the CPU.

* Every fixture model compiles, under both backends and the four benchmark models, to
  a program the engine accepts: ``kmc_check_program`` runs the check kmc_create and
  kmc_pool_add_model run before a program reaches the device.  Corrupted programs
  (a stream off its 16-byte placement, a reference outside the stream's slots, a
  table index outside its table, a stray unused reference) are refused.
* Table-form nli edits (packed references, constant references folded into the index
  base) pick the same process as the member scan of the group record (the nli_<G>
  functions, kmos/io/__init__.py:1497-2057) for random slot species, edit by edit:
  the program compiled with nli tables against the same model compiled without.
"""
import numpy as np
import pytest

from conftest import fixture_model, trimer_model
from kmos_gb300 import configs, engine as E, program as PG

MODELS = ["AB_model", "CO_oxidation_Ruo2", "ZGB_model", "default_xml", "pairwise_interaction", "pdopd_xml"]


def streams(words):
    """(process, stream offset, nlat, [(quad 0, packed references)] per edit, hot)."""
    w = [int(x) for x in words]
    P, off_hot, hot_len = w[3], w[21], w[20]
    hot = w[off_hot:off_hot + hot_len]
    out = []
    for p in range(P):
        off = hot[p]
        if off == 0:
            continue
        nlat, nchk, nwr, x = hot[off:off + 4]
        nedit, nq = x & 0xFFFF, (x >> 16) & 0xF
        rec = off + ((4 + nlat + 2 * nchk + 2 * nwr + 3) & ~3)
        edits = []
        for k in range(nedit):
            q0 = hot[rec + 4 * k:rec + 4 * k + 4]
            refs = [hot[rec + 4 * ((1 + c // 4) * nedit + k) + c % 4] for c in range(4 * nq)]
            edits.append((q0, refs))
        out.append((p, off, nlat, edits, hot))
    return out


def code(s, ns):
    return ns if s < 0 or s > ns else s


def by_table(q0, refs, latv, hot, ns):
    idx = q0[2] + sum(code(latv[r & 0xFF], ns) * (r >> 8) for r in refs)
    return hot[idx]


def by_scan(off, q0, latv, hot):
    e = off + q0[2]
    cnt = (hot[e] >> 8) & 0xFF
    rec = hot[e + 3]
    refs = hot[e + 4:e + 4 + cnt]
    M, K = hot[rec], hot[rec + 1]
    vals = [latv[r] if r >= 0 else -r - 2 for r in refs]
    result = 0
    for m in range(M):
        mem = hot[rec + 2 + K + m * (1 + K):rec + 2 + K + (m + 1) * (1 + K)]
        if all((mem[1 + k] & 0xFFFFFFFF) >> (31 if v < 0 else v) & 1 for k, v in enumerate(vals)):
            result = mem[0]
    return result


def compiled(name, backend, tables=True, monkeypatch=None):
    if not tables:
        monkeypatch.setattr(PG, "NLI_TABLE_MAX", 0)
    prog = PG.compile_model(trimer_model() if name == "trimer" else fixture_model(name), backend)
    if not tables:
        monkeypatch.undo()
    return prog


@pytest.mark.parametrize("name", MODELS)
@pytest.mark.parametrize("backend", ["local_smart", "lat_int"])
def test_programs_pass_the_engine_check(name, backend):
    prog = PG.compile_model(fixture_model(name), backend)
    E.check_program(prog)
    w = prog.words
    assert w[21] % 4 == 0
    for _p, off, *_ in streams(w):
        assert off % 4 == 0


@pytest.mark.parametrize("backend", ["local_smart", "lat_int"])
def test_trimer_programs_pass_the_engine_check(backend, monkeypatch):
    E.check_program(compiled("trimer", backend))
    E.check_program(compiled("trimer", backend, tables=False, monkeypatch=monkeypatch))


@pytest.mark.parametrize("config", [1, 2, 3, 4])
def test_benchmark_programs_pass_the_engine_check(config):
    E.check_program(configs.build(config, n=1, steps=0).program)


@pytest.mark.parametrize("name", ["CO_oxidation_Ruo2", "ZGB_model", "pairwise_interaction", "pdopd_xml",
                                  "default_xml", "trimer"])
def test_table_edits_equal_member_scans(name, monkeypatch):
    a = compiled(name, "lat_int")
    b = compiled(name, "lat_int", tables=False, monkeypatch=monkeypatch)
    E.check_program(b)
    ns = int(a.words[4])
    sa, sb = streams(a.words), streams(b.words)
    assert [s[0] for s in sa] == [s[0] for s in sb]
    rng = np.random.default_rng(7)
    checked = 0
    for (p, offa, nlat, ea, hota), (_p, offb, nlatb, eb, hotb) in zip(sa, sb):
        assert nlat == nlatb and len(ea) == len(eb)
        for _ in range(40):
            latv = [int(v) for v in rng.integers(-1, ns, size=nlat)]
            for (qa, ra), (qb, _rb) in zip(ea, eb):
                opa, opb = qa[0] & 0xFF, qb[0] & 0xFF
                assert qa[1] == qb[1]  # same target slot
                if opa < 6:
                    assert opa == opb
                    continue
                assert opb == opa - 2  # table del / add against scan del / add
                assert by_table(qa, ra, latv, hota, ns) == by_scan(offb, qb, latv, hotb)
                checked += 1
    assert checked > 100


def _first_table_edit(words):
    for p, off, nlat, edits, hot in streams(words):
        for k, (q0, refs) in enumerate(edits):
            if q0[0] & 0xFF >= 6 and refs:
                return p, off, nlat, k, q0, refs, len(edits)
    raise AssertionError("no table edit")


def test_corrupted_programs_are_refused():
    prog = PG.compile_model(fixture_model("pairwise_interaction"), "lat_int")
    w0 = np.array(prog.words, dtype=np.int32)
    E.check_program(w0)
    off_hot = int(w0[21])
    p, off, nlat, k, q0, refs, nedit = _first_table_edit(w0)
    hot = w0[off_hot:]
    nchk, nwr = int(hot[off + 1]), int(hot[off + 2])
    rec = off + ((4 + nlat + 2 * nchk + 2 * nwr + 3) & ~3)
    ref_at = off_hot + rec + 4 * (nedit + k)  # first packed reference of edit k

    def refused(mutate, what):
        w = w0.copy()
        mutate(w)
        with pytest.raises(E.KMCError) as e:
            E.check_program(w)
        assert e.value.code == 5, what

    refused(lambda w: w.__setitem__(off_hot + p, off + 1), "stream off its 16-byte placement")
    refused(lambda w: w.__setitem__(ref_at, (w[ref_at] & ~0xFF) | 127), "reference outside the slots")
    refused(lambda w: w.__setitem__(off_hot + rec + 4 * k + 2, 1 << 20), "index base outside the table")
    refused(lambda w: w.__setitem__(off_hot + rec + 4 * k + 1, nlat), "target outside the slots")
    cnt = (int(q0[0]) >> 8) & 0xFF
    if cnt < len(refs):
        at = off_hot + rec + 4 * ((1 + cnt // 4) * nedit + k) + cnt % 4
        refused(lambda w: w.__setitem__(at, 1), "unused reference not zero")

    def shift_hot(w):
        w[21] += 1
        w[20] -= 1

    refused(shift_hot, "hot section off 16 bytes")


def test_inline_add_conditions():
    """Adds with at most one condition carry it in their first quad: [h, target, slot,
    mask]; a slot outside the stream's slots is refused."""
    prog = PG.compile_model(fixture_model("ZGB_model"), "local_smart")
    w0 = np.array(prog.words, dtype=np.int32)
    off_hot = int(w0[21])
    found = 0
    for p, off, nlat, edits, hot in streams(w0):
        nchk, nwr = hot[off + 1], hot[off + 2]
        rec = off + ((4 + nlat + 2 * nchk + 2 * nwr + 3) & ~3)
        for k, (q0, _refs) in enumerate(edits):
            op, cnt = q0[0] & 0xFF, (q0[0] >> 8) & 0xFF
            if op != 3 or cnt > 1:
                continue
            assert 0 <= q0[2] < nlat
            if cnt == 0:
                assert q0[2] == 0 and q0[3] == 0
                continue
            found += 1
            w = w0.copy()
            w[off_hot + rec + 4 * k + 2] = nlat
            with pytest.raises(E.KMCError):
                E.check_program(w)
    assert found > 0


def test_dels_first_streams():
    """Streams whose del-kind edits all precede their add-kind edits, with no two adds
    and no two dels naming one (process, site), carry the dels-first flag (every lat_int stream does; the
    engine appends their adds in parallel after the dels); setting it on any other
    stream is refused."""
    for name in ("ZGB_model", "CO_oxidation_Ruo2", "pairwise_interaction"):
        lat = PG.compile_model(fixture_model(name), "lat_int")
        w = [int(x) for x in lat.words]
        hot = w[w[21]:w[21] + w[20]]
        assert all((hot[hot[p] + 3] >> 20) & 1 for p in range(w[3]) if hot[p])
    prog = PG.compile_model(fixture_model("ZGB_model"), "local_smart")
    w0 = np.array(prog.words, dtype=np.int32)
    off_hot = int(w0[21])
    refused = 0
    for p, off, nlat, edits, hot in streams(w0):
        flag = (hot[off + 3] >> 20) & 1
        kinds = [q0[0] & 0xFF for q0, _ in edits]
        dels = [i for i, k in enumerate(kinds) if k in (2, 4, 6)]
        adds = [i for i, k in enumerate(kinds) if k in (3, 5, 7)]
        keys = [(edits[i][0][0] >> 16, edits[i][0][1]) for i in adds]
        dkeys = [(edits[i][0][0] >> 16, edits[i][0][1]) for i in dels]
        ordered = not dels or not adds or max(dels) < min(adds)
        assert flag == int(ordered and len(set(keys)) == len(keys) and len(set(dkeys)) == len(dkeys))
        if not flag:
            w = w0.copy()
            w[off_hot + off + 3] |= 1 << 20
            with pytest.raises(E.KMCError):
                E.check_program(w)
            refused += 1
    assert refused > 0
