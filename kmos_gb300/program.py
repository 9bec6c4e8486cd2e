"""Compile a :class:`~kmos_gb300.model.Model` into the engine's *op program*.

kmos turns a model into generated Fortran (``proclist.f90`` for local_smart;
``run_proc_*.f90`` + ``nli_*.f90`` for lat_int).  The order of the book-keeping edits
in that code is observable: ``del_proc`` is a swap-remove (base.mpy:211-265), so the
order of every ``add_proc``/``del_proc`` decides which site the next uniform pick
returns.  This module produces the same edit sequences, in the same order, as a flat
int32 program that the CUDA engine (and the CPU oracle) interpret.

local_smart (kmos/io/__init__.py:305-465, 2219-2655):
  * ``run_proc_nr`` calls put/take/create/annihilate routines, one per action, in
    action order, at coordinates relative to the process's executing coordinate.
  * each routine is ``replace_species``; then guarded ``del_proc`` for every
    (process, condition) pair it disables, in process x condition order; then the
    ``add_proc`` if-tree built by ``_write_optimal_iftree``.  The if-tree is flattened
    here into its depth-first leaf order; at run time each leaf is added when all its
    conditions hold, which is exactly the set and order of adds the tree executes.
  * routine calls are inlined with their offsets composed, so one process becomes one
    straight op list.

lat_int (kmos/io/__init__.py:1497-2057):
  * processes are grouped into lateral-interaction groups (``_get_lat_int_groups``);
  * ``run_proc_<group>``: ``del_proc(nli_G(cell+o), cell+o+(0,0,0,1))`` for every
    modified (group, offset) in sorted ``"name offset"`` order, then the lattice
    writes, then ``add_proc`` for the same list;
  * ``nli_<group>`` is a pure function: the member whose conditions and bystanders all
    match the lattice, or 0.

Program layout (all int32; see ``include/kmc_gb300.h`` for the authoritative table)::

    [0] magic  [1] version  [2] backend  [3] nproc  [4] nspecies  [5] null_species
    [6] spuck  [7] dimension [8] ngroups [9] nlayers
    [10] off_proc_ops   -> nproc+1 offsets (op stream of process p = [off[p-1], off[p]))
    [11] off_touchup    -> spuck+1 offsets (touch-up stream of site n), lat_int: 2
    [12] off_groups     -> ngroups offsets to group records
    [13] off_site_layer -> spuck layer ids
    [14] off_site_default -> spuck default species ids
    [15] total length
    [16] max ops executed by one process (sizing hint)
    [17] hot-relative offset of the group-record offsets (ngroups entries)
    [18] hot-relative offset of the nli-table offsets (ngroups entries, 0 = none)
    [19] reach          -> largest |dx|, |dy|, |dz| of the fast streams, one byte each
    [20] hot section length, [21] off_hot (the hot section starts with the nproc+1
         hot-relative fast-stream offsets; 0 = no fast stream for that process)

Ops (first word: op | count << 8 | arg << 16; coordinates packed as four signed
bytes dx, dy, dz, n with n the absolute 1-based site index)::

    OP_REPLACE  [h, coord, old_species_mask, new_species]
    OP_GDEL     [h(arg=proc), coord]            if can_do(proc, site): del_proc
    OP_ADD      [h(count=k, arg=proc), coord, (coord, mask) * k]
    OP_LI_DEL   [h(arg=group), coord]           del_proc(nli_group(base+o), base+o, n=1)
    OP_LI_ADD   [h(arg=group), coord]           add_proc(nli_group(base+o), base+o, n=1)
    OP_STRIP    [h, coord]                      del every process available at site

Group record: ``[nmembers M, ncoords K, coord * K, (proc, mask * K) * M]``.
Species masks have bit ``s`` for species ``s`` and bit 31 for the null species -1.

Fast streams and the hot section (header words 17-22).  For the engine's gather /
evaluate / replay / scatter step every process stream is also emitted in a resolved
form.  The stream lists the distinct lattice coordinates it can touch (relative to the
base cell, every nli coordinate shifted by its op offset) as *slots*.  Because
``replace_species`` writes a constant species, the value any later read of a replaced
slot sees is known here: conditions on replaced slots are decided at compile time (an
add that can never fire is dropped), and every remaining read is of the value the slot
had before the step.  All edits of a step can therefore be evaluated in parallel::

    [nlat, nchk, nwr, nedit | nq << 16 | dels_first << 20, coord * nlat, (slot, old_mask) * nchk,
     (slot, species) * nwr, 0 * (pad to 4 words), quad 0 * nedit, ..., quad nq * nedit,
     variable parts...]
    quad 0 of edit k  [kind | cnt << 8 | arg << 16, target slot, x, 0]
    quad q >= 1       packed table references 4q-4 .. 4q-1 of edit k (slot | mul << 8)
    kind  2 = guarded del (arg = proc; x = 0)
          3 = add (arg = proc, cnt conditions): with at most one condition the quad
              holds it, [h, target slot, slot, mask] ([h, target slot, 0, 0] for none);
              else x = offset of its variable part [h, target slot, ref * cnt, mask * cnt]
          4 = nli del, 5 = nli add through a member scan (arg = group, cnt = the group's
              K; x = offset of [h, target slot, 0, record offset, ref * cnt], the record
              offset hot-relative)
          6 = nli del, 7 = nli add through a table (arg = group, cnt = its non-constant
              references; x = index base): the table entry is x + sum(code(slot_c) *
              mul_c) over the packed references, the constant references and the
              table's own offset folded into x; unused references are 0 (slot 0 times 0)
    ref   >= 0: slot index (value before the step); < 0: constant species -ref-2
    Every edit's target coordinate is a slot, so its site is gathered with the others.
    Edit k's quads lie nedit quads apart (lane k of a warp reads edit k: consecutive
    16-byte loads), and the stream, its quads and the hot section start on 16 bytes.
    dels_first = 1: every del-kind edit (2, 4, 6) comes before every add-kind edit (3, 5,
    7), and no two adds, nor two dels, can name the same (process, site) (distinct
    (proc, target) for kinds 2 and 3, distinct (group, target) for kinds 4-7, not both
    forms among the adds or among the dels): true of every lat_int stream.  The engine's
    replay then reads back only what the dels move, and logs nothing else.

``chk`` are the old-species checks of first replaces (later ones are checked here),
``wr`` the final species of every replaced slot.  Offsets of variable parts are
relative to the stream start.  The hot section (header word 21) holds the fast-stream offset table,
the streams, the group records and the nli tables with offsets relative to its own
start, so a block can copy it to shared memory in one piece.  Header word 19 is the
largest |offset| any fast stream reaches per axis: a lattice at least 2*reach+1 cells
wide keeps all slots distinct sites, which the fast path requires.

nli tables (in the hot section): for a group of K coordinates over ns species, a table of
(ns+1)^K process ids indexed by sum(code_k * (ns+1)^k), code = species or ns for the
null species; 0 when it would exceed 4096 entries (the engine then scans members).
"""
from __future__ import annotations

import functools
from dataclasses import dataclass
from typing import Dict, List, Sequence, Tuple

import numpy as np

from .model import Condition, Coord, Model, Process

MAGIC = 0x4B4D4331
VERSION = 1
BACKENDS = {"local_smart": 0, "lat_int": 1, "otf": 2}

OP_END = 0
OP_REPLACE = 1
OP_GDEL = 2
OP_ADD = 3
OP_LI_DEL = 4
OP_LI_ADD = 5
OP_STRIP = 6
OP_UPDATE = 7   # otf: if can_do(proc, site): update_rates_matrix with the rate re-evaluated

HEADER_WORDS = 24
FAST_MAX_SLOTS = 128
FAST_MAX_EDITS = 128
NLI_TABLE_MAX = 4096


def species_bit(sid: int) -> int:
    return 1 << (31 if sid < 0 else sid)


def mask_to_int32(mask: int) -> int:
    mask &= 0xFFFFFFFF
    return mask - (1 << 32) if mask & 0x80000000 else mask


def pack_coord(dx: int, dy: int, dz: int, n: int) -> int:
    for d in (dx, dy, dz):
        if not -128 <= d <= 127:
            raise ValueError("process offset %d out of the packed range" % d)
    if not 0 <= n <= 255:
        raise ValueError("site index %d out of the packed range" % n)
    w = (dx & 0xFF) | ((dy & 0xFF) << 8) | ((dz & 0xFF) << 16) | ((n & 0xFF) << 24)
    return w - (1 << 32) if w & 0x80000000 else w


def unpack_coord(w: int) -> Tuple[int, int, int, int]:
    w &= 0xFFFFFFFF

    def s8(v):
        return v - 256 if v & 0x80 else v

    return s8(w & 0xFF), s8((w >> 8) & 0xFF), s8((w >> 16) & 0xFF), (w >> 24) & 0xFF


def op_header(op: int, count: int = 0, arg: int = 0) -> int:
    if not 0 <= count <= 255 or not 0 <= arg <= 0x7FFF:
        raise ValueError("op field out of range")
    return op | (count << 8) | (arg << 16)


# ---- relative coordinates ---------------------------------------------------------
# A relative coordinate (dx, dy, dz, n): offset in unit cells from a base cell and the
# absolute site index n.  kmos writes these as "site + (/dx, dy, dz, A - B/)" strings;
# two such strings are equal exactly when (dx, dy, dz, n) are equal, which is what the
# if-tree construction compares.
RelCoord = Tuple[int, int, int, int]


def _sub(a: Coord, b: Coord, site_ids) -> RelCoord:
    """kmos ``Coord.__sub__`` (kmos/types.py:1867-1888) applied to a base whose site
    index is ``b``'s: the offset difference and the absolute index of ``a``'s site."""
    return (a.offset[0] - b.offset[0], a.offset[1] - b.offset[1], a.offset[2] - b.offset[2],
            site_ids[(a.layer, a.name)])


@dataclass
class AddItem:
    """One ``add_proc`` leaf: ``proc`` at ``target`` when every ``(coord, species)``
    condition holds."""

    conds: Tuple[Tuple[RelCoord, str], ...]
    proc: int
    target: RelCoord


def _most_common(coords: Sequence[RelCoord]) -> RelCoord:
    """kmos ``_most_common`` (kmos/io/__init__.py:98-115): the most frequent item,
    the earliest-seen one on ties."""
    counts: Dict[RelCoord, int] = {}
    first: Dict[RelCoord, int] = {}
    for i, c in enumerate(coords):
        counts[c] = counts.get(c, 0) + 1
        first.setdefault(c, i)
    return max(counts, key=lambda c: (counts[c], -first[c]))


def flatten_iftree(items: List[Tuple[Tuple[Tuple[RelCoord, str], ...], AddItem]]) -> List[AddItem]:
    """Depth-first leaf order of the tree ``_write_optimal_iftree`` builds
    (kmos/io/__init__.py:2568-2655).  ``items`` pairs each leaf's *remaining*
    conditions with the leaf itself (which keeps all of its conditions)."""
    out = [leaf for conds, leaf in items if not conds]
    items = [(conds, leaf) for conds, leaf in items if conds]
    if not items:
        return out
    mc = _most_common([c for conds, _ in items for c, _s in conds])
    answers = sorted({s for conds, _ in items for c, s in conds if c == mc})
    for answer in answers:
        nested = [it for it in items
                  if any(c == mc for c, _ in it[0])
                  and next(s for c, s in it[0] if c == mc) == answer]
        pruned = [(tuple((c, s) for c, s in conds if c != mc), leaf) for conds, leaf in nested]
        nested_ids = {id(it) for it in nested}
        items = [it for it in items if id(it) not in nested_ids]
        out.extend(flatten_iftree(pruned))
    if items:
        out.extend(flatten_iftree(items))
    return out


# ---- the program builder ------------------------------------------------------------
class _Writer:
    def __init__(self):
        self.words: List[int] = []

    def emit(self, *ws):
        self.words.extend(int(w) for w in ws)


def _rel_add(base: RelCoord, d: RelCoord) -> RelCoord:
    return (base[0] + d[0], base[1] + d[1], base[2] + d[2], d[3])


class ProgramBuilder:
    def __init__(self, model: Model, backend: str):
        if backend not in BACKENDS:
            raise ValueError("unknown backend %r" % backend)
        self.model = model
        self.backend = backend
        self.sid = model.species_ids()
        self.site_ids = model.site_ids()
        self.pid = model.process_ids()
        self.null = model.null_species()
        self.default = model.default_species
        if len(model.species) + (0 if self.null < 0 else 1) > 31:
            raise ValueError("at most 30 species are supported")

    # species helpers
    def species_id(self, name: str) -> int:
        name = name.strip()
        if name in ("null_species",):
            return self.null
        if name == "default_species":
            name = self.default
        return self.sid[name]

    def mask_of(self, names: str) -> int:
        m = 0
        for part in names.split(" or "):
            m |= species_bit(self.species_id(part))
        return mask_to_int32(m)

    # ---------------------------------------------------------------------------
    # local_smart
    # ---------------------------------------------------------------------------
    def _routine_ops(self, kind: str, species: str, layer: str, site: str) -> List[tuple]:
        """Ops of one put/take/create/annihilate routine, relative to its site
        (kmos/io/__init__.py:2219-2409, 2445-2560)."""
        m = self.model
        ops: List[tuple] = []
        enabled: List[Tuple[Tuple[Tuple[RelCoord, str], ...], AddItem]] = []
        disabled: List[Tuple[int, RelCoord]] = []
        n_site = self.site_ids[(layer, site)]
        if kind == "put":
            ops.append(("replace", (0, 0, 0, n_site), self.mask_of(self.default), self.species_id(species)))
        elif kind == "take":
            ops.append(("replace", (0, 0, 0, n_site), self.mask_of(species), self.species_id(self.default)))
        elif kind == "create":
            ops.append(("replace", (0, 0, 0, n_site), mask_to_int32(species_bit(self.null)), self.species_id(species)))
        elif kind == "annihilate":
            ops.append(("replace", (0, 0, 0, n_site), self.mask_of(species), self.null))
        for proc in m.processes:
            exe = proc.executing_coord()
            for cond in proc.conditions:
                if not (cond.coord.name == site and cond.coord.layer == layer):
                    continue
                if kind in ("put", "take"):
                    enables = (kind == "put" and species == cond.species) or \
                              (kind == "take" and cond.species == self.default)
                    disables = (kind == "put" and cond.species == self.default) or \
                               (kind == "take" and species == cond.species)
                    others = [o for o in proc.conditions if o.coord != cond.coord]
                else:
                    enables = kind == "create"
                    disables = kind == "annihilate"
                    others = list(proc.conditions)
                if enables:
                    conds = tuple((_sub(o.coord, cond.coord, self.site_ids), o.species) for o in others)
                    leaf = AddItem(conds, self.pid[proc.name], _sub(exe, cond.coord, self.site_ids))
                    enabled.append((conds, leaf))
                elif disables:
                    disabled.append((self.pid[proc.name], _sub(exe, cond.coord, self.site_ids)))
        for p, coord in disabled:
            ops.append(("gdel", p, coord))
        for leaf in flatten_iftree(enabled):
            ops.append(("add", leaf.proc, leaf.target, leaf.conds))
        return ops

    def _process_calls(self, proc: Process) -> List[Tuple[str, str, str, str, RelCoord]]:
        """The routine calls of ``run_proc_nr`` for one process
        (kmos/io/__init__.py:305-465): (kind, species, layer, site, base offset)."""
        exe = proc.executing_coord()
        calls = []
        for action in proc.actions:
            rel = _sub(action.coord, exe, self.site_ids)
            prev = [c for c in proc.conditions if c.coord == action.coord]
            previous = prev[0].species if prev else None
            a = action.species
            lay, nm = action.coord.layer, action.coord.name
            if a.startswith("^"):
                calls.append(("create", a[1:], lay, nm, rel))
            elif a.startswith("$"):
                calls.append(("annihilate", a[1:], lay, nm, rel))
            elif a == self.default and a != previous:
                if previous is None:
                    raise ValueError("process %s: action without a condition on the same site" % proc.name)
                calls.append(("take", previous, lay, nm, rel))
            elif previous != a:
                if previous is None:
                    raise ValueError("process %s: action without a condition on the same site" % proc.name)
                if previous != self.default:
                    calls.append(("take", previous, lay, nm, rel))
                calls.append(("put", a, lay, nm, rel))
        return calls

    def _touchup_ops(self, layer: str, site: str) -> List[tuple]:
        """``touchup_<layer>_<site>`` (kmos/io/__init__.py:2411-2443)."""
        n_site = self.site_ids[(layer, site)]
        ops: List[tuple] = [("strip", (0, 0, 0, n_site))]
        items = []
        for proc in self.model.processes:
            exe = proc.executing_coord()
            if exe.layer == layer and exe.name == site:
                conds = tuple((_sub(c.coord, exe, self.site_ids), c.species) for c in proc.conditions)
                items.append((conds, AddItem(conds, self.pid[proc.name], (0, 0, 0, n_site))))
        for leaf in flatten_iftree(items):
            ops.append(("add", leaf.proc, leaf.target, leaf.conds))
        return ops

    @staticmethod
    def _shift(ops: List[tuple], base: RelCoord) -> List[tuple]:
        out = []
        for op in ops:
            if op[0] == "replace":
                out.append(("replace", _rel_add(base, op[1]), op[2], op[3]))
            elif op[0] == "gdel":
                out.append(("gdel", op[1], _rel_add(base, op[2])))
            elif op[0] == "add":
                out.append(("add", op[1], _rel_add(base, op[2]),
                            tuple((_rel_add(base, c), s) for c, s in op[3])))
            else:
                raise AssertionError(op)
        return out

    def local_smart_streams(self):
        routines: Dict[tuple, List[tuple]] = {}
        proc_streams = []
        for proc in self.model.processes:
            stream: List[tuple] = []
            for kind, sp, lay, nm, rel in self._process_calls(proc):
                key = (kind, sp, lay, nm)
                if key not in routines:
                    routines[key] = self._routine_ops(kind, sp, lay, nm)
                stream.extend(self._shift(routines[key], rel))
            proc_streams.append(stream)
        touch_streams = [self._touchup_ops(ln, s.name) for ln, s in self.model.site_list()]
        return proc_streams, touch_streams

    # ---------------------------------------------------------------------------
    # lat_int
    # ---------------------------------------------------------------------------
    def lat_int_groups(self):
        """kmos ``_get_lat_int_groups`` (kmos/io/__init__.py:1497-1624).  Returns an
        ordered list of (group name, [members]) where each member is a dict with the
        process, its true conditions, true actions and bystanders."""
        singles = []
        for proc in self.model.processes:
            true_c, true_a, bystanders = [], [], []
            for cond in proc.conditions:
                corr = [a for a in proc.actions if a.coord == cond.coord]
                if corr:
                    if cond.species != corr[0].species:
                        true_c.append(cond)
                        true_a.append(corr[0])
                    else:
                        bystanders.append(cond)
                else:
                    bystanders.append(cond)
            for a in proc.actions:
                if a not in true_a and (a.species.startswith("^") or a.species.startswith("$")):
                    true_a.append(a)
            singles.append(dict(proc=proc, conds=true_c, actions=true_a, bystanders=bystanders))

        def by_cell(items):
            # cmp_coords (kmos/types.py:1950-1963): layer, then offset; the site name is
            # not compared, and Python's sort is stable.
            return sorted(items, key=lambda c: (c.coord.layer, c.coord.offset))

        groups: List[Tuple[str, list]] = []
        for s in singles:
            for _name, members in groups:
                p0 = members[0]
                if by_cell(p0["conds"]) != by_cell(s["conds"]):
                    continue
                if by_cell(p0["actions"]) != by_cell(s["actions"]):
                    continue
                if [c.coord for c in by_cell(p0["bystanders"])] != [c.coord for c in by_cell(s["bystanders"])]:
                    continue
                members.append(s)
                break
            else:
                groups.append((s["proc"].name, [s]))
        return groups

    def lat_int_streams(self):
        groups = self.lat_int_groups()
        gindex = {name: i for i, (name, _m) in enumerate(groups)}
        group_streams = []
        for gname, members in groups:
            p0 = members[0]
            modified = set()
            for action in p0["actions"]:
                for oname, others in groups:
                    rep = others[0]
                    for cond in rep["conds"] + rep["bystanders"]:
                        if action.coord.same_site_type(cond.coord):
                            off = tuple(a - b for a, b in zip(action.coord.offset, cond.coord.offset))
                            modified.add((oname, off))
            # kmos sorts by "%s %s" % (name, str(offset tuple)) (kmos/io/__init__.py:1850-1852)
            modified = sorted(modified, key=lambda x: "%s %s" % (x[0], "(%d, %d, %d)" % x[1]))
            ops: List[tuple] = []
            for oname, off in modified:
                ops.append(("li_del", gindex[oname], (off[0], off[1], off[2], 1)))
            matched = []
            for cond in p0["conds"]:
                action = [a for a in p0["actions"] if a.coord == cond.coord][0]
                matched.append(action)
                if action.species.startswith("$"):
                    old, new = cond.species, "null_species"
                elif action.species.startswith("^"):
                    old, new = "null_species", action.species[1:]
                else:
                    old, new = cond.species, action.species
                c = action.coord
                ops.append(("replace", (c.offset[0], c.offset[1], c.offset[2], self.site_ids[(c.layer, c.name)]),
                            self.mask_of(old), self.species_id(new)))
            for action in p0["actions"]:
                if action in matched:
                    continue
                if action.species.startswith("$"):
                    old, new = action.species[1:], "null_species"
                elif action.species.startswith("^"):
                    old, new = "null_species", action.species[1:]
                else:
                    raise ValueError("unmatched action that is not a multi-lattice action: %s" % (action,))
                c = action.coord
                ops.append(("replace", (c.offset[0], c.offset[1], c.offset[2], self.site_ids[(c.layer, c.name)]),
                            self.mask_of(old), self.species_id(new)))
            for oname, off in modified:
                ops.append(("li_add", gindex[oname], (off[0], off[1], off[2], 1)))
            group_streams.append(ops)
        # nli records (kmos/io/__init__.py:1985-2057)
        records = []
        for gname, members in groups:
            coord_lists = []
            for mem in members:
                conds = [c for c in sorted(mem["conds"] + mem["bystanders"],
                                           key=lambda c: (c.coord.layer, c.coord.offset)) if not c.implicit]
                coord_lists.append(conds)
            ref = [c.coord for c in coord_lists[0]]
            for cl in coord_lists[1:]:
                if [c.coord for c in cl] != ref:
                    raise ValueError("lat_int group %s: members test different coordinates" % gname)
            coords = [(c.offset[0], c.offset[1], c.offset[2], self.site_ids[(c.layer, c.name)]) for c in ref]
            mems = [(self.pid[mem["proc"].name], [self.mask_of(c.species) for c in cl])
                    for mem, cl in zip(members, coord_lists)]
            records.append((coords, mems))
        proc_group = {}
        for gi, (_g, members) in enumerate(groups):
            for mem in members:
                proc_group[self.pid[mem["proc"].name]] = gi
        touch = [("strip", (0, 0, 0, 1))] + [("li_add", gi, (0, 0, 0, 1)) for gi in range(len(groups))]
        return groups, group_streams, records, proc_group, touch

    # ---------------------------------------------------------------------------
    # serialisation
    # ---------------------------------------------------------------------------
    @staticmethod
    def _encode(ops: List[tuple], w: _Writer) -> int:
        """Append an op stream; returns the number of ops."""
        for op in ops:
            kind = op[0]
            if kind == "replace":
                w.emit(op_header(OP_REPLACE), pack_coord(*op[1]), op[2], op[3])
            elif kind == "gdel":
                w.emit(op_header(OP_GDEL, 0, op[1]), pack_coord(*op[2]))
            elif kind == "add":
                conds = op[3]
                w.emit(op_header(OP_ADD, len(conds), op[1]), pack_coord(*op[2]))
                for c, s in conds:
                    w.emit(pack_coord(*c), s)
            elif kind == "li_del":
                w.emit(op_header(OP_LI_DEL, 0, op[1]), pack_coord(*op[2]))
            elif kind == "li_add":
                w.emit(op_header(OP_LI_ADD, 0, op[1]), pack_coord(*op[2]))
            elif kind == "strip":
                w.emit(op_header(OP_STRIP), pack_coord(*op[1]))
            elif kind == "update":
                w.emit(op_header(OP_UPDATE, 0, op[1]), pack_coord(*op[2]))
            else:
                raise AssertionError(kind)
        w.emit(OP_END)
        return len(ops)

    @staticmethod
    def _fast_stream(stream, records, tabled=(), ns=0):
        """Resolved slot form of one process stream (see the module docstring); None
        when it exceeds the on-chip limits.  ``tabled``: groups with an nli table over
        ``ns`` species (their edits take the table form)."""
        slots: Dict[RelCoord, int] = {}

        def slot(c):
            if c not in slots:
                slots[c] = len(slots)
            return slots[c]

        static: Dict[int, int] = {}  # slot -> species written earlier in the stream
        chk: List[Tuple[int, int]] = []
        edits: List[List[int]] = []
        reach = [0, 0, 0]

        def ref(sl):
            return -(static[sl] + 2) if sl in static else sl

        def in_mask(sp, mask):
            return ((mask & 0xFFFFFFFF) >> (31 if sp < 0 else sp)) & 1

        for op in stream:
            kind = op[0]
            if kind == "replace":
                sl = slot(op[1])
                if sl in static:
                    if not in_mask(static[sl], op[2]):
                        raise ValueError("process replaces a species it has just written with another")
                else:
                    chk.append((sl, op[2]))
                static[sl] = op[3]
            elif kind == "gdel":
                edits.append([op_header(2, 0, op[1]), slot(op[2])])
                t = op[2]
                reach = [max(reach[i], abs(t[i])) for i in range(3)]
            elif kind == "add":
                refs, masks, dead = [], [], False
                for c, mk in op[3]:
                    sl = slot(c)
                    if sl in static:
                        if not in_mask(static[sl], mk):
                            dead = True
                        continue
                    refs.append(sl)
                    masks.append(mk)
                t = op[2]
                reach = [max(reach[i], abs(t[i])) for i in range(3)]
                if dead:
                    continue  # this add_proc can never fire after the writes before it
                edits.append([op_header(3, len(refs), op[1]), slot(op[2])] + refs + masks)
            elif kind in ("li_del", "li_add"):
                g, o = op[1], op[2]
                coords, _mems = records[g]
                refs = [ref(slot((o[0] + c[0], o[1] + c[1], o[2] + c[2], c[3]))) for c in coords]
                target = slot(o)
                if g in tabled:
                    # table index = sum(code_k * (ns+1)^k), code = species or ns for null
                    const, vslots, muls = 0, [], []
                    for k, r in enumerate(refs):
                        mul = (ns + 1) ** k
                        if r < 0:
                            sp = -r - 2
                            const += (ns if sp < 0 else sp) * mul
                        else:
                            vslots.append(r)
                            muls.append(mul)
                    # the table offset is added by build()
                    edits.append([op_header(6 if kind == "li_del" else 7, len(vslots), g), target,
                                  ("tabc", g, const)] + vslots + muls)
                else:
                    # the group's record offset is filled in by build()
                    edits.append([op_header(4 if kind == "li_del" else 5, len(coords), g), target,
                                  0, ("rec", g)] + refs)
                reach = [max(reach[i], abs(o[i])) for i in range(3)]
            else:
                return None
        if len(slots) > FAST_MAX_SLOTS or len(edits) > FAST_MAX_EDITS:
            return None
        coords = sorted(slots, key=slots.get)
        for c in coords:
            reach = [max(reach[i], abs(c[i])) for i in range(3)]
        wr = sorted(static.items())
        nedit = len(edits)
        # quads of packed table references: enough for the widest table edit
        nq = max([(e[0] >> 8 & 0xFF) for e in edits if (e[0] & 0xFF) >= 6] + [0])
        nq = (nq + 3) // 4
        if nq > 3:
            return None
        # every del-kind edit before every add-kind edit (lat_int streams: the del list,
        # the writes, the add list): the engine then appends the adds after the dels
        kinds = [e[0] & 0xFF for e in edits]
        dels = [i for i, op in enumerate(kinds) if op in (2, 4, 6)]
        adds = [i for i, op in enumerate(kinds) if op in (3, 5, 7)]
        # and no two adds, nor two dels, can name one (process, site): the appends then
        # commute, and no del reads the position entry another del cleared
        add_keys = [(kinds[i] == 3, edits[i][0] >> 16, edits[i][1]) for i in adds]
        del_keys = [(kinds[i] == 2, edits[i][0] >> 16, edits[i][1]) for i in dels]
        distinct = (len(set(add_keys)) == len(add_keys) and len({k[0] for k in add_keys}) <= 1 and
                    len(set(del_keys)) == len(del_keys) and len({k[0] for k in del_keys}) <= 1)
        dels_first = int(distinct and (not dels or not adds or max(dels) < min(adds)))
        head = [len(coords), len(chk), len(wr), nedit | (nq << 16) | (dels_first << 20)]
        head += [pack_coord(*c) for c in coords]
        for sl, mk in chk:
            head += [sl, mk]
        for sl, sp in wr:
            head += [sl, sp]
        head += [0] * (-len(head) % 4)
        quads = [[0] * (4 * nedit) for _ in range(1 + nq)]
        body: List = []
        body_at = len(head) + 4 * (1 + nq) * nedit
        for k, e in enumerate(edits):
            op, cnt = e[0] & 0xFF, e[0] >> 8 & 0xFF
            if op >= 6:
                x = e[2]
                for c in range(cnt):
                    quads[1 + c // 4][4 * k + c % 4] = e[3 + c] | (e[3 + cnt + c] << 8)
            elif op == 2:
                x = 0
            elif op == 3 and (cnt == 0 or (cnt == 1 and e[2] >= 0)):
                x, w = (e[2], e[3]) if cnt else (0, 0)  # the one condition, inline
                quads[0][4 * k:4 * k + 4] = [e[0], e[1], x, w]
                continue
            else:
                x = body_at + len(body)
                body += e
            quads[0][4 * k:4 * k + 4] = [e[0], e[1], x, 0]
        return head + [w for q in quads for w in q] + body, reach

    def build(self) -> "Program":
        m = self.model
        P = len(m.processes)
        w = _Writer()
        w.emit(*([0] * HEADER_WORDS))
        site_layer = [m.layer_ids()[ln] for ln, _s in m.site_list()]
        site_default = [self.species_id(m.site_default_species(s)) for _ln, s in m.site_list()]
        ngroups = 0
        if self.backend == "otf":
            return self._build_otf(w, site_layer, site_default)
        if self.backend == "local_smart":
            proc_streams, touch_streams = self.local_smart_streams()
            # add conditions carry species names; resolve them to masks
            def resolve(stream):
                out = []
                for op in stream:
                    if op[0] == "add":
                        out.append(("add", op[1], op[2], tuple((c, self.mask_of(s)) for c, s in op[3])))
                    else:
                        out.append(op)
                return out
            proc_streams = [resolve(s) for s in proc_streams]
            touch_streams = [resolve(s) for s in touch_streams]
            records = []
        else:
            groups, group_streams, records, proc_group, touch = self.lat_int_streams()
            ngroups = len(groups)
            proc_streams = [group_streams[proc_group[p]] for p in range(1, P + 1)]
            touch_streams = [touch]
        off_proc = len(w.words)
        w.emit(*([0] * (P + 1)))
        off_touch = len(w.words)
        w.emit(*([0] * (len(touch_streams) + 1)))
        off_groups = len(w.words)
        w.emit(*([0] * max(ngroups, 1)))
        off_site_layer = len(w.words)
        w.emit(*site_layer)
        off_site_default = len(w.words)
        w.emit(*site_default)
        max_ops = 0
        for p, stream in enumerate(proc_streams):
            w.words[off_proc + p] = len(w.words)
            max_ops = max(max_ops, self._encode(stream, w))
        w.words[off_proc + P] = len(w.words)
        for i, stream in enumerate(touch_streams):
            w.words[off_touch + i] = len(w.words)
            self._encode(stream, w)
        w.words[off_touch + len(touch_streams)] = len(w.words)
        for gi, (coords, mems) in enumerate(records):
            w.words[off_groups + gi] = len(w.words)
            w.emit(len(mems), len(coords), *[pack_coord(*c) for c in coords])
            for proc, masks in mems:
                w.emit(proc, *masks)
        # hot section: fast-stream offsets, fast streams, group records, nli tables;
        # offsets inside it are relative to its start
        w.emit(*([0] * (-len(w.words) % 4)))  # the hot section starts on 16 bytes
        off_hot = len(w.words)
        hot: List[int] = [0] * (P + 1)
        reach = [0, 0, 0]
        base = len(m.species) + 1
        tabled = {gi for gi, (coords, _mems) in enumerate(records) if base ** len(coords) <= NLI_TABLE_MAX}
        for p, stream in enumerate(proc_streams):
            fast = self._fast_stream(stream, records, tabled, len(m.species))
            if fast is None:
                continue
            words, rch = fast
            reach = [max(a, b) for a, b in zip(reach, rch)]
            hot.extend([0] * (-len(hot) % 4))  # streams start on 16 bytes
            hot[p] = len(hot)
            hot.extend(words)
        hot[P] = len(hot)
        fixups = [i for i, x in enumerate(hot) if isinstance(x, tuple)]
        grp_off = len(hot)
        hot.extend([0] * max(ngroups, 1))
        tab_off = len(hot)
        hot.extend([0] * max(ngroups, 1))
        for gi, (coords, mems) in enumerate(records):
            hot[grp_off + gi] = len(hot)
            hot.extend([len(mems), len(coords)] + [pack_coord(*c) for c in coords])
            for proc, masks in mems:
                hot.extend([proc] + list(masks))
        for gi, (coords, mems) in enumerate(records):
            K = len(coords)
            if gi not in tabled:
                continue
            table = []
            for idx in range(base ** K):
                codes, r = [], idx
                for _k in range(K):
                    codes.append(r % base)
                    r //= base
                if self.null >= 0:
                    species = codes  # multi-lattice: the null species is ns
                else:
                    species = [c if c < len(m.species) else -1 for c in codes]
                result = 0
                for proc, masks in mems:
                    if all((int(mk) & 0xFFFFFFFF) >> (31 if sp < 0 else sp) & 1 for sp, mk in zip(species, masks)):
                        result = proc
                table.append(result)
            hot[tab_off + gi] = len(hot)
            hot.extend(table)
        for i in fixups:
            what, gi = hot[i][0], hot[i][1]
            hot[i] = hot[tab_off + gi] + hot[i][2] if what == "tabc" else hot[grp_off + gi]
        w.emit(*hot)
        header = [MAGIC, VERSION, BACKENDS[self.backend], P, len(m.species), self.null, m.spuck,
                  m.dimension, ngroups, len(m.layers), off_proc, off_touch, off_groups,
                  off_site_layer, off_site_default, 0, max_ops, grp_off, tab_off,
                  reach[0] | (reach[1] << 8) | (reach[2] << 16), len(hot), off_hot]
        w.words[:len(header)] = header
        w.words[15] = len(w.words)
        arr = np.array([x if x < 2**31 else x - 2**32 for x in w.words], dtype=np.int64).astype(np.int32)
        return Program(self.model, self.backend, arr)


    def _build_otf(self, w: _Writer, site_layer, site_default) -> "Program":
        """Program of the otf backend (kmos_gb300/otf.py): per-process streams, the
        cell touch-up, one rate record per process; no fast streams."""
        from . import otf
        m = self.model
        P = len(m.processes)

        def resolve(stream):
            out = []
            for op in stream:
                if op[0] == "replace":
                    out.append(("replace", op[1], op[2], self.species_id(op[3])))
                elif op[0] == "add":
                    out.append(("add", op[1], op[2], tuple((c, self.mask_of(s)) for c, s in op[3])))
                else:
                    out.append(op)
            return out

        proc_streams = [resolve(otf.process_ops(m, proc, self.site_ids, self.mask_of)) for proc in m.processes]
        touch = resolve(otf.touchup_ops(m, self.site_ids))
        off_proc = len(w.words)
        w.emit(*([0] * (P + 1)))
        off_touch = len(w.words)
        w.emit(0, 0)
        off_groups = len(w.words)
        w.emit(0)
        off_site_layer = len(w.words)
        w.emit(*site_layer)
        off_site_default = len(w.words)
        w.emit(*site_default)
        max_ops = 0
        for p, stream in enumerate(proc_streams):
            w.words[off_proc + p] = len(w.words)
            max_ops = max(max_ops, self._encode(stream, w))
        w.words[off_proc + P] = len(w.words)
        w.words[off_touch] = len(w.words)
        self._encode(touch, w)
        w.words[off_touch + 1] = len(w.words)
        off_rate = len(w.words)
        w.emit(*([0] * (P + 1)))
        for p, proc in enumerate(m.processes):
            w.words[off_rate + p] = len(w.words)
            w.emit(*otf.rate_record(m, proc, self.species_id, self.site_ids))
        w.words[off_rate + P] = len(w.words)
        header = [MAGIC, VERSION, BACKENDS["otf"], P, len(m.species), self.null, m.spuck,
                  m.dimension, 0, len(m.layers), off_proc, off_touch, off_groups,
                  off_site_layer, off_site_default, 0, max_ops, 0, 0, 0, 0, 0,
                  off_rate, len(m.parameters) + len(otf.chempot_names(m))]
        w.words[:len(header)] = header
        w.words[15] = len(w.words)
        arr = np.array([x if x < 2**31 else x - 2**32 for x in w.words], dtype=np.int64).astype(np.int32)
        return Program(self.model, self.backend, arr)


@dataclass
class Program:
    model: Model
    backend: str
    words: np.ndarray  # int32

    @property
    def nproc(self) -> int:
        return int(self.words[3])

    def proc_stream(self, proc: int) -> List[tuple]:
        """Decode the op stream of process ``proc`` (1-based) for inspection."""
        off = int(self.words[10])
        return decode_stream(self.words, int(self.words[off + proc - 1]))

    def touchup_stream(self, i: int) -> List[tuple]:
        off = int(self.words[11])
        return decode_stream(self.words, int(self.words[off + i]))


def decode_stream(words: np.ndarray, pos: int) -> List[tuple]:
    ops = []
    while True:
        h = int(words[pos]) & 0xFFFFFFFF
        op, cnt, arg = h & 0xFF, (h >> 8) & 0xFF, (h >> 16) & 0xFFFF
        if op == OP_END:
            return ops
        if op == OP_REPLACE:
            ops.append(("replace", unpack_coord(int(words[pos + 1])), int(words[pos + 2]), int(words[pos + 3])))
            pos += 4
        elif op == OP_GDEL:
            ops.append(("gdel", arg, unpack_coord(int(words[pos + 1]))))
            pos += 2
        elif op == OP_ADD:
            conds = tuple((unpack_coord(int(words[pos + 2 + 2 * i])), int(words[pos + 3 + 2 * i])) for i in range(cnt))
            ops.append(("add", arg, unpack_coord(int(words[pos + 1])), conds))
            pos += 2 + 2 * cnt
        elif op == OP_LI_DEL:
            ops.append(("li_del", arg, unpack_coord(int(words[pos + 1]))))
            pos += 2
        elif op == OP_LI_ADD:
            ops.append(("li_add", arg, unpack_coord(int(words[pos + 1]))))
            pos += 2
        elif op == OP_STRIP:
            ops.append(("strip", unpack_coord(int(words[pos + 1]))))
            pos += 2
        elif op == OP_UPDATE:
            ops.append(("update", arg, unpack_coord(int(words[pos + 1]))))
            pos += 2
        else:
            raise ValueError("bad op %d at %d" % (op, pos))


def compile_model(model: Model, backend: str = "local_smart") -> Program:
    """Compile ``model`` for ``backend`` ("local_smart" or "lat_int")."""
    return ProgramBuilder(model, backend).build()
