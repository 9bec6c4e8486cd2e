"""Reads the op order out of Fortran that the reference's code generator wrote.

Used by make_golden.py (in a checkout of the reference) to turn generated
``proclist.f90`` (local_smart) and ``proclist.f90`` + ``run_proc_*.f90`` + ``nli_*.f90``
(lat_int) into plain op lists in the decoded form of kmos_gb300.program:

    ("replace", (dx, dy, dz, n), old_species_mask, new_species)
    ("gdel", proc, (dx, dy, dz, n))                 guarded del_proc
    ("add", proc, (dx, dy, dz, n), {((dx,dy,dz,n), mask), ...})
    ("li_del" | "li_add", group, (dx, dy, dz, 1))

Coordinates are relative to the process's base cell with n the absolute site index;
routine calls of run_proc_nr are inlined with their offsets composed.  Each add carries
the conditions of the select-case path that leads to it.  nli functions are returned as
trees that ``eval_nli`` evaluates on a species assignment.

Only the constructs the generator emits are recognised; anything else raises.
"""
import glob
import os
import re

_COORD = re.compile(r"^(l?site|cell)(?:\s*\+\s*\(/(.*)/\))?$")


def _strip(line):
    return line.split("!")[0].strip()


def parse_constants(texts):
    """integer parameters: species, processes, layers and site constants."""
    const = {}
    for text in texts:
        for m in re.finditer(r"integer\(kind=iint\),\s*parameter,\s*public\s*::\s*(\w+)\s*=\s*(-?\d+)", text):
            const[m.group(1).lower()] = int(m.group(2))
    return const


def subroutines(text):
    """name -> list of body lines (continuations joined)."""
    out, cur, name = {}, None, None
    pending = ""
    for raw in text.splitlines():
        line = _strip(raw)
        if pending:
            line = pending + line
            pending = ""
        if line.endswith("&"):
            pending = line[:-1]
            continue
        m = re.match(r"^(?:pure\s+)?(subroutine|function)\s+(\w+)\s*\(", line, re.I)
        if m and cur is None:
            name, cur = m.group(2).lower(), []
            continue
        if re.match(r"^end\s+(subroutine|function)\b", line, re.I):
            if name is not None:
                out[name] = cur
            name, cur = None, None
            continue
        if cur is not None and line and not re.match(r"^(integer|real|logical|character)\b.*::", line, re.I) \
                and not re.match(r"^(implicit|use)\b", line, re.I):
            cur.append(line)
    return out


def eval_expr(expr, const):
    expr = expr.strip().lower()
    toks = re.findall(r"[+-]?\s*\w+", expr)
    total = 0
    for t in toks:
        t = t.replace(" ", "")
        sign = -1 if t.startswith("-") else 1
        t = t.lstrip("+-")
        total += sign * (int(t) if t.isdigit() else const[t])
    return total


def parse_coord(text, const):
    """'site + (/a, b, c, e/)' -> (base, (a, b, c), e evaluated)."""
    m = _COORD.match(text.strip())
    if not m:
        raise ValueError("coordinate %r" % text)
    if not m.group(2):
        return m.group(1), (0, 0, 0), 0
    parts = [p.strip() for p in m.group(2).split(",")]
    return m.group(1), tuple(eval_expr(p, const) for p in parts[:3]), eval_expr(parts[3], const)


def _split_args(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _call(line):
    m = re.match(r"^call\s+(\w+)\s*\((.*)\)$", line, re.I)
    return (m.group(1).lower(), _split_args(m.group(2))) if m else (None, None)


def species_mask(names, const):
    mask = 0
    for n in names:
        sid = const[n.strip().lower()]
        mask |= 1 << (31 if sid < 0 else sid)
    return mask - (1 << 32) if mask & 0x80000000 else mask


# ------------------------------------------------------------------------ local_smart
def routine_ops(body, site_n, const, arg_species=None):
    """Ops of one put/take/create/annihilate/touchup routine relative to its site."""
    ops, stack = [], []  # stack of (coord, species mask or None)
    i = 0

    def co(text):
        base, off, e = parse_coord(text, const)
        return off + (site_n + e if base != "cell" else e,)

    while i < len(body):
        line = body[i]
        low = line.lower()
        name, args = _call(line)
        if name == "replace_species":
            old, new = args[1].lower(), args[2].lower()
            old = arg_species if old == "species" else old
            new = arg_species if new == "species" else new
            ops.append(("replace", co(args[0]), species_mask([old], const), const[new]))
        elif low.startswith("if(avail_sites(") or low.startswith("if (can_do(") or low.startswith("if(can_do("):
            # guarded del: if(...)then / call del_proc(p, coord) / endif
            name2, a2 = _call(body[i + 1])
            assert name2 == "del_proc" and body[i + 2].lower().startswith("endif"), body[i:i + 3]
            ops.append(("gdel", const[a2[0].lower()], co(a2[1])))
            i += 3
            continue
        elif low.startswith("select case(get_species("):
            inner = re.match(r"select case\(get_species\((.*)\)\)$", low).group(1)
            stack.append([co(inner), None])
        elif low.startswith("case default"):
            stack[-1][1] = "default"
        elif low.startswith("case("):
            stack[-1][1] = species_mask(_split_args(re.match(r"case\((.*)\)$", low).group(1)), const)
        elif low.startswith("end select"):
            stack.pop()
        elif name == "add_proc":
            conds = frozenset((c, m) for c, m in stack)
            ops.append(("add", const[args[0].lower()], co(args[1]), conds))
        elif name == "del_proc":
            ops.append(("del", const[args[0].lower()], co(args[1])))
        else:
            raise ValueError("unrecognised line %r" % line)
        i += 1
    return ops


def local_smart_ops(directory):
    """{proc id: [ops]} and {site n: touch-up ops} of a local_smart export."""
    text = open(os.path.join(directory, "proclist.f90")).read()
    lat = open(os.path.join(directory, "lattice.f90")).read()
    const = parse_constants([text, lat])
    subs = subroutines(text)
    sites = {k: v for k, v in const.items()
             if re.search(r"parameter,\s*public\s*::\s*%s\s*=" % k, lat, re.I) and k != "spuck" and
             k not in ("nr_of_layers", "model_dimension") and not k.startswith("default_layer")}
    site_names = sorted((k for k in sites if any(
        ("_" + k) in r or r.endswith(k) for r in subs)), key=len, reverse=True)

    def routine_site(rname):
        for sname in site_names:
            if rname.endswith("_" + sname):
                return const[sname]
        raise ValueError("no site for routine %s" % rname)

    procs = {}
    body = subs["run_proc_nr"]
    cur = None
    for line in body:
        m = re.match(r"^case\((\w+)\)$", line, re.I)
        if m:
            cur = const[m.group(1).lower()]
            procs[cur] = []
            continue
        name, args = _call(line)
        if cur is None or name is None or name == "increment_procstat":
            continue
        base, off, _e = parse_coord(args[0], const)
        arg_sp = args[1].lower() if len(args) > 1 else None
        rops = routine_ops(subs[name], routine_site(name), const, arg_sp)
        procs[cur].extend(shift(rops, off))
    touch = {}
    for rname, rbody in subs.items():
        if rname.startswith("touchup_"):
            touch[routine_site(rname)] = routine_ops(rbody, routine_site(rname), const)
    return procs, touch, const


def shift(ops, off):
    def sh(c):
        return (c[0] + off[0], c[1] + off[1], c[2] + off[2], c[3])

    out = []
    for op in ops:
        if op[0] == "replace":
            out.append(("replace", sh(op[1]), op[2], op[3]))
        elif op[0] in ("gdel", "del"):
            out.append((op[0], op[1], sh(op[2])))
        elif op[0] == "add":
            out.append(("add", op[1], sh(op[2]), frozenset((sh(c), m) for c, m in op[3])))
        else:
            out.append(op)
    return out


# ----------------------------------------------------------------------------- lat_int
def lat_int_ops(directory):
    """{proc id: [ops]}, {group name: nli tree}, group names in file order."""
    texts = [open(f).read() for f in sorted(glob.glob(os.path.join(directory, "*.f90")))]
    const = parse_constants(texts)
    proclist = subroutines(open(os.path.join(directory, "proclist.f90")).read())
    # process -> group from run_proc_nr's select case
    proc_group = {}
    cur = []
    for line in proclist["run_proc_nr"]:
        m = re.match(r"^case\s*\((.*)\)$", line, re.I)
        if m:
            cur = [const[n.strip().lower()] for n in m.group(1).split(",")]
            continue
        mm = re.match(r"^call\s+run_proc_(\w+)\(cell\)$", line, re.I)
        if mm:
            for p in cur:
                proc_group[p] = mm.group(1).lower()
    groups = []
    runs, nlis = {}, {}
    for f in sorted(glob.glob(os.path.join(directory, "run_proc_*.f90"))):
        for name, body in subroutines(open(f).read()).items():
            g = name[len("run_proc_"):]
            groups.append(g)
            runs[g] = body
    for f in sorted(glob.glob(os.path.join(directory, "nli_*.f90"))):
        for name, body in subroutines(open(f).read()).items():
            nlis[name[len("nli_"):]] = nli_tree(body, const, name)
    gidx = {g: i for i, g in enumerate(groups)}
    gops = {}
    for g, body in runs.items():
        ops = []
        i = 0
        while i < len(body):
            line = body[i]
            m = re.match(r"^call\s+(del_proc|add_proc)\(nli_(\w+)\((.*?)\),\s*(.*)\)$", line, re.I)
            if m:
                _b, off, e = parse_coord(m.group(4), const)
                ops.append(("li_del" if m.group(1).lower() == "del_proc" else "li_add",
                            gidx[m.group(2).lower()], off + (e,)))
                i += 1
                continue
            name, args = _call(line)
            if name == "replace_species":
                _b, off, e = parse_coord(args[0], const)
                ops.append(("replace", off + (e,), species_mask([args[1]], const), const[args[2].lower()]))
                i += 1
                continue
            m = re.match(r"^select case\(get_species\(\((.*)\)\)\)$", line, re.I)
            if m:  # replace with "or" alternatives
                _b, off, e = parse_coord(m.group(1), const)
                olds, new = [], None
                i += 1
                while not body[i].lower().startswith("case default"):
                    name, args = _call(body[i])
                    if name == "replace_species":
                        olds.append(args[1])
                        new = const[args[2].lower()]
                    i += 1
                while not body[i].lower().startswith("end select"):
                    i += 1
                ops.append(("replace", off + (e,), species_mask(olds, const), new))
                i += 1
                continue
            raise ValueError("unrecognised line %r" % line)
        gops[g] = ops
    procs = {p: gops[g] for p, g in proc_group.items()}
    return procs, {gidx[g]: t for g, t in nlis.items()}, groups, const


def nli_tree(body, const, fname):
    """Nested select-case tree: ("sel", coord, [(mask or 'default', subtree)]) or
    ("ret", value)."""
    pos = 0

    def block():
        nonlocal pos
        line = body[pos].lower()
        m = re.match(r"^select case\(get_species\((.*)\)\)$", line)
        if m:
            _b, off, e = parse_coord(m.group(1), const)
            pos += 1
            cases = []
            while not body[pos].lower().startswith("end select"):
                cl = body[pos].lower()
                if cl.startswith("case default"):
                    key = "default"
                else:
                    key = species_mask(_split_args(re.match(r"case\s*\((.*)\)$", cl).group(1)), const)
                pos += 1
                cases.append((key, block()))
            pos += 1
            return ("sel", off + (e,), cases)
        m = re.match(r"^%s\s*=\s*(\w+);\s*return$" % fname, line)
        if m:
            pos += 1
            v = m.group(1)
            return ("ret", int(v) if v.isdigit() else const[v])
        raise ValueError("nli line %r" % line)

    return block()


def eval_nli(tree, species_at):
    """Value of an nli tree; species_at(coord) -> species id."""
    while tree[0] == "sel":
        s = species_at(tree[1])
        bit = 31 if s < 0 else s
        nxt = None
        for key, sub in tree[2]:
            if key != "default" and ((key & 0xFFFFFFFF) >> bit) & 1:
                nxt = sub
                break
        if nxt is None:
            nxt = [sub for key, sub in tree[2] if key == "default"][0]
        tree = nxt
    return tree[1]


def tree_coords(tree, out=None):
    out = [] if out is None else out
    if tree[0] == "sel":
        if tree[1] not in out:
            out.append(tree[1])
        for _k, sub in tree[2]:
            tree_coords(sub, out)
    return out


# ------------------------------------------------------------------------------ otf
def _otf_body_ops(body, const):
    """Ops of a run_proc_<name>(cell) or touchup_cell body of the otf generator
    (kmos/io/__init__.py:3240-3597): guarded dels and rate updates, replaces, adds under
    select-case paths.  Coordinates are relative to the process's cell."""
    ops, stack, i = [], [], 0

    def coord(text):
        base, off, e = parse_coord(text, const)
        if base != "cell":
            raise ValueError(text)
        return off + (e,)

    while i < len(body):
        line = body[i]
        low = line.lower().replace(" ", "")
        m = re.match(r"^if\(can_do\((\w+),(cell\+\(/.*/\))\)\)then$", low)
        if m:
            proc, target = const[m.group(1)], coord(m.group(2))
            name, args = _call(body[i + 1].lower())
            if name == "del_proc":
                ops.append(("gdel", proc, target))
            elif name == "update_rates_matrix":
                ops.append(("update", proc, target))
            else:
                raise ValueError(body[i + 1])
            assert body[i + 2].lower().replace(" ", "") == "endif", body[i + 2]
            i += 3
            continue
        name, args = _call(line.lower())
        if name == "replace_species":
            old = species_mask([args[1]], const)
            ops.append(("replace", coord(args[0]), old, const[args[2].strip()]))
        elif name == "add_proc":
            conds = sorted((c, mk) for c, mk in stack)
            ops.append(("add", const[args[0].strip()], coord(args[1]), conds))
        elif low.startswith("selectcase(get_species("):
            inner = re.match(r"select case\(get_species\((.*)\)\)$", line.lower()).group(1)
            stack.append([coord(inner), None])
        elif low.startswith("case("):
            stack[-1][1] = species_mask(_split_args(re.match(r"case\((.*)\)$", low).group(1)), const)
        elif low.startswith("endselect"):
            stack.pop()
        elif low.startswith("site=cell+") or low.startswith("doproc_nr=1") or low.startswith("enddo"):
            pass
        elif low.startswith("if(avail_sites(proc_nr") or low.startswith("calldel_proc(proc_nr") or low == "endif":
            pass  # touchup_cell's strip loop
        elif name is None and low not in ("return",):
            raise ValueError("unrecognised line %r" % line)
        i += 1
    return ops


def otf_ops(directory):
    """{'procs': {proc: ops}, 'touchups': {'1': ops}, 'rates': {proc: rate function}}
    from an otf export (proclist.f90, run_proc_*.f90, proclist_pars.f90)."""
    texts = {os.path.basename(f): open(f).read() for f in glob.glob(os.path.join(directory, "*.f90"))}
    const = parse_constants([texts["proclist_constants.f90"], texts["lattice.f90"]])
    procs = {}
    for fname, text in texts.items():
        if not fname.startswith("run_proc_"):
            continue
        for sub, body in subroutines(text).items():
            procs[const[sub[len("run_proc_"):]]] = _otf_body_ops(body, const)
    touch = _otf_body_ops(subroutines(texts["proclist.f90"])["touchup_cell"], const)
    touch = [("strip", (0, 0, 0, 1))] + touch
    pars = subroutines(texts["proclist_pars.f90"])
    rates = {}
    for sub, body in pars.items():
        if not sub.startswith("gr_"):
            continue
        name = sub[3:]
        byst, cur = [], None
        for line in body:
            low = line.lower().replace(" ", "")
            m = re.match(r"^selectcase\(get_species\((cell\+\(/.*/\))\)\)$", low)
            if m:
                base, off, e = parse_coord(m.group(1), const)
                cur = [off + (e,), []]
                byst.append(cur)
                continue
            m = re.match(r"^case\((\w+)\)$", low)
            if m:
                spec = const[m.group(1)]
                continue
            m = re.match(r"^nr_vars\((\d+)\)=nr_vars\(\d+\)\+1$", low)
            if m:
                cur[1].append((spec, int(m.group(1)) - 1))
        expr = " ".join(pars["rate_" + name])
        m = re.search(r"rate_%s\s*=\s*(.*?)\s*return" % name, expr, re.I)
        rates[const[name]] = {"bystanders": byst, "expr": m.group(1) if m else ""}
    return {"procs": procs, "touchups": {"1": touch}, "rates": rates}
