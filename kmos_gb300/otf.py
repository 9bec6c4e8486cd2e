"""The otf ("on-the-fly") backend: per-site rates that depend on bystanders.

kmos's otf backend (kmos/io/__init__.py:2657-3723, kmos/fortran_src/base_otf.f90) keeps,
beside avail_sites, a rate for every available (process, site) entry: ``rates_matrix(p,
i)`` belongs to the i-th entry of process p's list and moves with it when del_proc
swaps the last entry into a hole (base_otf.f90:221-331).  Every step re-sums each list
left to right (update_accum_rate, base_otf.f90:687-716), picks the process from those
totals and then the entry from the running sum of the chosen list (determine_procsite,
base_otf.f90:1213-1277).

The rate of an entry is ``gr_<process>(cell)`` (io:2657-2965): count the bystanders'
species into ``nr_<species>_<flag>`` variables and evaluate the process's ``otf_rate``
expression, a Fortran expression over ``base_rate`` (the process's rate constant),
the model's parameters (``userpar``), those counts, unit constants and aux variables.
Without an ``otf_rate`` the rate is the rate constant.

A process instance is anchored at a *cell*: its entry is the site (cell, 1) whatever
the process's executing coordinate, and its conditions, actions and bystanders are read
at cell + their own offsets.  ``run_proc_<name>`` (io:3328-3597) is, in order:
  1. guarded del_proc of every (process, relative cell) an action disables;
  2. replace_species for every action;
  3. update_rates_matrix (rate re-evaluated) of every available (process, relative cell)
     whose bystanders an action touches, unless the action disables it;
  4. add_proc with the rate of every (process, relative cell) an action enables, through
     the same if-tree as local_smart (``_write_optimal_iftree_otf``).
The (process, relative cell) lists are de-duplicated through Python sets of offset
tuples, exactly as the generator does; their iteration order is part of the op order.
``touchup_cell`` (io:3240-3285) strips the cell's entries and re-adds through the if-tree
over every process's conditions.

Program form (backend 2).  The header is the local_smart/lat_int one (program.py) with
one touch-up stream (the cell's) and no hot section; ops are OP_REPLACE, OP_GDEL,
OP_ADD (the add evaluates the rate), OP_STRIP and::

    OP_UPDATE   [h(arg=proc), coord]     if can_do(proc, site): update_rates_matrix(
                                         proc, site, gr_proc(cell of coord))

Header word 22 = offset of P+1 rate-record offsets, word 23 = number of user parameters
plus chemical potentials (``mu_*``, the generator's chempots array, which follow the
parameters in the engine's parameter vector).
Rate record of process p::

    [nbyst, nvars, ncode, stack, (coord, npairs, (species, var) * npairs) * nbyst, code...]

A bystander adds one to ``nr_vars[var]`` for each pair whose species it holds.  ``code``
is a postfix program of one-word instructions ``opcode | kind << 8 | arg << 16`` with
constants in the words that follow; values are typed at compile time the way Fortran
types them (integer, default real = IEEE single, real(8) = double):

    PUSH_BASE, PUSH_PAR k, PUSH_NR v, PUSH_INT [value], PUSH_CONST [lo, hi],
    LOAD_AUX a, STORE_AUX a, STORE_RESULT, END,
    ADD SUB MUL DIV NEG (kind), POWI (real kind ** integer: libgcc's __powi binary
    method; integer ** integer), POW EXP LOG SQRT ABS (kind), CVT (from kind -> to kind)

Integer literals are integers, real literals without a ``d`` exponent are default reals
(single precision: the generated Fortran is compiled without -fdefault-real-8,
kmos/utils/__init__.py:452-457), unit constants are double parameters initialised from a
single-precision literal printed with ``%.10e`` (io:2728-2738).  Everything but exp, log
and real ** real is exact IEEE arithmetic, so rates and trajectories match the
reference's bit for bit; exp, log and pow match it to the libraries' last-place error.
"""
from __future__ import annotations

import io
import math
import re
import struct
import tokenize
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .model import Model, Process
from . import rates as R

OP_UPDATE = 7

# expression instructions
I_END, I_PUSH_BASE, I_PUSH_PAR, I_PUSH_NR, I_PUSH_INT, I_PUSH_CONST = 0, 1, 2, 3, 4, 5
I_LOAD_AUX, I_STORE_AUX, I_STORE_RESULT = 6, 7, 8
I_ADD, I_SUB, I_MUL, I_DIV, I_NEG, I_POWI, I_POW, I_EXP, I_LOG, I_SQRT, I_ABS, I_CVT = range(10, 22)
K_INT, K_F32, K_F64 = 0, 1, 2
STACK_MAX = 16
AUX_MAX = 8

_FUNCS = {"exp": I_EXP, "log": I_LOG, "sqrt": I_SQRT, "abs": I_ABS,
          "dexp": I_EXP, "dlog": I_LOG, "dsqrt": I_SQRT, "dabs": I_ABS}


def ins(op: int, kind: int = 0, arg: int = 0) -> int:
    return op | (kind << 8) | (arg << 16)


def _f64_words(v: float) -> List[int]:
    lo, hi = struct.unpack("<ii", struct.pack("<d", v))
    return [lo, hi]


def _f32(v: float) -> float:
    return float(np.float32(v))


# ------------------------------------------------------------------------------------
# expression compiler
# ------------------------------------------------------------------------------------
class ExprError(ValueError):
    pass


class _Compiler:
    """Fortran expression -> typed postfix code.  Grammar (Fortran precedence):
    expr := [+|-] term {(+|-) term};  term := factor {(*|/) factor};
    factor := primary [** factor];  primary := number | name | name(expr) | (expr),
    with ``a * -b`` accepted as gfortran does (the sign applies to the factor)."""

    def __init__(self, names: Dict[str, tuple]):
        self.names = names      # name -> ("par", k) | ("nr", v) | ("const", value) | ("aux", a)
        self.code: List[int] = []
        self.depth = 0
        self.max_depth = 0

    # stack bookkeeping
    def _push(self, n=1):
        self.depth += n
        self.max_depth = max(self.max_depth, self.depth)

    def emit(self, *ws, push=0):
        self.code.extend(int(w) for w in ws)
        if push > 0:
            self._push(push)
        else:
            self.depth += push

    def cvt(self, frm: int, to: int):
        if frm != to:
            self.emit(ins(I_CVT, frm, to))

    # tokens
    def parse(self, toks: List[Tuple[int, str, int]]) -> int:
        self.toks, self.i = toks, 0
        k = self.expr()
        if self.i != len(self.toks):
            raise ExprError("unexpected %r" % self.toks[self.i][1])
        return k

    def peek(self):
        return self.toks[self.i][1] if self.i < len(self.toks) else None

    def take(self):
        t = self.toks[self.i]
        self.i += 1
        return t

    def expr(self) -> int:
        sign = None
        if self.peek() in ("+", "-"):
            sign = self.take()[1]
        k = self.term_with_lookahead()
        if sign == "-":
            self.emit(ins(I_NEG, k))
        while self.peek() in ("+", "-"):
            op = I_ADD if self.take()[1] == "+" else I_SUB
            k = self.rhs(k, self.term_with_lookahead, op)
        return k

    def rhs(self, ka: int, parse_b, op: int) -> int:
        """Compile b after a; a's conversion to the common kind is patched in when b's
        kind turns out wider (Fortran promotes the narrower operand)."""
        mark = len(self.code)
        depth = self.depth
        kb = parse_b()
        k = max(ka, kb)
        if ka != k:
            # insert a's conversion before b's code (a is on top of the stack there)
            self.code[mark:mark] = [ins(I_CVT, ka, k)]
        if kb != k:
            self.cvt(kb, k)
        self.depth = depth
        self.emit(ins(op, k))
        return k

    def term_with_lookahead(self) -> int:
        k = self.factor()
        while self.peek() in ("*", "/"):
            op = I_MUL if self.take()[1] == "*" else I_DIV
            k = self.rhs(k, self.signed_factor, op)
        return k

    def signed_factor(self) -> int:
        if self.peek() in ("+", "-"):
            s = self.take()[1]
            k = self.signed_factor()
            if s == "-":
                self.emit(ins(I_NEG, k))
            return k
        return self.factor()

    def factor(self) -> int:
        ka = self.primary()
        if self.peek() == "**":
            self.take()
            mark = len(self.code)
            depth = self.depth
            kb = self.signed_factor_pow()
            self.depth = depth
            if kb == K_INT:
                # real ** integer (and integer ** integer): __powi
                self.emit(ins(I_POWI, ka))
                return ka
            k = max(ka, kb)
            if ka != k:
                self.code[mark:mark] = [ins(I_CVT, ka, k)]
            if kb != k:
                self.cvt(kb, k)
            self.emit(ins(I_POW, k))
            return k
        return ka

    def signed_factor_pow(self) -> int:
        # right-associative: a ** b ** c = a ** (b ** c); a leading sign (a ** -n) is a
        # gfortran extension with the sign on the factor
        if self.peek() in ("+", "-"):
            s = self.take()[1]
            k = self.signed_factor_pow()
            if s == "-":
                self.emit(ins(I_NEG, k))
            return k
        return self.factor()

    def number(self, text: str) -> int:
        t = text.lower()
        if re.fullmatch(r"\d+", t):
            v = int(t)
            if v >= 2 ** 31:
                raise ExprError("integer literal %s out of range" % text)
            self.emit(ins(I_PUSH_INT), v, push=1)
            return K_INT
        if "d" in t:
            self.emit(ins(I_PUSH_CONST, K_F64), *_f64_words(float(t.replace("d", "e"))), push=1)
            return K_F64
        self.emit(ins(I_PUSH_CONST, K_F32), *_f64_words(_f32(float(t))), push=1)
        return K_F32

    def primary(self) -> int:
        if self.i >= len(self.toks):
            raise ExprError("unexpected end of expression")
        kind, text, _pos = self.take()
        if text == "(":
            k = self.expr()
            if self.peek() != ")":
                raise ExprError("missing )")
            self.take()
            return k
        if kind == tokenize.NUMBER:
            return self.number(text)
        if kind != tokenize.NAME:
            raise ExprError("unexpected %r" % text)
        if self.peek() == "(":
            if text.lower() not in _FUNCS:
                raise ExprError("function %s is not supported" % text)
            self.take()
            k = self.expr()
            if self.peek() != ")":
                raise ExprError("missing ) after %s(" % text)
            self.take()
            if k == K_INT:
                raise ExprError("%s of an integer" % text)
            self.emit(ins(_FUNCS[text.lower()], k))
            return k
        if text == "base_rate":
            self.emit(ins(I_PUSH_BASE), push=1)
            return K_F64
        if text not in self.names:
            raise ExprError("unknown name %r" % text)
        what = self.names[text]
        if what[0] == "par":
            self.emit(ins(I_PUSH_PAR, 0, what[1]), push=1)
            return K_F64
        if what[0] == "nr":
            self.emit(ins(I_PUSH_NR, 0, what[1]), push=1)
            return K_INT
        if what[0] == "aux":
            self.emit(ins(I_LOAD_AUX, 0, what[1]), push=1)
            return K_F64
        self.emit(ins(I_PUSH_CONST, K_F64), *_f64_words(what[1]), push=1)
        return K_F64


def _tokens(text: str) -> List[Tuple[int, str, int]]:
    """Python tokens of one expression line, with Fortran ``1.0d-3`` literals joined."""
    try:
        raw = list(tokenize.generate_tokens(io.StringIO(text).readline))
    except tokenize.TokenError as e:
        raise ExprError("cannot tokenize %r" % text) from e
    toks = [(t.type, t.string, t.start[1], t.end[1]) for t in raw
            if t.type not in (tokenize.NEWLINE, tokenize.NL, tokenize.ENDMARKER, tokenize.INDENT,
                              tokenize.DEDENT, tokenize.COMMENT)]
    out: List[Tuple[int, str, int]] = []
    i = 0
    while i < len(toks):
        ty, s, a, b = toks[i]
        if ty == tokenize.NUMBER and i + 1 < len(toks) and toks[i + 1][2] == b and \
                re.fullmatch(r"[dD]\d*", toks[i + 1][1]):
            lit, j = s + toks[i + 1][1], i + 2
            if toks[i + 1][1] in ("d", "D") and j + 1 < len(toks) and toks[j][1] in ("+", "-") \
                    and toks[j][2] == toks[i + 1][3] and toks[j + 1][0] == tokenize.NUMBER:
                lit += toks[j][1] + toks[j + 1][1]
                j += 2
            out.append((tokenize.NUMBER, lit, a))
            i = j
            continue
        out.append((ty, s, a))
        i += 1
    return out


def unit_constant(name: str) -> float:
    """A unit constant as the generated module declares it: ``%.10e`` of its value, a
    default-real (single precision) literal widened to double (io:2728-2733)."""
    return _f32(float("%.10e" % R.UNITS[name]))


def mass_constant(name: str) -> float:
    return _f32(float("%.10e" % R.evaluate_rate_expression(name)))


def nr_var_names(proc: Process) -> List[str]:
    """The ``nr_<species>_<flag>`` variables of gr_<proc> in the generator's order
    (io:2800-2830): every (allowed species, flag) pair of the bystanders plus those the
    expression names, sorted by (flag, species) as split on underscores."""
    used = set()
    # the whole expression is tokenized at once, as _parse_otf_rate does (io:3066-3085)
    expr = (proc.otf_rate or "").replace("base_rate", "rates").replace("otf_rate", "gr")
    for _ty, s, _a in _tokens(expr.replace("beta", "(1/(kboltzmann*T))")):
        if s.startswith("nr_"):
            used.add(s)
    nr_vars = list(used)
    specs: Dict[str, List[str]] = {}
    flags = []
    for b in proc.bystanders:
        for flg in b.flag.split():
            specs.setdefault(flg, []).extend(b.allowed_species)
            flags.append(flg)
    for flg in sorted(set(flags)):
        for spec in sorted(specs[flg]):
            v = "nr_%s_%s" % (spec, flg)
            if v not in nr_vars:
                nr_vars.append(v)
    return sorted(nr_vars, key=lambda x: (x.split("_")[2], x.split("_")[1]))


def chempot_names(model: Model) -> List[str]:
    """The ``mu_<species>`` chemical potentials any rate_constant or otf_rate names, sorted
    (io:2966-2998): the generated module's ``chempots`` array, set by update_chempot.
    Here they follow the user parameters in the engine's parameter vector.  As in the
    reference, each expression is tokenized whole after the rate aliases (an expression
    that does not tokenize is an error), and every ``mu_`` name is a chemical potential,
    also when a user parameter has that name (_parse_otf_rate tests ``mu_`` first,
    io:3086-3090)."""
    found = set()
    for proc in model.processes:
        for expr in (proc.rate_constant or "", proc.otf_rate or ""):
            toks = _tokens(expr.replace("beta", "(1/(kboltzmann*T))"))
            found.update(t for ty, t, _a in toks if ty == tokenize.NAME and t.startswith("mu_"))
    return sorted(found)


def compile_rate(model: Model, proc: Process) -> Tuple[List[str], List[int], int]:
    """(nr variable names, code, stack depth) of gr_<proc> (io:2800-2965, 3000-3122)."""
    params = sorted(p.name for p in model.parameters)
    nr_vars = nr_var_names(proc)
    names: Dict[str, tuple] = {}
    for k, pn in enumerate(params):
        names[pn] = ("par", k)
    for j, mu in enumerate(chempot_names(model)):   # chempots(mu) after the parameters
        names[mu] = ("par", len(params) + j)
    for v, nv in enumerate(nr_vars):
        names[nv] = ("nr", v)
    c = _Compiler(names)
    expr = proc.otf_rate
    if not expr or not expr.strip():
        c.emit(ins(I_PUSH_BASE), push=1)
        c.emit(ins(I_STORE_RESULT), push=-1)
        c.emit(ins(I_END))
        return nr_vars, c.code, c.max_depth
    lines = [l for l in expr.split("\n")]
    if len(lines) == 1 and "=" not in lines[0]:
        lines[0] = "otf_rate =" + lines[0]
    elif len(lines) == 1 and "otf_rate" not in lines[0]:
        raise ExprError("a one-line otf_rate with '=' must assign otf_rate")
    elif "otf_rate" not in expr:
        raise ExprError("a multi-line otf_rate must assign otf_rate")
    naux = 0
    for line in lines:
        if not line.strip():
            continue
        for old, new in (("beta", "(1/(kboltzmann*T))"),):  # kmos rate_aliases
            line = line.replace(old, new)
        if "=" not in line:
            raise ExprError("otf_rate line without an assignment: %r" % line)
        lhs, rhs = line.split("=", 1)
        lhs = lhs.strip()
        toks = _tokens(rhs)
        for ty, s, _a in toks:
            if ty == tokenize.NAME and s not in names and s not in _FUNCS and s != "base_rate":
                if s in R.UNITS:
                    names[s] = ("const", unit_constant(s))
                elif s.startswith("m_"):
                    names[s] = ("const", mass_constant(s))
        k = c.parse(toks)
        c.cvt(k, K_F64)   # every assignment target is real(8)
        if lhs == "otf_rate":
            c.emit(ins(I_STORE_RESULT), push=-1)
        else:
            if lhs not in names:
                if naux >= AUX_MAX:
                    raise ExprError("more than %d auxiliary variables" % AUX_MAX)
                names[lhs] = ("aux", naux)
                naux += 1
            if names[lhs][0] != "aux":
                raise ExprError("cannot assign to %s" % lhs)
            c.emit(ins(I_STORE_AUX, 0, names[lhs][1]), push=-1)
    c.emit(ins(I_END))
    if c.max_depth > STACK_MAX:
        raise ExprError("otf_rate of %s needs a stack deeper than %d" % (proc.name, STACK_MAX))
    return nr_vars, c.code, c.max_depth


def powi(x: float, m: int, kind: int):
    """x ** m for an integer m by libgcc's __powi (right-to-left binary powering, the
    reciprocal of the result for negative m), each product rounded to ``kind``."""
    rnd = _f32 if kind == K_F32 else (lambda v: v)
    if kind == K_INT:
        n = abs(m)
        y = x if n % 2 else 1
        while True:
            n >>= 1
            if not n:
                break
            x = x * x
            if n % 2:
                y = y * x
        if m < 0:
            return 0 if abs(y) != 1 else (y if (-m) % 2 else 1)
        return y
    n = abs(m)
    y = x if n % 2 else 1.0
    while True:
        n >>= 1
        if not n:
            break
        x = rnd(x * x)
        if n % 2:
            y = rnd(y * x)
    return rnd(1.0 / y) if m < 0 else y


def evaluate(code: Sequence[int], base: float, userpar: Sequence[float], nr: Sequence[int]) -> float:
    """Runs a rate program in Python (the same arithmetic as the engine's and the
    oracle's evaluators)."""
    st: List[float] = []
    aux = [0.0] * AUX_MAX
    result = 0.0
    pc = 0
    code = [int(w) for w in code]
    while True:
        w = code[pc] & 0xFFFFFFFF
        op, kind, arg = w & 0xFF, (w >> 8) & 0xFF, w >> 16
        pc += 1
        if op == I_END:
            return result
        if op == I_PUSH_BASE:
            st.append(base)
        elif op == I_PUSH_PAR:
            st.append(float(userpar[arg]))
        elif op == I_PUSH_NR:
            st.append(int(nr[arg]))
        elif op == I_PUSH_INT:
            st.append(int(code[pc]))
            pc += 1
        elif op == I_PUSH_CONST:
            st.append(struct.unpack("<d", struct.pack("<ii", code[pc], code[pc + 1]))[0])
            pc += 2
        elif op == I_LOAD_AUX:
            st.append(aux[arg])
        elif op == I_STORE_AUX:
            aux[arg] = st.pop()
        elif op == I_STORE_RESULT:
            result = st.pop()
        elif op in (I_ADD, I_SUB, I_MUL, I_DIV):
            b, a = st.pop(), st.pop()
            if kind == K_INT:
                if op == I_ADD:
                    v = a + b
                elif op == I_SUB:
                    v = a - b
                elif op == I_MUL:
                    v = a * b
                else:  # Fortran integer division truncates toward zero
                    v = 0 if b == 0 else (abs(a) // abs(b)) * (1 if (a < 0) == (b < 0) else -1)
                st.append(((int(v) + 2**31) % 2**32) - 2**31)
            else:
                if op == I_ADD:
                    v = a + b
                elif op == I_SUB:
                    v = a - b
                elif op == I_MUL:
                    v = a * b
                else:
                    v = a / b if b != 0 else (math.copysign(math.inf, a) * math.copysign(1.0, b) if a != 0 else math.nan)
                st.append(_f32(v) if kind == K_F32 else v)
        elif op == I_NEG:
            st.append(-st.pop())
        elif op == I_POWI:
            m, x = int(st.pop()), st.pop()
            st.append(powi(x, m, kind))
        elif op == I_POW:
            b, a = st.pop(), st.pop()
            st.append(float(np.float32(a) ** np.float32(b)) if kind == K_F32 else math.pow(a, b))
        elif op in (I_EXP, I_LOG, I_SQRT, I_ABS):
            a = st.pop()
            f = {I_EXP: math.exp, I_LOG: math.log, I_SQRT: math.sqrt, I_ABS: abs}[op]
            st.append(_f32(f(a)) if kind == K_F32 else f(a))
        elif op == I_CVT:
            a = st.pop()
            st.append(_f32(a) if arg == K_F32 else float(a))
        else:
            raise ValueError("bad instruction %d" % op)


# ------------------------------------------------------------------------------------
# op streams
# ------------------------------------------------------------------------------------
def _off(a, b) -> Tuple[int, int, int]:
    return (a.offset[0] - b.offset[0], a.offset[1] - b.offset[1], a.offset[2] - b.offset[2])


def process_ops(model: Model, exec_proc: Process, site_ids, species_mask) -> List[tuple]:
    """run_proc_<exec_proc> (io:3328-3597) as ops relative to the process's cell."""
    procs = sorted(model.processes, key=lambda p: p.name)        # data.get_processes()
    pid = model.process_ids()
    n = len(procs)
    inh: List[list] = [[] for _ in range(n)]
    enh: List[list] = [[] for _ in range(n)]
    aff: List[list] = [[] for _ in range(n)]
    for act in exec_proc.actions:
        for ip, proc in enumerate(procs):
            for cond in proc.conditions:
                if cond.coord.name == act.coord.name and cond.coord.layer == act.coord.layer:
                    rel = _off(act.coord, cond.coord)
                    (inh if cond.species != act.species else enh)[ip].append(rel)
            for b in proc.bystanders:
                if b.coord.name == act.coord.name and b.coord.layer == act.coord.layer:
                    aff[ip].append(_off(act.coord, b.coord))
    for ip in range(n):
        inh[ip] = [r for r in set(inh[ip])]
    for ip in range(n):
        enh[ip] = [r for r in set(enh[ip]) if r not in inh[ip]]
        aff[ip] = [r for r in set(aff[ip]) if r not in inh[ip]]
    ops: List[tuple] = []
    for ip in range(n):
        for rel in inh[ip]:
            ops.append(("gdel", pid[procs[ip].name], rel + (1,)))
    for act in exec_proc.actions:
        prev = [c for c in exec_proc.conditions if c.coord == act.coord]
        if len(prev) != 1:
            raise ValueError("process %s: %d conditions on the site of an action" % (exec_proc.name, len(prev)))
        ops.append(("replace", tuple(act.coord.offset) + (site_ids[(act.coord.layer, act.coord.name)],),
                    species_mask(prev[0].species), act.species))
    for ip in range(n):
        for rel in aff[ip]:
            ops.append(("update", pid[procs[ip].name], rel + (1,)))
    items = []
    for ip in range(n):
        for rel in enh[ip]:
            other = []
            for cond in procs[ip].conditions:
                for act in exec_proc.actions:
                    if act.coord.name == cond.coord.name and act.coord.layer == cond.coord.layer \
                            and rel == _off(act.coord, cond.coord):
                        if act.species != cond.species:
                            raise ValueError("discrepancy in process selected for enabling")
                        break
                else:
                    o = cond.coord.offset
                    other.append(((o[0] + rel[0], o[1] + rel[1], o[2] + rel[2],
                                   site_ids[(cond.coord.layer, cond.coord.name)]), cond.species))
            items.append((tuple(other), (pid[procs[ip].name], rel + (1,))))
    ops.extend(_iftree_adds(items))
    return ops


def _iftree_adds(items) -> List[tuple]:
    """Adds of ``_write_optimal_iftree_otf`` (io:3598-3723) in the tree's depth-first
    leaf order, each with the conditions of its path."""
    from .program import AddItem, flatten_iftree
    leaves = [(conds, AddItem(conds, proc, target)) for conds, (proc, target) in items]
    return [("add", leaf.proc, leaf.target, leaf.conds) for leaf in flatten_iftree(leaves)]


def touchup_ops(model: Model, site_ids) -> List[tuple]:
    """touchup_cell (io:3240-3285): strip the cell's entries, then the if-tree over every
    process's conditions (processes in file order)."""
    pid = model.process_ids()
    items = []
    for proc in model.processes:
        conds = tuple((tuple(c.coord.offset) + (site_ids[(c.coord.layer, c.coord.name)],), c.species)
                      for c in proc.conditions)
        items.append((conds, (pid[proc.name], (0, 0, 0, 1))))
    return [("strip", (0, 0, 0, 1))] + _iftree_adds(items)


def rate_record(model: Model, proc: Process, species_id, site_ids) -> List[int]:
    """[nbyst, nvars, ncode, stack, (coord, npairs, (species, var) * npairs) * nbyst, code]"""
    from .program import pack_coord
    nr_vars, code, depth = compile_rate(model, proc)
    body: List[int] = []
    for b in proc.bystanders:
        pairs = []
        for spec in b.allowed_species:
            for flg in b.flag.split():
                pairs += [species_id(spec), nr_vars.index("nr_%s_%s" % (spec, flg))]
        o = b.coord.offset
        body += [pack_coord(o[0], o[1], o[2], site_ids[(b.coord.layer, b.coord.name)]), len(pairs) // 2] + pairs
    return [len(proc.bystanders), len(nr_vars), len(code), depth] + body + code


def user_parameters(model: Model) -> List[str]:
    """userpar order: parameters sorted by name (io:2705-2714)."""
    return sorted(p.name for p in model.parameters)


def user_parameter_values(model: Model, overrides: Optional[Dict[str, object]] = None) -> List[float]:
    """update_user_parameter values as kmos.run sets them (kmos/run/__init__.py:2416-2427):
    each parameter's value (its first word) evaluated as a rate expression."""
    params = {p.name: {"value": p.value} for p in model.parameters}
    for k, v in (overrides or {}).items():
        params[k] = {"value": v}
    return [float(R.evaluate_rate_expression(str(params[n]["value"]).split(" ")[0], params))
            for n in user_parameters(model)]
