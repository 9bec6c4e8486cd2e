"""Host-side evaluation of kmos rate-constant expressions.

kmos evaluates each process's ``rate_constant`` string in Python before it calls
``base.set_rate_const`` (kmos/__init__.py:67-190, kmos/run/__init__.py:2369-2437):
``beta`` is textually replaced by ``(1/(kboltzmann*T))``; the tokens ``sqrt exp sin cos
pi pow log`` become ``math.*``; unit names become their CODATA-2010 values
(kmos/units.py); ``m_<formula>`` becomes the summed atomic mass in u; parameters are
substituted by their (string) values, with unit names inside those values expanded
as well; the result is ``eval``-ed.  The engine only sees the resulting FP64 numbers.

The constant values below are the ones kmos uses (CODATA 2010) so that the same
expression yields the same double.  Atomic masses are the IUPAC conventional atomic
weights that ASE's ``atomic_masses`` table carries for the elements kmos models use.
Chemical potentials ``mu_<species>`` need JANAF tables that are not shipped here: they
can be given as parameters; otherwise they evaluate to 0, as kmos does for species it
has no table for.
"""
from __future__ import annotations

import io
import math
import re
import tokenize
import warnings
from typing import Dict, List, Mapping

# CODATA 2010 values, as in kmos/units.py
UNITS = {
    "pi": 3.14159265358979323846,
    "c": 2.99792458e8,
    "h": 6.62606957e-34,
    "hbar": 1.054571726e-34,
    "eV": 1.602176565e-19,
    "kboltzmann": 1.3806488e-23,
    "umass": 1.660538921e-27,
    "angstrom": 1.0e-10,
    "bar": 1.0e5,
}
UNIT_KEYS = ["pi", "c", "h", "hbar", "eV", "kboltzmann", "umass", "angstrom", "bar"]

ATOMIC_MASSES = {
    "H": 1.008, "He": 4.002602, "Li": 6.94, "Be": 9.0121831, "B": 10.81, "C": 12.011,
    "N": 14.007, "O": 15.999, "F": 18.998403163, "Ne": 20.1797, "Na": 22.98976928,
    "Mg": 24.305, "Al": 26.9815385, "Si": 28.085, "P": 30.973761998, "S": 32.06,
    "Cl": 35.45, "Ar": 39.948, "K": 39.0983, "Ca": 40.078, "Ti": 47.867, "Fe": 55.845,
    "Co": 58.933194, "Ni": 58.6934, "Cu": 63.546, "Zn": 65.38, "Ru": 101.07,
    "Rh": 102.9055, "Pd": 106.42, "Ag": 107.8682, "Ir": 192.217, "Pt": 195.084,
    "Au": 196.966569,
}

_MATH = ["sqrt", "exp", "sin", "cos", "pi", "pow", "log"]


def _formula_symbols(formula: str) -> List[str]:
    """Expand a chemical formula such as ``O2`` or ``CO`` into element symbols."""
    out = []
    for sym, count in re.findall(r"([A-Z][a-z]?)(\d*)", formula):
        out.extend([sym] * (int(count) if count else 1))
    if "".join(re.findall(r"[A-Z][a-z]?\d*", formula)) != formula:
        raise ValueError("cannot parse formula %r" % formula)
    return out


def evaluate_rate_expression(expr: str, parameters: Mapping[str, Mapping[str, object]] = None) -> float:
    """Evaluate one rate expression the way kmos does.  ``parameters`` maps names to
    ``{"value": v}`` (kmc_settings.py layout) or directly to values."""
    parameters = parameters or {}
    if not expr:
        return 0.0
    expr = expr.replace("beta", "(1/(kboltzmann*T))")
    toks = list(tokenize.generate_tokens(io.StringIO(expr).readline))
    out = []
    for kind, tok, _s, _e, _l in toks:
        if tok in _MATH:
            out.append((kind, "math." + tok))
        elif tok in UNITS:
            out.append((kind, str(UNITS[tok])))
        elif tok.startswith("m_"):
            syms = _formula_symbols("_".join(tok.split("_")[1:]))
            out.append((kind, "%s" % sum(ATOMIC_MASSES[s] for s in syms)))
        elif tok.startswith("mu_") and tok not in parameters:
            warnings.warn("no chemical potential table for %s; using 0" % tok)
            out.append((kind, "0"))
        elif tok in parameters:
            value = parameters[tok]
            value = value["value"] if isinstance(value, Mapping) else value
            text = str(value)
            for unit in UNIT_KEYS:
                text = text.replace(unit, "%s" % UNITS[unit])
            out.append((kind, text))
        else:
            out.append((kind, tok))
    code = tokenize.untokenize(out)
    return float(eval(code, {"__builtins__": {}, "math": math}))


def model_rates(model, parameters: Dict[str, object] = None) -> List[float]:
    """Rate constants of every process of ``model`` (process order), with the model's
    parameters overridden by ``parameters``."""
    params = {p.name: {"value": p.value} for p in model.parameters}
    for k, v in (parameters or {}).items():
        params[k] = {"value": v}
    rates = []
    for p in model.processes:
        r = evaluate_rate_expression(p.rate_constant, params)
        if r < 0:
            raise ValueError("%s: negative rate constant %r" % (p.name, r))
        rates.append(r)
    return rates
