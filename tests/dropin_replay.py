"""Recording and replaying the calls kmos.run makes on the f2py module ``kmc_model``.

tests/golden/make_kmc_model_run.py runs the reference's own ``kmos.run.KMC_Model``
(kmos/run/__init__.py) over this package's drop-in module, with every access to the
module's ``base`` / ``lattice`` / ``proclist`` objects going through a ``Recorder``: the
log holds each call with its arguments and result (and each constant read) in the order
the reference's code made them.  ``replay`` makes the same calls on a freshly configured
drop-in and compares every result, so a log recorded with the CPU oracle as the engine
checks the GPU engine against the reference's code path call by call.

``OracleTrajectory`` is the drop-in's engine interface (kmos_gb300.engine.Trajectory)
served by the oracle: test infrastructure, used to record logs without a GPU.
"""
from __future__ import annotations

import math

import numpy as np

from kmos_gb300 import engine as E
from oracle import oracle as O

RTOL = 1e-12  # kmc_time, kmc_time_step and integ_rates: device log() against glibc's


class OracleTrajectory:
    """engine.Trajectory's interface for one oracle trajectory (test only)."""

    def __init__(self, program, size, layer: int = 0, seed: int = 1, rng: int = E.RNG_GFORTRAN, traj: int = 0):
        self.o = O.Oracle(program, size, layer=layer, seed=seed, rng=rng, traj=traj)
        self.P, self.V, self.spuck, self.nspecies = self.o.P, self.o.V, self.o.spuck, self.o.nspecies

    def close(self):
        self.o = None

    def set_rate_const(self, proc, rate):
        O.lib().oracle_set_rate_const(self.o.h, int(proc), float(rate))

    def update_accum_rate(self):
        self.o.update_accum_rate()

    def update_integ_rate(self):
        self.o.update_integ_rate()

    def do_kmc_steps(self, n):
        self.o.do_kmc_steps(int(n))

    def get_next_kmc_step(self):
        return self.o.get_next_kmc_step()

    def run_proc_nr(self, proc, site):
        self.o.run_proc_nr(int(proc), int(site))

    def touchup(self, site):
        self.o.touchup(int(site))

    def touchup_many(self, sites):
        for s in sites:
            self.o.touchup(int(s))

    def get_species(self, site):
        return self.o.get_species(int(site))

    def replace_species(self, site, old, new):
        self.o.replace_species(int(site), int(old), int(new))

    @property
    def kmc_time(self):
        return self.o.kmc_time

    @property
    def kmc_time_step(self):
        return self.o.kmc_time_step

    @property
    def kmc_step(self):
        return self.o.kmc_step

    @property
    def walltime(self):
        return 0.0

    def procstat(self):
        return self.o.procstat()

    def integ_rates(self):
        return self.o.integ_rates()

    def rates(self):
        return self.o.rates()

    def accum_rates(self):
        return self.o.accum_rates()

    def nr_of_sites(self):
        return self.o.nr_of_sites()

    def avail_site(self, proc, idx, sw):
        return O.lib().oracle_get_avail_site(self.o.h, int(proc), int(idx), int(sw))

    def occupation(self):
        return self.o.occupation()


# ------------------------------------------------------------------ JSON-safe values
def enc(v):
    if isinstance(v, np.ndarray):
        return {"nd": enc(v.tolist()), "dtype": str(v.dtype)}
    if isinstance(v, (np.bool_, bool)):
        return bool(v)
    if isinstance(v, (np.integer, int)):
        return int(v)
    if isinstance(v, (np.floating, float)):
        f = float(v)
        return {"f": repr(f)} if not math.isfinite(f) else f
    if isinstance(v, tuple):
        return {"tuple": [enc(x) for x in v]}
    if isinstance(v, list):
        return [enc(x) for x in v]
    if isinstance(v, str) or v is None:
        return v
    return {"repr": repr(v)}


def dec(v):
    if isinstance(v, dict):
        if "nd" in v:
            return np.array(dec(v["nd"]), dtype=v["dtype"])
        if "tuple" in v:
            return tuple(dec(x) for x in v["tuple"])
        if "f" in v:
            return float(v["f"])
        return v
    if isinstance(v, list):
        return [dec(x) for x in v]
    return v


class Recorder:
    """Forwards attribute access to ``target`` and logs it into ``log``."""

    def __init__(self, name, target, log):
        object.__setattr__(self, "_name", name)
        object.__setattr__(self, "_target", target)
        object.__setattr__(self, "_log", log)

    def __dir__(self):
        return dir(self._target)

    def __getattr__(self, attr):
        v = getattr(self._target, attr)
        if callable(v):
            def call(*args):
                r = v(*args)
                self._log.append({"ns": self._name, "op": "call", "attr": attr, "args": enc(list(args)),
                                  "result": enc(r)})
                return r
            return call
        self._log.append({"ns": self._name, "op": "get", "attr": attr, "value": enc(v)})
        return v

    def __setattr__(self, attr, value):
        self._log.append({"ns": self._name, "op": "set", "attr": attr, "value": enc(value)})
        setattr(self._target, attr, value)


# ------------------------------------------------------------------ replay
def same(got, want, where):
    """Exact for integers, booleans and strings; within RTOL for floats."""
    if isinstance(want, np.ndarray):
        got = np.asarray(got)
        assert got.shape == want.shape, where
        if want.dtype.kind == "f":
            np.testing.assert_allclose(got, want, rtol=RTOL, atol=0, err_msg=where)
        else:
            np.testing.assert_array_equal(got, want, err_msg=where)
    elif isinstance(want, (tuple, list)):
        assert len(got) == len(want), where
        for g, w in zip(got, want):
            same(g, w, where)
    elif isinstance(want, float):
        assert got == want or abs(float(got) - want) <= RTOL * abs(want), "%s: %r != %r" % (where, got, want)
    else:
        assert got == want, "%s: %r != %r" % (where, got, want)


def replay(log, namespaces):
    """Makes every logged call on ``namespaces`` ({'base': ..., 'lattice': ..., 'proclist':
    ...}) and compares each result and constant with the log."""
    for k, e in enumerate(log):
        obj = namespaces[e["ns"]]
        where = "call %d: %s.%s" % (k, e["ns"], e["attr"])
        if e["op"] == "get":
            same(getattr(obj, e["attr"]), dec(e["value"]), where)
        elif e["op"] == "set":
            setattr(obj, e["attr"], dec(e["value"]))
        else:
            r = getattr(obj, e["attr"])(*dec(e["args"]))
            same(r, dec(e["result"]), where)
