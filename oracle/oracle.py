"""ctypes front end of the CPU oracle (``kmc_oracle.c``).

TEST INFRASTRUCTURE ONLY: tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline use this module as the oracle.  The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "kmc_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

RNG_GFORTRAN = 0
RNG_PHILOX = 1

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-O2 -ffp-contract=off, no FMA contraction)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
                               "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
        P32 = ctypes.POINTER(ctypes.c_int32)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [P32, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    i32, ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(ctypes.c_int)]
        L.oracle_destroy.argtypes = [vp]
        for name in ("oracle_run_proc_nr",):
            getattr(L, name).argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.oracle_touchup.argtypes = [vp, ctypes.c_int]
        L.oracle_set_rate_const.argtypes = [vp, ctypes.c_int, dbl]
        L.oracle_update_accum_rate.argtypes = [vp]
        L.oracle_update_integ_rate.argtypes = [vp]
        L.oracle_do_kmc_steps.argtypes = [vp, i64]
        L.oracle_get_next_kmc_step.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.oracle_trace_steps.argtypes = [vp, i64, P32]
        L.oracle_replace_species.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        for name, res in (("oracle_get_species", ctypes.c_int), ("oracle_get_volume", ctypes.c_int)):
            getattr(L, name).restype = res
        L.oracle_get_species.argtypes = [vp, ctypes.c_int]
        L.oracle_get_volume.argtypes = [vp]
        L.oracle_get_nrofsites.argtypes = [vp, ctypes.c_int]
        L.oracle_get_avail_site.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        for name in ("oracle_get_kmc_time", "oracle_get_kmc_time_step"):
            getattr(L, name).restype = dbl
            getattr(L, name).argtypes = [vp]
        L.oracle_get_kmc_step.restype = i64
        L.oracle_get_kmc_step.argtypes = [vp]
        for name in ("oracle_get_rate", "oracle_get_accum_rate", "oracle_get_integ_rate"):
            getattr(L, name).restype = dbl
            getattr(L, name).argtypes = [vp, ctypes.c_int]
        L.oracle_get_procstat.restype = i64
        L.oracle_get_procstat.argtypes = [vp, ctypes.c_int]
        L.oracle_get_counters.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(i64)]
        L.oracle_reset_counters.argtypes = [vp]
        L.oracle_export.argtypes = [vp, P32, P32, P32, P32, ctypes.POINTER(i64), ctypes.POINTER(dbl)]
        L.oracle_get_occupation.argtypes = [vp, ctypes.c_int, ctypes.POINTER(dbl)]
        L.oracle_philox.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
        L.oracle_draws.argtypes = [vp, i64, ctypes.POINTER(dbl)]
        L.oracle_rebuild_tables.argtypes = [vp, P32]
        L.oracle_set_user_parameter.argtypes = [vp, ctypes.c_int, dbl]
        L.oracle_recalculate_rates_matrix.argtypes = [vp]
        L.oracle_get_rates_matrix.restype = dbl
        L.oracle_get_rates_matrix.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def _p32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class OracleError(RuntimeError):
    pass


class Oracle:
    """One trajectory of the oracle.  ``program`` is a ``kmos_gb300.program.Program``
    (or its int32 word array)."""

    def __init__(self, program, size, layer=0, seed=1, rng=RNG_GFORTRAN, traj=0):
        words = np.ascontiguousarray(getattr(program, "words", program), dtype=np.int32)
        self._words = words
        size = list(size) + [1] * (3 - len(size))
        st = ctypes.c_int(0)
        L = lib()
        self.h = L.oracle_create(_p32(words), len(words), size[0], size[1], size[2], layer,
                                 int(np.int32(seed)), rng, traj, ctypes.byref(st))
        if not self.h:
            raise OracleError("oracle_create failed")
        if st.value:
            raise OracleError("initialize_state failed with %d" % st.value)
        self.P = int(words[3])
        self.nspecies = int(words[4])
        self.spuck = int(words[6])
        self.size = size
        self.V = L.oracle_get_volume(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def _check(self, st):
        if st:
            raise OracleError("oracle error %d" % st)

    def set_rates(self, rates):
        for p, r in enumerate(rates, start=1):
            lib().oracle_set_rate_const(self.h, p, float(r))

    def update_accum_rate(self):
        lib().oracle_update_accum_rate(self.h)

    def update_integ_rate(self):
        lib().oracle_update_integ_rate(self.h)

    # otf backend
    def set_user_parameters(self, values):
        for k, v in enumerate(values, start=1):
            lib().oracle_set_user_parameter(self.h, k, float(v))

    def recalculate_rates_matrix(self):
        self._check(lib().oracle_recalculate_rates_matrix(self.h))

    def rates_matrix(self):
        """[P][V+1]: rates_matrix(p, i) of list position i (index 0 unused), and the
        process total rates_matrix(p, V+1) as a separate [P] vector."""
        L, V = lib(), self.V
        out = np.zeros((self.P, V + 1))
        ns = self.nr_of_sites()
        for p in range(1, self.P + 1):
            for i in range(1, int(ns[p - 1]) + 1):
                out[p - 1, i] = L.oracle_get_rates_matrix(self.h, p, i)
        tot = np.array([L.oracle_get_rates_matrix(self.h, p, V + 1) for p in range(1, self.P + 1)])
        return out, tot

    def do_kmc_steps(self, n):
        self._check(lib().oracle_do_kmc_steps(self.h, int(n)))

    def trace(self, n):
        out = np.zeros(2 * n, dtype=np.int32)
        self._check(lib().oracle_trace_steps(self.h, int(n), _p32(out)))
        return out.reshape(n, 2)

    def get_next_kmc_step(self):
        p, s = ctypes.c_int(), ctypes.c_int()
        self._check(lib().oracle_get_next_kmc_step(self.h, ctypes.byref(p), ctypes.byref(s)))
        return p.value, s.value

    def run_proc_nr(self, proc, site):
        self._check(lib().oracle_run_proc_nr(self.h, proc, site))

    def touchup(self, site):
        self._check(lib().oracle_touchup(self.h, site))

    def replace_species(self, site, old, new):
        self._check(lib().oracle_replace_species(self.h, site, old, new))

    def get_species(self, site):
        return lib().oracle_get_species(self.h, site)

    @property
    def kmc_time(self):
        return lib().oracle_get_kmc_time(self.h)

    @property
    def kmc_time_step(self):
        return lib().oracle_get_kmc_time_step(self.h)

    @property
    def kmc_step(self):
        return lib().oracle_get_kmc_step(self.h)

    def procstat(self):
        return np.array([lib().oracle_get_procstat(self.h, p) for p in range(1, self.P + 1)], dtype=np.int64)

    def integ_rates(self):
        return np.array([lib().oracle_get_integ_rate(self.h, p) for p in range(1, self.P + 1)])

    def rates(self):
        return np.array([lib().oracle_get_rate(self.h, p) for p in range(1, self.P + 1)])

    def accum_rates(self):
        return np.array([lib().oracle_get_accum_rate(self.h, p) for p in range(1, self.P + 1)])

    def nr_of_sites(self):
        return np.array([lib().oracle_get_nrofsites(self.h, p) for p in range(1, self.P + 1)], dtype=np.int32)

    def counters(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        lib().oracle_get_counters(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def reset_counters(self):
        lib().oracle_reset_counters(self.h)

    def export(self):
        V, P = self.V, self.P
        lat = np.zeros(V, np.int32)
        as1 = np.zeros(P * (V + 1), np.int32)
        as2 = np.zeros(P * (V + 1), np.int32)
        ns = np.zeros(P, np.int32)
        ps = np.zeros(P, np.int64)
        ig = np.zeros(P, np.float64)
        lib().oracle_export(self.h, _p32(lat), _p32(as1), _p32(as2), _p32(ns),
                            ps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                            ig.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return dict(lattice=lat, as1=as1.reshape(P, V + 1), as2=as2.reshape(P, V + 1), nsites=ns,
                    procstat=ps, integ=ig)

    def rebuild_tables(self, lattice):
        """Sets the lattice and derives every table from it by touch-ups
        (oracle_rebuild_tables); returns export()."""
        lat = np.ascontiguousarray(lattice, dtype=np.int32)
        self._check(lib().oracle_rebuild_tables(self.h, _p32(lat)))
        return self.export()

    def occupation(self, nspecies_out=None):
        ns = self.nspecies if nspecies_out is None else nspecies_out
        out = np.zeros(ns * self.spuck)
        lib().oracle_get_occupation(self.h, ns, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out.reshape(ns, self.spuck)

    def draws(self, n):
        out = np.zeros(3 * n)
        lib().oracle_draws(self.h, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out.reshape(n, 3)


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().oracle_philox(c, k, o)
    return list(o)
