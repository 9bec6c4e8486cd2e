"""ctypes binding of ``libkmcgb300.so`` (include/kmc_gb300.h).

:class:`Trajectory` is one trajectory behind the f2py-style module interface (the plain
drop-in); :class:`Pool` holds many resident trajectories for batching and serving.
There is no CPU fallback: if the library or a CUDA device is missing, calls raise.
"""
from __future__ import annotations

import ctypes
import os
import struct
from typing import Iterable, List, Optional, Sequence

import numpy as np

from . import build as _build

KMC_OK = 0
ERRORS = {
    1: "bad argument",
    2: "replace_species: wrong species on site",
    3: "dead lock: no process available",
    4: "avail_sites inconsistency",
    5: "malformed model program",
    6: "device arena full",
    7: "CUDA error",
    8: "cancelled",
    9: "no CUDA device",
}
RNG_GFORTRAN = 0
RNG_PHILOX = 1

# Every function the header declares: name -> (restype, argtypes)
_vp, _i32, _i64, _dbl, _u32, _sz = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_uint32, ctypes.c_size_t
_P = ctypes.POINTER
_p32, _p64, _pd, _pu32 = _P(_i32), _P(_i64), _P(_dbl), _P(_u32)
SIGNATURES = {
    "kmc_last_error": (ctypes.c_char_p, []),
    "kmc_version": (ctypes.c_char_p, []),
    "kmc_check_program": (_i32, [_p32, _i32]),
    "kmc_check_image": (_i32, [_p32, _i32, _vp, _sz]),
    "kmc_create": (_i32, [_p32, _i32, _p32, _i32, _i32, _i32, _u32, _P(_vp)]),
    "kmc_destroy": (_i32, [_vp]),
    "kmc_set_rate_const": (_i32, [_vp, _i32, _dbl]),
    "kmc_update_accum_rate": (_i32, [_vp]),
    "kmc_update_integ_rate": (_i32, [_vp]),
    "kmc_do_steps": (_i32, [_vp, _i64]),
    "kmc_trace_steps": (_i32, [_vp, _i64, _p32]),
    "kmc_get_next_step": (_i32, [_vp, _p32, _p32]),
    "kmc_run_proc_nr": (_i32, [_vp, _i32, _i32]),
    "kmc_touchup": (_i32, [_vp, _i32]),
    "kmc_touchup_many": (_i32, [_vp, _p32, _i32]),
    "kmc_get_species": (_i32, [_vp, _i32, _p32]),
    "kmc_replace_species": (_i32, [_vp, _i32, _i32, _i32]),
    "kmc_get_kmc_time": (_i32, [_vp, _pd]),
    "kmc_set_kmc_time": (_i32, [_vp, _dbl]),
    "kmc_get_kmc_time_step": (_i32, [_vp, _pd]),
    "kmc_get_kmc_step": (_i32, [_vp, _p64]),
    "kmc_get_volume": (_i32, [_vp, _p32]),
    "kmc_get_nr_of_proc": (_i32, [_vp, _p32]),
    "kmc_get_procstat": (_i32, [_vp, _p64]),
    "kmc_get_integ_rates": (_i32, [_vp, _pd]),
    "kmc_get_rates": (_i32, [_vp, _pd]),
    "kmc_get_accum_rates": (_i32, [_vp, _pd]),
    "kmc_get_nr_of_sites": (_i32, [_vp, _p32]),
    "kmc_get_avail_site": (_i32, [_vp, _i32, _i32, _i32, _p32]),
    "kmc_get_lattice": (_i32, [_vp, _p32]),
    "kmc_get_tables": (_i32, [_vp, _p32, _p32]),
    "kmc_get_occupation": (_i32, [_vp, _pd]),
    "kmc_pool_create": (_i32, [_i32, _sz, _i32, _P(_vp)]),
    "kmc_pool_destroy": (_i32, [_vp]),
    "kmc_pool_add_model": (_i32, [_vp, _p32, _i32, _p32]),
    "kmc_pool_slot_bytes": (_i32, [_vp, _i32, _p32, _P(_sz)]),
    "kmc_pool_free_bytes": (_i32, [_vp, _P(_sz), _P(_sz)]),
    "kmc_pool_admit": (_i32, [_vp, _i32, _p32, _i32, _i32, _i32, _u32, _pd, _p32]),
    "kmc_pool_admit_many": (_i32, [_vp, _i32, _p32, _p32, _i32, _p32, _i32, _pu32, _pd, _p32, _p32]),
    "kmc_pool_release": (_i32, [_vp, _i32]),
    "kmc_pool_run": (_i32, [_vp, _p32, _p64, _i32]),
    "kmc_pool_run_graph": (_i32, [_vp, _p32, _i64, _i32]),
    "kmc_pool_sync": (_i32, [_vp]),
    "kmc_pool_cancel": (_i32, [_vp]),
    "kmc_pool_get_status": (_i32, [_vp, _i32, _p32]),
    "kmc_pool_get_clock": (_i32, [_vp, _i32, _pd, _p64]),
    "kmc_pool_get_procstat": (_i32, [_vp, _i32, _p64]),
    "kmc_pool_get_integ_rates": (_i32, [_vp, _i32, _pd]),
    "kmc_pool_get_nr_of_sites": (_i32, [_vp, _i32, _p32]),
    "kmc_pool_get_lattice": (_i32, [_vp, _i32, _p32]),
    "kmc_pool_get_tables": (_i32, [_vp, _i32, _p32, _p32]),
    "kmc_pool_set_rates": (_i32, [_vp, _i32, _pd]),
    "kmc_pool_occupation_counts": (_i32, [_vp, _p32, _i32, _i32, _p64]),
    "kmc_pool_occupation_counts_static": (_i32, [_vp, _p32, _i32, _i32, _p64]),
    "kmc_pool_set_trajectories_per_warp": (_i32, [_vp, _i32]),
    "kmc_pool_set_tables_on_chip": (_i32, [_vp, _i32]),
    "kmc_pool_set_solo": (_i32, [_vp, _i32]),
    "kmc_pool_get_results": (_i32, [_vp, _p32, _i32, _i32, _p64, _pd, _pd, _p64, _p32]),
    "kmc_pool_set_launch": (_i32, [_vp, _i32, _i32]),
    "kmc_pool_set_fast_path": (_i32, [_vp, _i32]),
    "kmc_pool_set_table_placement": (_i32, [_vp, _i32]),
    "kmc_pool_last_kernel_ms": (_i32, [_vp, _P(ctypes.c_float)]),
    "kmc_pool_timer_start": (_i32, [_vp]),
    "kmc_pool_timer_stop": (_i32, [_vp, _P(ctypes.c_float)]),
    "kmc_pool_launch_count": (_i32, [_vp, _p64]),
    "kmc_pool_phase_cycles": (_i32, [_vp, _P(ctypes.c_uint64), _i32]),
    "kmc_pool_save_state": (_i32, [_vp, _i32, _vp, _sz, _P(_sz)]),
    "kmc_pool_restore_state": (_i32, [_vp, _i32, _vp, _sz, _p32]),
    "kmc_save_state": (_i32, [_vp, _vp, _sz, _P(_sz)]),
    "kmc_load_state": (_i32, [_vp, _vp, _sz]),
    "kmc_save_reload": (_i32, [_vp, ctypes.c_char_p]),
    "kmc_reload_info": (_i32, [ctypes.c_char_p, _p32, _p32, _p32]),
    "kmc_check_reload": (_i32, [_p32, _i32, _p32, ctypes.c_char_p]),
    "kmc_load_reload": (_i32, [_vp, ctypes.c_char_p]),
    "kmc_get_walltime": (_i32, [_vp, _pd]),
    "kmc_pool_sample_begin": (_i32, [_vp, _p32, _i32]),
    "kmc_pool_sample": (_i32, [_vp, _p32, _i32]),
    "kmc_pool_sample_end": (_i32, [_vp, _p32, _i32, _i32, _i32, _pd, _p64, _pd, _pd, _p64, _p32]),
    "kmc_pool_sample_run": (_i32, [_vp, _p32, _i32, _i32, _i64, _i32, _i32, _pd, _p64, _pd, _pd, _p64, _p32]),
    "kmc_otf_check_program": (_i32, [_p32, _i32]),
    "kmc_otf_create": (_i32, [_p32, _i32, _p32, _i32, _i32, _i32, _i32, _u32, _P(_vp)]),
    "kmc_otf_destroy": (_i32, [_vp]),
    "kmc_otf_set_rate_const": (_i32, [_vp, _i32, _dbl]),
    "kmc_otf_set_user_parameter": (_i32, [_vp, _i32, _dbl]),
    "kmc_otf_recalculate_rates_matrix": (_i32, [_vp]),
    "kmc_otf_update_accum_rate": (_i32, [_vp]),
    "kmc_otf_update_integ_rate": (_i32, [_vp]),
    "kmc_otf_do_steps": (_i32, [_vp, _i64]),
    "kmc_otf_trace_steps": (_i32, [_vp, _i32, _i64, _p32]),
    "kmc_otf_get_next_step": (_i32, [_vp, _i32, _p32, _p32]),
    "kmc_otf_run_proc_nr": (_i32, [_vp, _i32, _i32, _i32]),
    "kmc_otf_get_state": (_i32, [_vp, _i32, _p32, _p32, _p32, _p32, _p64, _pd, _pd, _pd, _pd, _pd, _p64]),
    "kmc_otf_last_kernel_ms": (_i32, [_vp, _P(ctypes.c_float)]),
    "kmc_otf_launch_count": (_i32, [_vp, _p64]),
    "kmc_otf_phase_cycles": (_i32, [_vp, ctypes.POINTER(ctypes.c_uint64), _i32]),
    "kmc_otf_set_rate_tables": (_i32, [_vp, _i32]),
    "kmc_otf_set_kmc_time": (_i32, [_vp, _i32, _dbl]),
    "kmc_otf_replace_species": (_i32, [_vp, _i32, _i32, _i32, _i32]),
    "kmc_otf_touchup_cells": (_i32, [_vp, _i32, _i32, _p32]),
    "kmc_otf_set_state": (_i32, [_vp, _i32, _p32, _p32, _p32, _p64, _pd, _pd, _i64]),
    "kmc_otf_save_reload": (_i32, [_vp, _i32, ctypes.c_char_p, _dbl]),
    "kmc_otf_load_reload": (_i32, [_vp, _i32, ctypes.c_char_p, _pd]),
    "kmc_otf_get_rate_consts": (_i32, [_vp, _pd]),
    "kmc_otf_set_constant_rate_sums": (_i32, [_vp, _i32]),
    "kmc_otf_rate_table_entries": (_i32, [_vp, _p32]),
}

_lib = None


class KMCError(RuntimeError):
    def __init__(self, code: int, text: str = ""):
        self.code = code
        super().__init__("%s (status %d)%s" % (ERRORS.get(code, "error"), code, ": " + text if text else ""))


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True, path: Optional[str] = None):
    """Loads the engine library (building it first if it is missing or stale).  ``path``,
    or else the environment variable KMC_GB300_LIB, selects another build of the same
    C-ABI (the phase-timing or the KMC_DEBUG build)."""
    global _lib
    if _lib is None:
        path = path or os.environ.get("KMC_GB300_LIB") or None
        if path is None and build_if_missing and _build.needs_build():
            _build.build()
        lib = path or _build.LIB
        if not os.path.exists(lib):
            raise RuntimeError("kmc engine library %s is missing; run kmos_gb300.build.build()" % lib)
        L = ctypes.CDLL(lib)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != KMC_OK:
        raise KMCError(rc, load().kmc_last_error().decode(errors="replace"))


def _a32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _dims3(size: Sequence[int]) -> np.ndarray:
    size = [int(s) for s in size] + [1] * (3 - len(size))
    return _a32(size[:3])


class Trajectory:
    """One trajectory on the GPU (``kmc_create``).  ``program`` is a compiled
    :class:`~kmos_gb300.program.Program` or its int32 words."""

    def __init__(self, program, size, layer: int = 0, seed: int = 1, rng: int = RNG_GFORTRAN, traj: int = 0):
        L = load()
        words = _a32(getattr(program, "words", program))
        self._words = words
        dims = _dims3(size)
        h = ctypes.c_void_p()
        _check(L.kmc_create(_ptr(words, _i32), len(words), _ptr(dims, _i32), int(layer),
                            int(np.int32(seed)), int(rng), int(traj) & 0xFFFFFFFF, ctypes.byref(h)))
        self.h = h
        self.P = int(words[3])
        self.nspecies = int(words[4])
        self.spuck = int(words[6])
        self.size = [int(x) for x in dims]
        v = _i32()
        _check(L.kmc_get_volume(self.h, ctypes.byref(v)))
        self.V = v.value

    def close(self):
        if getattr(self, "h", None):
            load().kmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --- base ---
    def set_rate_const(self, proc: int, rate: float):
        _check(load().kmc_set_rate_const(self.h, int(proc), float(rate)))

    def set_rates(self, rates: Iterable[float]):
        for p, r in enumerate(rates, start=1):
            self.set_rate_const(p, r)

    def update_accum_rate(self):
        _check(load().kmc_update_accum_rate(self.h))

    def update_integ_rate(self):
        _check(load().kmc_update_integ_rate(self.h))

    # --- proclist ---
    def do_kmc_steps(self, n: int):
        _check(load().kmc_do_steps(self.h, int(n)))

    def trace(self, n: int) -> np.ndarray:
        out = np.zeros(2 * int(n), dtype=np.int32)
        _check(load().kmc_trace_steps(self.h, int(n), _ptr(out, _i32)))
        return out.reshape(-1, 2)

    def get_next_kmc_step(self):
        p, s = _i32(), _i32()
        _check(load().kmc_get_next_step(self.h, ctypes.byref(p), ctypes.byref(s)))
        return p.value, s.value

    def run_proc_nr(self, proc: int, site: int):
        _check(load().kmc_run_proc_nr(self.h, int(proc), int(site)))

    def touchup(self, site: int):
        _check(load().kmc_touchup(self.h, int(site)))

    def touchup_many(self, sites):
        """Touch-ups of many sites in order, one launch (``kmc_touchup_many``)."""
        sites = np.ascontiguousarray(sites, dtype=np.int32)
        _check(load().kmc_touchup_many(self.h, _ptr(sites, _i32), len(sites)))

    def get_species(self, site: int) -> int:
        s = _i32()
        _check(load().kmc_get_species(self.h, int(site), ctypes.byref(s)))
        return s.value

    def replace_species(self, site: int, old: int, new: int):
        _check(load().kmc_replace_species(self.h, int(site), int(old), int(new)))

    # --- getters ---
    @property
    def kmc_time(self) -> float:
        t = _dbl()
        _check(load().kmc_get_kmc_time(self.h, ctypes.byref(t)))
        return t.value

    @kmc_time.setter
    def kmc_time(self, t: float):
        _check(load().kmc_set_kmc_time(self.h, float(t)))

    @property
    def kmc_time_step(self) -> float:
        t = _dbl()
        _check(load().kmc_get_kmc_time_step(self.h, ctypes.byref(t)))
        return t.value

    @property
    def kmc_step(self) -> int:
        s = _i64()
        _check(load().kmc_get_kmc_step(self.h, ctypes.byref(s)))
        return s.value

    def _vec(self, fn, dtype, ctype, n=None):
        out = np.zeros(self.P if n is None else n, dtype=dtype)
        _check(fn(self.h, _ptr(out, ctype)))
        return out

    def procstat(self):
        return self._vec(load().kmc_get_procstat, np.int64, _i64)

    def integ_rates(self):
        return self._vec(load().kmc_get_integ_rates, np.float64, _dbl)

    def rates(self):
        return self._vec(load().kmc_get_rates, np.float64, _dbl)

    def accum_rates(self):
        return self._vec(load().kmc_get_accum_rates, np.float64, _dbl)

    def nr_of_sites(self):
        return self._vec(load().kmc_get_nr_of_sites, np.int32, _i32)

    def avail_site(self, proc: int, idx: int, sw: int) -> int:
        o = _i32()
        _check(load().kmc_get_avail_site(self.h, int(proc), int(idx), int(sw), ctypes.byref(o)))
        return o.value

    def lattice(self) -> np.ndarray:
        return self._vec(load().kmc_get_lattice, np.int32, _i32, self.V)

    def tables(self):
        as1 = np.zeros(self.P * (self.V + 1), np.int32)
        as2 = np.zeros(self.P * (self.V + 1), np.int32)
        _check(load().kmc_get_tables(self.h, _ptr(as1, _i32), _ptr(as2, _i32)))
        return as1.reshape(self.P, self.V + 1), as2.reshape(self.P, self.V + 1)

    def occupation(self) -> np.ndarray:
        out = np.zeros(self.nspecies * self.spuck)
        _check(load().kmc_get_occupation(self.h, _ptr(out, _dbl)))
        return out.reshape(self.nspecies, self.spuck)

    @property
    def walltime(self) -> float:
        t = _dbl()
        _check(load().kmc_get_walltime(self.h, ctypes.byref(t)))
        return t.value

    # --- saving and restoring ---
    def save_state(self) -> bytes:
        """Compact binary image of the trajectory (``kmc_save_state``)."""
        n = ctypes.c_size_t()
        _check(load().kmc_save_state(self.h, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        _check(load().kmc_save_state(self.h, buf, n.value, ctypes.byref(n)))
        return buf.raw[:n.value]

    def load_state(self, image: bytes):
        """Loads an image of the same model and system size (``kmc_load_state``)."""
        _check(load().kmc_load_state(self.h, image, len(image)))

    def save_reload(self, path: str):
        """base.save_system: writes ``path`` in the reference's .reload layout."""
        _check(load().kmc_save_reload(self.h, os.fsencode(path)))

    def load_reload(self, path: str):
        """Second pass of base.reload_system into this trajectory."""
        _check(load().kmc_load_reload(self.h, os.fsencode(path)))


def check_program(program) -> None:
    """Raises KMCError (KMC_ERR_PROGRAM) unless the engine accepts the model program
    (``kmc_check_program``; no GPU needed).  ``program``: a Program or its int32 words."""
    words = np.ascontiguousarray(getattr(program, "words", program), dtype=np.int32)
    _check(load().kmc_check_program(_ptr(words, _i32), len(words)))


def check_image(program, image: bytes) -> None:
    """Raises KMCError unless ``image`` (a state image, ``Pool.save_state``) would be
    accepted for ``program`` (``kmc_check_image``; no GPU needed)."""
    words = np.ascontiguousarray(getattr(program, "words", program), dtype=np.int32)
    buf = ctypes.create_string_buffer(bytes(image), len(image))
    _check(load().kmc_check_image(_ptr(words, _i32), len(words), ctypes.cast(buf, ctypes.c_void_p), len(image)))


def reload_info(path: str):
    """(nr_of_proc, volume, system size or None) of a .reload file (``kmc_reload_info``)."""
    P, V = _i32(), _i32()
    dims = np.zeros(3, np.int32)
    _check(load().kmc_reload_info(os.fsencode(path), ctypes.byref(P), ctypes.byref(V), _ptr(dims, _i32)))
    return P.value, V.value, (None if dims[0] == 0 else [int(d) for d in dims])


def check_reload(program, size, path: str) -> None:
    """Raises KMCError unless the .reload file at ``path`` would be accepted for
    ``program`` (lattice or otf) on a lattice of ``size`` (``kmc_check_reload``; no GPU
    needed)."""
    words = np.ascontiguousarray(getattr(program, "words", program), dtype=np.int32)
    dims = _dims3(size)
    _check(load().kmc_check_reload(_ptr(words, _i32), len(words), _ptr(dims, _i32), os.fsencode(path)))


class Pool:
    """Many resident trajectories in one device arena (``kmc_pool_*``)."""

    def __init__(self, arena_bytes: int, max_slots: int, device: int = 0):
        L = load()
        h = ctypes.c_void_p()
        _check(L.kmc_pool_create(int(device), int(arena_bytes), int(max_slots), ctypes.byref(h)))
        self.h = h
        self.models: List[np.ndarray] = []
        self.slot_model = {}
        self.slot_volume = {}

    def close(self):
        if getattr(self, "h", None):
            load().kmc_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_model(self, program) -> int:
        words = _a32(getattr(program, "words", program))
        mid = _i32()
        _check(load().kmc_pool_add_model(self.h, _ptr(words, _i32), len(words), ctypes.byref(mid)))
        self.models.append(words)
        return mid.value

    def nproc(self, model_id: int) -> int:
        return int(self.models[model_id][3])

    def slot_bytes(self, model_id: int, size) -> int:
        b = _sz()
        dims = _dims3(size)
        _check(load().kmc_pool_slot_bytes(self.h, int(model_id), _ptr(dims, _i32), ctypes.byref(b)))
        return b.value

    def free_bytes(self):
        t, l = _sz(), _sz()
        _check(load().kmc_pool_free_bytes(self.h, ctypes.byref(t), ctypes.byref(l)))
        return t.value, l.value

    def admit(self, model_id: int, size, rates, layer: int = 0, seed: int = 1, rng: int = RNG_PHILOX,
              traj: int = 0) -> int:
        return self.admit_many([model_id], [size], [rates], layer=layer, seeds=[seed], rng=rng, trajs=[traj])[0]

    def admit_many(self, model_ids, sizes, rates_list, layer: int = 0, seeds=None, rng: int = RNG_PHILOX,
                   trajs=None) -> List[int]:
        n = len(model_ids)
        mids = _a32(model_ids)
        dims = _a32(np.concatenate([_dims3(s) for s in sizes]))
        seeds = _a32(seeds if seeds is not None else [1] * n)
        trajs = np.ascontiguousarray(trajs if trajs is not None else np.arange(n), dtype=np.uint32)
        offs, flat = [], []
        for r in rates_list:
            offs.append(len(flat))
            flat.extend(float(x) for x in r)
        offs = _a32(offs)
        flat = np.ascontiguousarray(flat, dtype=np.float64)
        slots = np.zeros(n, np.int32)
        _check(load().kmc_pool_admit_many(self.h, n, _ptr(mids, _i32), _ptr(dims, _i32), int(layer),
                                          _ptr(seeds, _i32), int(rng), _ptr(trajs, _u32), _ptr(flat, _dbl),
                                          _ptr(offs, _i32), _ptr(slots, _i32)))
        for s, m, sz in zip(slots, model_ids, sizes):
            self.slot_model[int(s)] = int(m)
            d = _dims3(sz)
            self.slot_volume[int(s)] = int(d[0]) * int(d[1]) * int(d[2]) * int(self.models[int(m)][6])
        return [int(s) for s in slots]

    def release(self, slot: int):
        _check(load().kmc_pool_release(self.h, int(slot)))
        self.slot_model.pop(int(slot), None)
        self.slot_volume.pop(int(slot), None)

    def run(self, slots, steps, sync: bool = True):
        slots = _a32(slots)
        steps = np.ascontiguousarray(np.broadcast_to(np.asarray(steps, dtype=np.int64), slots.shape))
        _check(load().kmc_pool_run(self.h, _ptr(slots, _i32), _ptr(steps, _i64), len(slots)))
        if sync:
            self.sync()

    def run_graph(self, slots, steps: int, sync: bool = True):
        slots = _a32(slots)
        _check(load().kmc_pool_run_graph(self.h, _ptr(slots, _i32), int(steps), len(slots)))
        if sync:
            self.sync()

    def sync(self):
        _check(load().kmc_pool_sync(self.h))

    def cancel(self):
        _check(load().kmc_pool_cancel(self.h))

    def set_launch(self, warps_per_block: int = 0, blocks_per_sm: int = 0):
        _check(load().kmc_pool_set_launch(self.h, int(warps_per_block), int(blocks_per_sm)))

    def set_fast_path(self, enable: bool):
        _check(load().kmc_pool_set_fast_path(self.h, 1 if enable else 0))

    def set_trajectories_per_warp(self, n: int):
        """1: 32 lanes per trajectory; 2: two trajectories per warp, 16 lanes each."""
        _check(load().kmc_pool_set_trajectories_per_warp(self.h, int(n)))

    def set_solo(self, enable: bool):
        """Small launches of models with up to 8 processes: steps on one lane per trajectory."""
        _check(load().kmc_pool_set_solo(self.h, 1 if enable else 0))

    def set_tables_on_chip(self, enable: bool):
        """Lattice and avail_sites tables in shared memory for launches where they fit."""
        _check(load().kmc_pool_set_tables_on_chip(self.h, 1 if enable else 0))

    def set_table_placement(self, shared: bool):
        """Hot section (fast streams, nli tables) in shared memory (True) or read from
        global memory (False)."""
        _check(load().kmc_pool_set_table_placement(self.h, 1 if shared else 0))

    def last_kernel_ms(self) -> float:
        ms = ctypes.c_float()
        _check(load().kmc_pool_last_kernel_ms(self.h, ctypes.byref(ms)))
        return ms.value

    def timer_start(self):
        _check(load().kmc_pool_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = ctypes.c_float()
        _check(load().kmc_pool_timer_stop(self.h, ctypes.byref(ms)))
        return ms.value

    def phase_cycles(self, reset: bool = True) -> np.ndarray:
        """Per-phase cycle sums of the step kernel (library built with KMC_PHASE_TIMING)."""
        out = np.zeros(16, np.uint64)
        _check(load().kmc_pool_phase_cycles(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                            1 if reset else 0))
        return out

    def launch_count(self) -> int:
        c = _i64()
        _check(load().kmc_pool_launch_count(self.h, ctypes.byref(c)))
        return c.value

    def status(self, slot: int) -> int:
        s = _i32()
        _check(load().kmc_pool_get_status(self.h, int(slot), ctypes.byref(s)))
        return s.value

    def clock(self, slot: int):
        t, k = _dbl(), _i64()
        _check(load().kmc_pool_get_clock(self.h, int(slot), ctypes.byref(t), ctypes.byref(k)))
        return t.value, k.value

    def _pvec(self, fn, slot, dtype, ctype):
        out = np.zeros(self.nproc(self.slot_model[int(slot)]), dtype=dtype)
        _check(fn(self.h, int(slot), _ptr(out, ctype)))
        return out

    def procstat(self, slot):
        return self._pvec(load().kmc_pool_get_procstat, slot, np.int64, _i64)

    def integ_rates(self, slot):
        return self._pvec(load().kmc_pool_get_integ_rates, slot, np.float64, _dbl)

    def nr_of_sites(self, slot):
        return self._pvec(load().kmc_pool_get_nr_of_sites, slot, np.int32, _i32)

    def volume(self, slot) -> int:
        return self.slot_volume[int(slot)]

    def lattice(self, slot, volume: Optional[int] = None):
        out = np.zeros(self.volume(slot), np.int32)
        _check(load().kmc_pool_get_lattice(self.h, int(slot), _ptr(out, _i32)))
        return out

    def tables(self, slot, volume: Optional[int] = None):
        volume = self.volume(slot)
        P = self.nproc(self.slot_model[int(slot)])
        as1 = np.zeros(P * (volume + 1), np.int32)
        as2 = np.zeros(P * (volume + 1), np.int32)
        _check(load().kmc_pool_get_tables(self.h, int(slot), _ptr(as1, _i32), _ptr(as2, _i32)))
        return as1.reshape(P, volume + 1), as2.reshape(P, volume + 1)

    def set_rates(self, slot: int, rates):
        """New rate constants for a resident trajectory (``kmc_pool_set_rates``)."""
        r = np.ascontiguousarray(rates, dtype=np.float64)
        if len(r) != self.nproc(self.slot_model[int(slot)]):
            raise ValueError("one rate per process")
        _check(load().kmc_pool_set_rates(self.h, int(slot), _ptr(r, _dbl)))

    def results(self, slots, stride: int):
        """procstat [n, stride], integ [n, stride], kmc_time [n], kmc_step [n], status [n]
        of many slots, gathered on the device and copied back in one transfer."""
        slots = _a32(slots)
        n = len(slots)
        ps = np.zeros((n, stride), np.int64)
        ig = np.zeros((n, stride), np.float64)
        t = np.zeros(n, np.float64)
        k = np.zeros(n, np.int64)
        st = np.zeros(n, np.int32)
        _check(load().kmc_pool_get_results(self.h, _ptr(slots, _i32), n, int(stride), _ptr(ps, _i64), _ptr(ig, _dbl),
                                           _ptr(t, _dbl), _ptr(k, _i64), _ptr(st, _i32)))
        return ps, ig, t, k, st

    def occupation_counts_static(self, slots, stride: int) -> np.ndarray:
        """occupation_counts through the entry point that allocates no device memory
        (for callers that cannot allocate: a spent memory budget, or a section where an
        allocation would synchronise the device).  Its scratch is a fixed static array
        shared by every call: at most 4096 slots and 64 counters per slot, and calls that
        overlap on the GPU must be serialised by the caller."""
        slots = _a32(slots)
        out = np.zeros(len(slots) * stride, np.int64)
        _check(load().kmc_pool_occupation_counts_static(self.h, _ptr(slots, _i32), len(slots), int(stride),
                                                         _ptr(out, _i64)))
        return out.reshape(len(slots), stride)

    def occupation_counts(self, slots, stride: int) -> np.ndarray:
        slots = _a32(slots)
        out = np.zeros(len(slots) * stride, np.int64)
        _check(load().kmc_pool_occupation_counts(self.h, _ptr(slots, _i32), len(slots), int(stride), _ptr(out, _i64)))
        return out.reshape(len(slots), stride)

    # --- saving and restoring (base.save_system / reload_system) ---
    def save_state(self, slot: int) -> bytes:
        """Compact binary image of a resident trajectory (``kmc_pool_save_state``)."""
        n = ctypes.c_size_t()
        _check(load().kmc_pool_save_state(self.h, int(slot), None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        _check(load().kmc_pool_save_state(self.h, int(slot), buf, n.value, ctypes.byref(n)))
        return buf.raw[:n.value]

    def restore_state(self, model_id: int, image: bytes) -> int:
        """Admits a trajectory from an image of model ``model_id``; returns its slot."""
        slot = _i32()
        _check(load().kmc_pool_restore_state(self.h, int(model_id), image, len(image), ctypes.byref(slot)))
        s = slot.value
        self.slot_model[s] = int(model_id)
        self.slot_volume[s] = struct.unpack_from("<i", image, 44)[0]
        return s

    # --- on-device sampling (get_std_sampled_data) ---
    def sample_begin(self, slots):
        slots = _a32(slots)
        _check(load().kmc_pool_sample_begin(self.h, _ptr(slots, _i32), len(slots)))

    def sample(self, slots):
        slots = _a32(slots)
        _check(load().kmc_pool_sample(self.h, _ptr(slots, _i32), len(slots)))

    def _sample_out(self, slots):
        n = len(slots)
        occ_stride = max(int(self.models[self.slot_model[int(s)]][4]) * int(self.models[self.slot_model[int(s)]][6])
                         for s in slots)
        proc_stride = max(self.nproc(self.slot_model[int(s)]) for s in slots)
        return dict(occ=np.zeros((n, occ_stride)), dprocstat=np.zeros((n, proc_stride), np.int64),
                    dinteg=np.zeros((n, proc_stride)), times=np.zeros((n, 2)), steps=np.zeros(n, np.int64),
                    status=np.zeros(n, np.int32)), occ_stride, proc_stride

    def _out_args(self, out):
        return (_ptr(out["occ"], _dbl), _ptr(out["dprocstat"], _i64), _ptr(out["dinteg"], _dbl),
                _ptr(out["times"], _dbl), _ptr(out["steps"], _i64), _ptr(out["status"], _i32))

    def sample_end(self, slots) -> dict:
        """Ends the sampling records: per slot the kmc_time_step-weighted mean occupation
        ``occ`` ([nspecies*spuck]), ``dprocstat`` / ``dinteg`` since sample_begin,
        ``times`` (total_time, simulated_time), ``steps`` and ``status``."""
        slots = _a32(slots)
        out, os_, ps_ = self._sample_out(slots)
        _check(load().kmc_pool_sample_end(self.h, _ptr(slots, _i32), len(slots), os_, ps_, *self._out_args(out)))
        return out

    def sample_run(self, slots, samples: int, steps_per_sample: int) -> dict:
        """sample_begin, ``samples`` x (run ``steps_per_sample`` steps, sample), sample_end,
        queued on the device in one call."""
        slots = _a32(slots)
        out, os_, ps_ = self._sample_out(slots)
        _check(load().kmc_pool_sample_run(self.h, _ptr(slots, _i32), len(slots), int(samples), int(steps_per_sample),
                                          os_, ps_, *self._out_args(out)))
        return out


def check_otf_program(words) -> None:
    """The checks kmc_otf_create makes on an otf program, on the CPU."""
    w = _a32(getattr(words, "words", words))
    _check(load().kmc_otf_check_program(_ptr(w, _i32), len(w)))


class OtfBatch:
    """``ntraj`` independent trajectories of one otf program on the GPU (``kmc_otf_*``):
    trajectory t draws Philox numbers keyed (seed, traj0 + t), or all share the gfortran
    stream of ``seed``.  Rate constants and user parameters apply to every trajectory."""

    def __init__(self, program, size, ntraj: int = 1, layer: int = 0, seed: int = 1, rng: int = RNG_PHILOX,
                 traj0: int = 0):
        L = load()
        words = _a32(getattr(program, "words", program))
        self._words = words
        dims = _dims3(size)
        h = ctypes.c_void_p()
        _check(L.kmc_otf_create(_ptr(words, _i32), len(words), _ptr(dims, _i32), int(layer), int(ntraj),
                                int(np.int32(seed)), int(rng), int(traj0) & 0xFFFFFFFF, ctypes.byref(h)))
        self.h = h
        self.P = int(words[3])
        self.spuck = int(words[6])
        self.size = [int(x) for x in dims]
        self.V = int(np.prod(self.size)) * self.spuck
        self.ntraj = int(ntraj)

    def close(self):
        if getattr(self, "h", None):
            load().kmc_otf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_rate_const(self, proc: int, rate: float):
        _check(load().kmc_otf_set_rate_const(self.h, int(proc), float(rate)))

    def set_rates(self, rates: Iterable[float]):
        for p, r in enumerate(rates, start=1):
            self.set_rate_const(p, r)

    def set_user_parameter(self, k: int, value: float):
        _check(load().kmc_otf_set_user_parameter(self.h, int(k), float(value)))

    def set_user_parameters(self, values: Iterable[float]):
        for k, v in enumerate(values, start=1):
            self.set_user_parameter(k, v)

    def recalculate_rates_matrix(self):
        _check(load().kmc_otf_recalculate_rates_matrix(self.h))

    def update_accum_rate(self):
        _check(load().kmc_otf_update_accum_rate(self.h))

    def update_integ_rate(self):
        _check(load().kmc_otf_update_integ_rate(self.h))

    def do_kmc_steps(self, n: int):
        _check(load().kmc_otf_do_steps(self.h, int(n)))

    def trace(self, traj: int, n: int) -> np.ndarray:
        out = np.zeros(2 * int(n), dtype=np.int32)
        _check(load().kmc_otf_trace_steps(self.h, int(traj), int(n), _ptr(out, _i32)))
        return out.reshape(-1, 2)

    def get_next_kmc_step(self, traj: int = 0):
        p, s = _i32(), _i32()
        _check(load().kmc_otf_get_next_step(self.h, int(traj), ctypes.byref(p), ctypes.byref(s)))
        return p.value, s.value

    def run_proc_nr(self, proc: int, site: int, traj: int = 0):
        _check(load().kmc_otf_run_proc_nr(self.h, int(traj), int(proc), int(site)))

    def set_kmc_time(self, traj: int, t: float):
        _check(load().kmc_otf_set_kmc_time(self.h, int(traj), float(t)))

    def replace_species(self, traj: int, site: int, old: int, new: int):
        _check(load().kmc_otf_replace_species(self.h, int(traj), int(site), int(old), int(new)))

    def touchup_cells(self, traj: int, cells):
        """touchup_cell of each (x, y, z) in order, one launch (``kmc_otf_touchup_cells``)."""
        c = np.ascontiguousarray(np.asarray(cells, dtype=np.int32).reshape(-1, 3))
        _check(load().kmc_otf_touchup_cells(self.h, int(traj), len(c), _ptr(c, _i32)))

    def set_state(self, traj: int, lattice, as1, nsites, procstat, integ=None, kmc_time: float = 0.0,
                  kmc_time_step: float = 0.0, kmc_step: int = 0):
        """Uploads one trajectory's state (``kmc_otf_set_state``); as1 is [P][V+1]."""
        lat = _a32(lattice)
        a1 = _a32(np.asarray(as1).reshape(-1))
        ns = _a32(nsites)
        ps = np.ascontiguousarray(procstat, dtype=np.int64)
        ig = None if integ is None else np.ascontiguousarray(integ, dtype=np.float64)
        clock = np.array([kmc_time, kmc_time_step], dtype=np.float64)
        _check(load().kmc_otf_set_state(self.h, int(traj), _ptr(lat, _i32), _ptr(a1, _i32), _ptr(ns, _i32),
                                        _ptr(ps, _i64), None if ig is None else _ptr(ig, _dbl), _ptr(clock, _dbl),
                                        int(kmc_step)))

    def save_reload(self, traj: int, path: str, walltime: float = 0.0):
        _check(load().kmc_otf_save_reload(self.h, int(traj), os.fsencode(path), float(walltime)))

    def load_reload(self, traj: int, path: str) -> float:
        """Loads a .reload file into one trajectory; returns the file's walltime."""
        w = _dbl()
        _check(load().kmc_otf_load_reload(self.h, int(traj), os.fsencode(path), ctypes.byref(w)))
        return w.value

    def rate_consts(self) -> np.ndarray:
        out = np.zeros(self.P, np.float64)
        _check(load().kmc_otf_get_rate_consts(self.h, _ptr(out, _dbl)))
        return out

    STATE_FIELDS = ("lattice", "as1", "as2", "nsites", "procstat", "integ", "accum", "rates_matrix", "totals",
                    "clock")

    def state(self, traj: int = 0, fields: Optional[Sequence[str]] = None) -> dict:
        """lattice, as1, as2, nsites, procstat, integ, accum, rates_matrix ([P][V+1]),
        totals, kmc_time, kmc_time_step, kmc_step of one trajectory (``fields``: copy only
        those of STATE_FIELDS; "clock" is kmc_time, kmc_time_step and kmc_step)."""
        P, V = self.P, self.V
        want = set(self.STATE_FIELDS if fields is None else fields)
        shapes = {"lattice": (V, np.int32), "as1": (P * (V + 1), np.int32), "as2": (P * (V + 1), np.int32),
                  "nsites": (P, np.int32), "procstat": (P, np.int64), "integ": (P, np.float64),
                  "accum": (P, np.float64), "rates_matrix": (P * (V + 1), np.float64), "totals": (P, np.float64),
                  "clock": (2, np.float64)}
        ctype = {np.int32: _i32, np.int64: _i64, np.float64: _dbl}
        arrs = {k: np.zeros(n, dt) for k, (n, dt) in shapes.items() if k in want}
        ptr = {k: (_ptr(arrs[k], ctype[shapes[k][1]]) if k in arrs else None) for k in shapes}
        step = _i64()
        _check(load().kmc_otf_get_state(self.h, int(traj), ptr["lattice"], ptr["as1"], ptr["as2"], ptr["nsites"],
                                        ptr["procstat"], ptr["integ"], ptr["accum"], ptr["rates_matrix"],
                                        ptr["totals"], ptr["clock"], ctypes.byref(step) if "clock" in want else None))
        out = {}
        for k, a in arrs.items():
            if k in ("as1", "as2", "rates_matrix"):
                out[k] = a.reshape(P, V + 1)
            elif k == "clock":
                out.update(kmc_time=float(a[0]), kmc_time_step=float(a[1]), kmc_step=step.value)
            else:
                out[k] = a
        return out

    def last_kernel_ms(self) -> float:
        ms = ctypes.c_float()
        _check(load().kmc_otf_last_kernel_ms(self.h, ctypes.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        n = _i64()
        _check(load().kmc_otf_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def set_rate_tables(self, on: bool) -> None:
        """Rates looked up in per-process tables of every bystander-count combination
        (the default where the model has them) or evaluated by the rate programs."""
        _check(load().kmc_otf_set_rate_tables(self.h, 1 if on else 0))

    def set_constant_rate_sums(self, on: bool) -> None:
        """Running sums of constant-rate processes' lists from per-process tables (the
        default) or always re-summed."""
        _check(load().kmc_otf_set_constant_rate_sums(self.h, 1 if on else 0))

    def rate_table_entries(self) -> int:
        n = ctypes.c_int32()
        _check(load().kmc_otf_rate_table_entries(self.h, ctypes.byref(n)))
        return n.value

    def phase_cycles(self, reset: bool = True) -> np.ndarray:
        """Per-phase cycle sums of the otf step loop (library built with KMC_PHASE_TIMING)."""
        out = np.zeros(8, np.uint64)
        _check(load().kmc_otf_phase_cycles(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                           1 if reset else 0))
        return out
