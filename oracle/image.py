"""The engine's state-image layout written from an oracle trajectory.

TEST INFRASTRUCTURE ONLY: the tests use it to check the engine's image reader and
validator (``kmc_check_image``, ``kmc_pool_restore_state``) against a writer that shares
no code with the engine's own.  The product never imports it.

Layout (the engine's ``ImageHeader`` / ``image_layout``), little-endian, natural
alignment:
  header  magic "KMCS", version 1, FNV-1a-64 hash of the program words, P, nspecies,
          spuck, backend, X, Y, Z, V, layer, status, rng_kind, accum_from, seed, traj,
          kmc_time, kmc_time_step, kmc_step, rng[4], nentries, total bytes (144 bytes)
  vectors at 144: rates, integ_rates, accum_rates (P doubles each), procstat (P int64),
          nr_of_sites (P int32)
  lattice at the next 16-byte boundary: V int8 species
  entries at the next 16-byte boundary: avail_sites(p, 1..nr_of_sites(p), 1), process
          after process (int32); the position column is their inverse and not stored.
"""
from __future__ import annotations

import ctypes

import numpy as np

MAGIC = 0x53434D4B
VERSION = 1


class Header(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_uint32), ("version", ctypes.c_uint32), ("program_hash", ctypes.c_uint64),
                ("P", ctypes.c_int32), ("nspecies", ctypes.c_int32), ("spuck", ctypes.c_int32),
                ("backend", ctypes.c_int32), ("X", ctypes.c_int32), ("Y", ctypes.c_int32), ("Z", ctypes.c_int32),
                ("V", ctypes.c_int32), ("layer", ctypes.c_int32), ("status", ctypes.c_int32),
                ("rng_kind", ctypes.c_int32), ("accum_from", ctypes.c_int32), ("seed", ctypes.c_uint32),
                ("traj", ctypes.c_uint32), ("kmc_time", ctypes.c_double), ("kmc_time_step", ctypes.c_double),
                ("kmc_step", ctypes.c_int64), ("rng", ctypes.c_uint64 * 4), ("nentries", ctypes.c_int64),
                ("bytes", ctypes.c_uint64)]


def program_hash(words) -> int:
    """FNV-1a, 64 bit, over the program's int32 words as little-endian bytes."""
    h = 1469598103934665603
    for b in np.asarray(words, dtype="<i4").tobytes():
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def _up16(x: int) -> int:
    return (x + 15) // 16 * 16


def write_image(program, oracle, size, seed: int, traj: int, layer: int = 0) -> bytes:
    """Image of ``oracle`` (an Oracle stepped only by do_kmc_steps on the Philox stream,
    so its draw counter is its kmc_step) for ``program`` on a lattice of ``size``."""
    w = np.asarray(program.words, dtype=np.int32)
    ex = oracle.export()
    P, V = oracle.P, oracle.V
    X, Y = int(size[0]), int(size[1])
    Z = int(size[2]) if len(size) > 2 else 1
    ns = ex["nsites"].astype(np.int32)
    entries = np.concatenate([ex["as1"][p, 1:1 + ns[p]] for p in range(P)]).astype(np.int32)
    h = Header()
    h.magic, h.version, h.program_hash = MAGIC, VERSION, program_hash(w)
    h.P, h.nspecies, h.spuck, h.backend = P, int(w[4]), int(w[6]), int(w[2])
    h.X, h.Y, h.Z, h.V = X, Y, Z, V
    h.layer, h.status, h.rng_kind, h.accum_from = layer, 0, 1, 0
    h.seed, h.traj = seed, traj
    h.kmc_time, h.kmc_time_step, h.kmc_step = oracle.kmc_time, oracle.kmc_time_step, oracle.kmc_step
    h.rng[0] = oracle.kmc_step
    h.nentries = len(entries)
    vec = ctypes.sizeof(Header)
    lat = _up16(vec + 36 * P)
    ent = _up16(lat + V)
    total = ent + 4 * len(entries)
    h.bytes = total
    buf = bytearray(total)
    buf[:vec] = bytes(h)
    vectors = (np.asarray(oracle.rates(), "<f8").tobytes() + np.asarray(ex["integ"], "<f8").tobytes() +
               np.asarray(oracle.accum_rates(), "<f8").tobytes() + np.asarray(ex["procstat"], "<i8").tobytes() +
               ns.astype("<i4").tobytes())
    buf[vec:vec + len(vectors)] = vectors
    buf[lat:lat + V] = ex["lattice"].astype(np.int8).tobytes()
    buf[ent:ent + 4 * len(entries)] = entries.astype("<i4").tobytes()
    return bytes(buf)
