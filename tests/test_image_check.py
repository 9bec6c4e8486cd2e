"""State images checked on the CPU (kmc_check_image: the checks kmc_pool_restore_state
and kmc_load_state make before a trajectory reaches the device), against images written
from oracle trajectories by an independent writer (oracle/image.py).

* Images of three models pass; the same image is refused for another model program.
* Corrupted images are refused with the status the restore would give: a table entry
  off the lattice or listed twice, nr_of_sites that do not add up (KMC_ERR_TABLE), a
  truncated image, an unknown species, a bad size (KMC_ERR_ARG).
* Random byte corruption never crashes the check (run in a child process).
"""
import os
import struct
import subprocess
import sys

import numpy as np
import pytest

from conftest import fixture_model
from kmos_gb300 import engine as E, program as PG
from oracle import image as IM, oracle as O

CASES = [("pairwise_interaction", "lat_int", (16, 16)), ("ZGB_model", "local_smart", (12, 10)),
         ("CO_oxidation_Ruo2", "lat_int", (8, 9))]


def oracle_image(name, backend, size, steps=2500, seed=5, traj=2):
    prog = PG.compile_model(fixture_model(name), backend)
    o = O.Oracle(prog, size, seed=seed, rng=O.RNG_PHILOX, traj=traj)
    o.set_rates((10.0 ** np.random.default_rng(1).uniform(-1, 3, size=prog.nproc)).tolist())
    o.update_accum_rate()
    o.do_kmc_steps(steps)
    return prog, o, IM.write_image(prog, o, size, seed=seed, traj=traj)


@pytest.mark.parametrize("name,backend,size", CASES)
def test_oracle_images_pass(name, backend, size):
    prog, _o, img = oracle_image(name, backend, size)
    E.check_image(prog, img)
    other = PG.compile_model(fixture_model("AB_model"), "local_smart")
    with pytest.raises(E.KMCError) as e:
        E.check_image(other, img)
    assert e.value.code == 1


def _sections(img):
    h = IM.Header.from_buffer_copy(img[:ctypes_size()])
    vec = ctypes_size()
    lat = (vec + 36 * h.P + 15) // 16 * 16
    ent = (lat + h.V + 15) // 16 * 16
    return h, vec, lat, ent


def ctypes_size():
    import ctypes
    return ctypes.sizeof(IM.Header)


def test_corrupted_images_are_refused():
    prog, o, img = oracle_image(*CASES[0])
    h, vec, lat, ent = _sections(img)
    P, V = h.P, h.V

    def refused(mutate, code):
        b = bytearray(img)
        mutate(b)
        with pytest.raises(E.KMCError) as e:
            E.check_image(prog, bytes(b))
        assert e.value.code == code

    assert h.nentries >= 2
    refused(lambda b: b.__setitem__(slice(ent, ent + 4), struct.pack("<i", V + 1)), 4)  # off the lattice
    refused(lambda b: b.__setitem__(slice(ent, ent + 4), struct.pack("<i", 0)), 4)
    ns = np.frombuffer(img, "<i4", P, vec + 32 * P)
    p = int(np.argmax(ns >= 2))
    first = ent + 4 * int(ns[:p].sum())
    refused(lambda b: b.__setitem__(slice(first + 4, first + 8), bytes(b[first:first + 4])), 4)  # listed twice
    refused(lambda b: b.__setitem__(slice(vec + 32 * P, vec + 32 * P + 4), struct.pack("<i", int(ns[0]) + 1)), 4)
    refused(lambda b: b.__setitem__(lat, 0x7F), 1)  # unknown species
    refused(lambda b: b.__setitem__(slice(32, 36), struct.pack("<i", h.X + 1)), 1)  # size and volume disagree
    with pytest.raises(E.KMCError) as e:
        E.check_image(prog, img[:-4])
    assert e.value.code == 1


def fuzz(seed: int, trials: int):
    prog, _o, img = oracle_image(*CASES[int(seed) % len(CASES)], steps=800)
    rng = np.random.default_rng(seed)
    accepted = refused = 0
    for _ in range(trials):
        b = bytearray(img)
        for _ in range(int(rng.integers(1, 5))):
            i = int(rng.integers(0, len(b)))
            b[i] = int(rng.integers(0, 256))
        if rng.random() < 0.1:
            b = b[:int(rng.integers(0, len(b)))]
        try:
            E.check_image(prog, bytes(b))
            accepted += 1
        except E.KMCError as e:
            if e.code not in (1, 4):
                raise SystemExit("refused with status %d" % e.code)
            refused += 1
    return accepted, refused


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_corrupted_images_never_crash_the_check(seed):
    r = subprocess.run([sys.executable, __file__, str(seed), "1500"], capture_output=True, text=True, timeout=600,
                       cwd=os.path.dirname(os.path.abspath(__file__)))
    assert r.returncode == 0, "check crashed or failed (status %d): %s" % (r.returncode, r.stderr[-2000:])
    accepted, refused = map(int, r.stdout.split()[-2:])
    assert refused > 0 and accepted + refused == 1500


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    a, r = fuzz(int(sys.argv[1]), int(sys.argv[2]))
    print(a, r)
