"""The host-side program check (kmc_check_program, run by kmc_create and
kmc_pool_add_model before a program reaches the device) against malformed programs:
random words of compiled programs are overwritten with random values, values near the
int32 limits, small shifts, flipped bits and small negatives.  Every such program must be
refused with KMC_ERR_PROGRAM or accepted -- never crash the host (offsets are checked
in 64-bit arithmetic, so none can wrap past a bound).  The fuzzing runs in a child
process, so that a crash shows as a failed test rather than a lost test run.
"""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def fuzz(seed: int, trials: int) -> tuple:
    import numpy as np

    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.dirname(HERE))
    from conftest import fixture_model, trimer_model
    from kmos_gb300 import configs, engine as E, program as PG

    progs = [PG.compile_model(fixture_model(n), b) for n in ("pairwise_interaction", "ZGB_model", "CO_oxidation_Ruo2")
             for b in ("lat_int", "local_smart")]
    progs += [PG.compile_model(trimer_model(), "local_smart"), configs.build(3, n=1, steps=0).program]
    rng = np.random.default_rng(seed)
    accepted = refused = 0
    for trial in range(trials):
        w = np.array(progs[trial % len(progs)].words, dtype=np.int32)
        for _ in range(int(rng.integers(1, 4))):
            i = int(rng.integers(0, len(w)))
            how = int(rng.integers(0, 5))
            if how == 0:
                w[i] = int(rng.integers(-2**31, 2**31, dtype=np.int64))
            elif how == 1:
                w[i] = (int(w[i]) + int(rng.integers(-4, 5)) + 2**31) % 2**32 - 2**31
            elif how == 2:
                w[i] = 2**31 - 1 - int(rng.integers(0, 8))
            elif how == 3:
                w[i] = np.uint32((int(w[i]) & 0xFFFFFFFF) ^ (1 << int(rng.integers(0, 32)))).view(np.int32)
            else:
                w[i] = -int(rng.integers(1, 8))
        try:
            E.check_program(w)
            accepted += 1
        except E.KMCError as e:
            if e.code != 5:
                raise SystemExit("refused with status %d, not KMC_ERR_PROGRAM" % e.code)
            refused += 1
    return accepted, refused


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_malformed_programs_never_crash_the_check(seed):
    r = subprocess.run([sys.executable, __file__, str(seed), "2500"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, "check crashed or failed (status %d): %s" % (r.returncode, r.stderr[-2000:])
    accepted, refused = map(int, r.stdout.split()[-2:])
    assert refused > 0 and accepted + refused == 2500


if __name__ == "__main__":
    a, r = fuzz(int(sys.argv[1]), int(sys.argv[2]))
    print(a, r)
