"""The KMC_DEBUG build of the engine (kmos_gb300.build.build(debug=True)): its kernels
check every table and lattice index they compute from table contents and stop the step
with ST_TABLE on one out of range -- the device-side counterpart of the host's program
and state checks, where a sanitizer cannot run.  The GPU parity tests, which drive every
path of the step kernel (all fixture models and edit forms, 96 and 174 processes, full
write logs, pools of mixed models), run against it and must pass: no index of those runs
leaves its range."""
import os
import subprocess
import sys

import pytest

from kmos_gb300 import build

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_parity_suite_under_the_debug_build():
    lib = build.build(debug=True)
    env = {**os.environ, "KMC_GB300_LIB": lib}
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
                        os.path.join(HERE, "test_gpu_parity.py"), "-k", "not cancel"],
                       env=env, capture_output=True, text=True, timeout=1800, cwd=os.path.dirname(HERE))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
