"""The product path has no CPU fallback: without its CUDA library, or without a CUDA
device, every entry point a user reaches (the engine's classes and the drop-in f2py
module's proclist.init) raises instead of computing on the host.  Runs on a machine
without a GPU; skipped where a device is present."""
import os
import re
import subprocess
import sys

import pytest

from conftest import ROOT, fixture_model
from kmos_gb300 import engine as E
from kmos_gb300 import kmc_model as K
from kmos_gb300 import program as PG

KMC_ERR_NODEVICE = int(re.search(r"#define KMC_ERR_NODEVICE (\d+)",
                                 open(os.path.join(ROOT, "include", "kmc_gb300.h")).read()).group(1))
NO_DEVICE = not os.path.exists("/dev/nvidiactl")
needs_no_device = pytest.mark.skipif(not NO_DEVICE, reason="a CUDA device is present")


def test_missing_library_raises():
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from kmos_gb300 import engine\n"
            "try:\n"
            "    engine.load()\n"
            "except RuntimeError as e:\n"
            "    print('raised:', e)\n"
            "else:\n"
            "    print('loaded')\n") % ROOT
    env = dict(os.environ, KMC_GB300_LIB=os.path.join(ROOT, "_no_such_dir", "libkmcgb300.so"))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("raised:") and "missing" in out.stdout


@needs_no_device
@pytest.mark.parametrize("backend", ["local_smart", "lat_int"])
def test_trajectory_and_pool_need_a_device(backend):
    prog = PG.compile_model(fixture_model("CO_oxidation_Ruo2"), backend)
    with pytest.raises(E.KMCError) as err:
        E.Trajectory(prog, (4, 4))
    assert err.value.code == KMC_ERR_NODEVICE
    with pytest.raises(E.KMCError) as err:
        E.Pool(1 << 20, 4)
    assert err.value.code == KMC_ERR_NODEVICE


@needs_no_device
def test_otf_batch_needs_a_device():
    prog = PG.compile_model(fixture_model("intZGB_otf"), "otf")
    with pytest.raises(E.KMCError) as err:
        E.OtfBatch(prog, (8, 8), ntraj=2)
    assert err.value.code == KMC_ERR_NODEVICE


@needs_no_device
@pytest.mark.parametrize("name, backend", [("CO_oxidation_Ruo2", "local_smart"), ("intZGB_otf", "otf")])
def test_dropin_init_needs_a_device(name, backend):
    K.configure(fixture_model(name), backend)
    with pytest.raises(E.KMCError) as err:
        K.proclist.init((4, 4), "kmc_model", 0, 42, True)
    assert err.value.code == KMC_ERR_NODEVICE
