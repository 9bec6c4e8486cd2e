"""Measures the GPU's FP64 throughput and latency (tests/gpu_probes/fp64_probe.cu) and
prints them; the engine's design assumes FP64 is scarce and slow.  The assertion only
checks that the probe ran."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_fp64_probe(tmp_path):
    exe = str(tmp_path / "fp64_probe")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                           os.path.join(ROOT, "tests", "gpu_probes", "fp64_probe.cu")])
    out = subprocess.check_output([exe], text=True, timeout=120)
    print(out)
    assert "latency DADD" in out and "err=no error" in out
