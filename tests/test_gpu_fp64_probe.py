"""Measures the GPU's FP64 throughput and latency (tests/gpu_probes/fp64_probe.cu) and
its memory latencies (tests/gpu_probes/latency_probe.cu) and prints them; the engine's
design follows from these numbers.  The assertions only check that the probes ran."""
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


def test_latency_probe(tmp_path):
    exe = str(tmp_path / "latency_probe")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                           os.path.join(ROOT, "tests", "gpu_probes", "latency_probe.cu")])
    out = subprocess.check_output([exe], text=True, timeout=120)
    print(out)
    assert "HBM" in out and "err=no error" in out
