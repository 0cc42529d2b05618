"""The reference-side binding is a drop-in for the reference's CUDA factory.

Where the reference tree is present, oracle/Makefile links the reference's own
objects with banjo_gb300/adapter/Gb300LatticeBackend.cpp in place of
src/fastlattice/CudaLatticeUnavailable.cpp and runs tests/adapter_driver.cpp,
an ordinary reference program. Without a device the factory must throw
std::runtime_error, the stub's contract; with one, the GB300 backend must agree
with CpuLatticeBackend<float> bit for bit.
"""
import os
import subprocess

import pytest

import oracle


def _reference_present():
    return oracle.reference_present()


@pytest.mark.skipif(not _reference_present(), reason="the reference tree is not present here")
def test_binding_replaces_the_cuda_stub(gbl):
    oracle.build_reference()
    subprocess.run(["make", "-s", "-C", oracle.HERE, "adapter"], check=True)
    r = subprocess.run([os.path.join(oracle.HERE, "_ref", "adapter_driver")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASS" in r.stdout
    if not gbl.available():
        assert "cudaLatticeAvailable=0" in r.stdout and "runtime_error" in r.stdout


@pytest.mark.skipif(not _reference_present(), reason="the reference tree is not present here")
def test_binding_carries_every_field():
    """The binding over a recording stand-in for the library (no device): every
    field of LatticeSchedule, LatticeState, StepSettings, SphereState,
    RunControl and the wrenches arrives in its C field, and every field of the
    RunStatus, sources, downloaded state, first-failure list and frames the
    library hands back arrives in its reference field."""
    oracle.build_reference()
    subprocess.run(["make", "-s", "-C", oracle.HERE, "adapter-stub"], check=True)
    r = subprocess.run([os.path.join(oracle.HERE, "_ref", "adapter_stub_driver")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "[PASS]" in r.stdout
