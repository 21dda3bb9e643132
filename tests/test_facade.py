"""CPU tests of the C++ façade (relion_gb300/acc): the reference's accelerated
E-step classes -- AccProjector, AccBackprojector (src/acc/acc_projector.h:17,
src/acc/acc_backprojector.h:24), MlDeviceBundle and MlOptimiserCuda
(src/acc/cuda/cuda_ml_optimiser.h:18,77) -- compile into
libgbrelion_acc.so over the C ABI, export the reference's member functions,
and a program built against them links and loads the library.  The E-step
through them is checked against the ctypes path on the GPU
(test_gpu_facade.py)."""
import os
import subprocess

import pytest


def _symbols(path):
    p = subprocess.run(["nm", "-DC", "--defined-only", path], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    if p.returncode != 0:
        pytest.skip("nm unavailable: %s" % p.stderr.strip())
    return p.stdout


def test_facade_exports_reference_members(facade_driver):
    from relion_gb300 import build as gbuild
    syms = _symbols(gbuild.ACC_LIB)
    for name in ("AccProjector::setMdlDim(", "AccProjector::initMdl(", "AccBackprojector::setMdlDim(",
                 "AccBackprojector::initMdl()", "AccBackprojector::getMdlData(",
                 "MlDeviceBundle::setupFixedSizedObjects()", "MlDeviceBundle::setupTunableSizedObjects(",
                 "MlOptimiserCuda::MlOptimiserCuda(MlOptimiser*, MlDeviceBundle*, char const*)",
                 "MlOptimiserCuda::doThreadExpectationSomeParticles(int)"):
        assert name in syms, name


def test_facade_program_links_and_loads(facade_driver):
    p = subprocess.run([facade_driver, "--version"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=60)
    assert p.returncode == 0, p.stderr
    assert "sm_103a" in p.stdout


def test_facade_reports_library_errors(facade_driver, tmp_path):
    # a request for a class count the header cannot satisfy: the façade
    # raises with the library's (or its own) message, exit status 1
    req = tmp_path / "bad.bin"
    req.write_bytes(b"\0" * 16)
    p = subprocess.run([facade_driver, str(req), str(tmp_path / "out.bin")], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=60)
    assert p.returncode == 1 and "facade_estep:" in p.stderr
