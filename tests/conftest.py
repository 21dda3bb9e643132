import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as obuild
    obuild.build()
    from oracle import pyoracle
    return pyoracle


@pytest.fixture(scope="session")
def facade_driver(tmp_path_factory):
    """tests/cpp/facade_estep.cpp compiled against the C++ façade library
    (relion_gb300/_build/libgbrelion_acc.so, built with libgbrelion)."""
    import subprocess
    from relion_gb300 import build as gbuild
    gbuild.build()
    exe = str(tmp_path_factory.mktemp("facade") / "facade_estep")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "relion_gb300", "acc"), os.path.join(ROOT, "tests", "cpp", "facade_estep.cpp"),
           "-o", exe, "-L", gbuild.BUILD, "-lgbrelion_acc", "-lgbrelion", "-Wl,-rpath," + gbuild.BUILD]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert p.returncode == 0, p.stdout
    return exe
