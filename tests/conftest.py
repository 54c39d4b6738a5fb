import importlib
import os
import platform
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libvsr.so")


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("anari-visionaray_gb300")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def device(pkg):
    dev = pkg.vsr.Device()
    yield dev
    dev.close()


@pytest.fixture(scope="session")
def contracted(oracle, tmp_path_factory):
    """Path of a second liboracle.so built with multiply-add contraction
    (-ffp-contract=fast): it rounds like a compiler that fuses multiplies
    and adds, so comparing it with the plain oracle measures how sensitive a
    scene is to last-bit differences."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("fma") / "liboracle.so")
    flags = ["-std=c++17", "-O3", "-fPIC", "-pthread", "-shared", "-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # x86 needs FMA enabled; aarch64 has it
    src = os.path.join(ROOT, "oracle", "oracle.cpp")
    subprocess.run([cxx, *flags, "-o", out, src], check=True)
    return out
