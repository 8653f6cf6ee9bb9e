import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libns3d_oracle.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: long-running CPU case")


def build_oracle():
    src = os.path.join(ROOT, "oracle", "ns3d_oracle.cpp")
    if not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return ORACLE_LIB


@pytest.fixture(scope="session")
def oracle():
    from ns3d_gb300 import capi
    return capi.load(build_oracle())


@pytest.fixture(scope="session")
def gpulib():
    import ns3d_gb300
    if not os.path.exists(ns3d_gb300.LIB_PATH):
        ns3d_gb300.build()
    return ns3d_gb300.lib()
