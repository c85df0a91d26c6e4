"""Shared test setup.

* registers the ``gpu`` marker (tests that need a CUDA device);
* puts the repository root and oracle/ on sys.path;
* builds the oracle (plain C, gcc) and the CUDA library (nvcc, sm_103a) when
  they are missing, so a fresh checkout runs ``pytest`` directly.
"""

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
for p in (ROOT, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _ensure_oracle():
    lib = os.path.join(ORACLE, "_build", "libek_oracle.so")
    if not os.path.exists(lib):
        env = dict(os.environ, EK_SKIP_REF="1")
        subprocess.run(["sh", os.path.join(ORACLE, "build.sh")], check=True, env=env)


def _ensure_library():
    from euler_kokkos_gb300 import build as B

    if not B.up_to_date():
        B.build()


@pytest.fixture(scope="session", autouse=True)
def built_artifacts():
    _ensure_oracle()
    _ensure_library()
    yield


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
