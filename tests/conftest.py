import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

ORACLE_DIR = os.path.join(ROOT, "oracle")
PORT_BIN = os.path.join(ORACLE_DIR, "_build", "motex_port")
PORT_LIB = os.path.join(ORACLE_DIR, "_build", "libmotex_port.so")
GOLDEN = os.path.join(ROOT, "tests", "golden", "cases")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_port():
    """The CPU restatement (oracle/_build/motex_port); built on demand."""
    if not (os.path.exists(PORT_BIN) and os.path.exists(PORT_LIB)):
        subprocess.run(["make", "-C", ORACLE_DIR, "-j4"], check=True, capture_output=True)
    return PORT_BIN


@pytest.fixture(scope="session")
def native_built():
    """libmotex_gpu.so + motexGPU, built in-tree on demand."""
    from motex_gb300 import build
    build.build()
    from motex_gb300 import native
    return native


@pytest.fixture(scope="session")
def gpu_ctx(native_built):
    ctx = native_built.Context(0)
    yield ctx
    ctx.close()


def _case_dirs():
    if not os.path.isdir(GOLDEN):
        return []
    return sorted(d for d in os.listdir(GOLDEN) if os.path.isdir(os.path.join(GOLDEN, d)))


def _has_outputs(name):
    with open(os.path.join(GOLDEN, name, "case.json")) as f:
        return "outputs" in json.load(f)


def golden_cases():
    """Cases with one main output (plus an optional SMILE-like file)."""
    return [d for d in _case_dirs() if not _has_outputs(d)]


def mode_cases():
    """Background (-b) and word-search (-I) cases: several output files."""
    return [d for d in _case_dirs() if _has_outputs(d)]


def strip_volatile(text: str) -> str:
    return "".join(l for l in text.splitlines(True)
                   if not l.startswith(("# Rundate:", "# Run on ", "User time:")))
