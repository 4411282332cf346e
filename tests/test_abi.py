"""The C ABI library loads and exports every entry point include/motex_gpu.h declares."""
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions():
    with open(os.path.join(ROOT, "include", "motex_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^[a-z_ 0-9]+\**\s*\*?\s*(motex_[a-z_]+)\s*\(", text, re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("motex_gpu_run", "motex_gpu_extract_pair", "motex_ctx_create", "motex_gpu_execute"):
        assert n in names


def test_library_exports_every_declared_symbol(native_built):
    lib = native_built.load_library()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert sorted(native_built.EXPORTS) == declared_functions()
    out = subprocess.run(["nm", "-D", native_built.LIB_PATH], capture_output=True, text=True).stdout
    for name in declared_functions():
        assert re.search(r" T " + name + r"$", out, re.M), name


def test_error_strings(native_built):
    lib = native_built.load_library()
    for code in range(0, -8, -1):
        assert lib.motex_gpu_strerror(code)
    assert lib.motex_gpu_strerror(-99) == b"unknown error"


def test_no_silent_fallback_without_gpu(native_built):
    """Without a GPU the product path fails loudly (no CPU fallback)."""
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    with pytest.raises(native_built.MotexError) as ei:
        native_built.Context(0)
    assert ei.value.code == -3
