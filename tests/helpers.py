"""Shared helpers of the test-suite: running the CLIs on a case directory."""
import json
import os
import shutil
import subprocess
import tempfile

from conftest import GOLDEN, strip_volatile


def load_case(name):
    d = os.path.join(GOLDEN, name)
    with open(os.path.join(d, "case.json")) as f:
        meta = json.load(f)
    with open(os.path.join(d, "expected.motex")) as f:
        expected = f.read()
    return d, meta["args"], expected


def expected_smile(name):
    """The case's stored SMILE-like output, or None when it has none."""
    path = os.path.join(GOLDEN, name, "expected.smile")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return f.read()


def read_smile(case_dir, binary, args, extra=(), timeout=600):
    """Run a motex CLI that writes out.smile; returns (rc, main output, SMILE output, stderr)."""
    with tempfile.TemporaryDirectory() as tmp:
        for f in os.listdir(case_dir):
            shutil.copy(os.path.join(case_dir, f), tmp)
        p = subprocess.run([binary] + list(args) + list(extra), cwd=tmp, capture_output=True, text=True,
                           timeout=timeout)
        outs = []
        for name in ("out.motex", "out.smile"):
            path = os.path.join(tmp, name)
            outs.append(None)
            if os.path.exists(path):
                with open(path) as f:
                    outs[-1] = strip_volatile(f.read())
        return p.returncode, outs[0], outs[1], p.stderr


def run_cli(binary, case_dir, args, extra=(), files=None, timeout=600):
    """Run a motex CLI from a scratch copy of case_dir; returns (rc, output, stderr)."""
    with tempfile.TemporaryDirectory() as tmp:
        if case_dir:
            for f in os.listdir(case_dir):
                shutil.copy(os.path.join(case_dir, f), tmp)
        for name, text in (files or {}).items():
            with open(os.path.join(tmp, name), "w") as f:
                f.write(text)
        p = subprocess.run([binary] + list(args) + list(extra), cwd=tmp, capture_output=True, text=True,
                           timeout=timeout)
        out = None
        op = os.path.join(tmp, "out.motex")
        if os.path.exists(op):
            with open(op) as f:
                out = strip_volatile(f.read())
        return p.returncode, out, p.stderr
