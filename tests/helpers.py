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


def load_mode_case(name):
    """(case dir, args, {output file: expected text}) of a -b / -I case."""
    d = os.path.join(GOLDEN, name)
    with open(os.path.join(d, "case.json")) as f:
        meta = json.load(f)
    expected = {}
    for o in meta["outputs"]:
        with open(os.path.join(d, "expected." + (o[4:] if o.startswith("out.") else o))) as f:
            expected[o] = f.read()
    return d, meta["args"], expected


def run_outputs(binary, case_dir, args, outputs, extra=(), timeout=600):
    """Run a motex CLI on a scratch copy of case_dir; returns (rc, {output: text or None}, stderr)."""
    with tempfile.TemporaryDirectory() as tmp:
        for f in os.listdir(case_dir):
            shutil.copy(os.path.join(case_dir, f), tmp)
        p = subprocess.run([binary] + list(args) + list(extra), cwd=tmp, capture_output=True, text=True,
                           timeout=timeout)
        got = {}
        for o in outputs:
            path = os.path.join(tmp, o)
            got[o] = None
            if os.path.exists(path):
                with open(path) as f:
                    got[o] = strip_volatile(f.read())
        return p.returncode, got, p.stderr


def same_but_pvalues(a, b, rel=1e-5, abs_tol=1e-15):
    """Line-by-line equality, except that the p-value (the 8th field of an
    8-field motif line) may differ by a rounding: the reference computes it
    in long double, which is 80-bit x87 on x86-64 and binary128 on aarch64.
    Returns the first differing pair of lines, or None."""
    la, lb = a.splitlines(), b.splitlines()
    if len(la) != len(lb):
        return ("line count", len(la), len(lb))
    for x, y in zip(la, lb):
        if x == y:
            continue
        fx, fy = x.split(" "), y.split(" ")
        if len(fx) != 8 or len(fy) != 8 or fx[:7] != fy[:7]:
            return (x, y)
        try:
            px, py = float(fx[7]), float(fy[7])
        except ValueError:
            return (x, y)
        if not abs(px - py) <= rel * max(abs(px), abs(py)) + abs_tol:
            return (x, y)
    return None
