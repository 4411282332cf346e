"""The full-size configurations against the reference itself: motexGPU's
output file, without the two volatile header lines, has the SHA-256 and line
count of the reference's (motexOMP built from the reference sources) on the
same seeded input and switches.  The hashes were made on x86-64 by
tests/golden/make_fullsize_hashes.py and are stored in
tests/golden/fullsize.json; the inputs are regenerated here by the same
seeded generators."""
import hashlib
import importlib.util
import json
import os
import subprocess
import tempfile

import pytest

from conftest import strip_volatile
from motex_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "golden", "fullsize.json")
TABLE = json.load(open(TABLE_PATH)) if os.path.exists(TABLE_PATH) else {}

_spec = importlib.util.spec_from_file_location("make_fullsize_hashes",
                                               os.path.join(HERE, "golden", "make_fullsize_hashes.py"))
_gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(_gen)


def test_table_covers_the_configurations():
    """Every full-size configuration has a pinned hash (CPU check of the fixture)."""
    assert set(TABLE) <= set(_gen.CASES)
    for name, e in TABLE.items():
        # at least the header and the footer (a configuration may print no motif)
        assert len(e["sha256"]) == 64 and e["lines"] >= 14, name


@pytest.mark.parametrize("name", sorted(TABLE))
def test_inputs_match_pinned_generators(name):
    """The seeded generators still produce the inputs the reference ran on
    (CPU check: a changed generator would otherwise show up only as a GPU
    hash mismatch)."""
    entry = TABLE[name]
    if "input_sha256" not in entry:
        pytest.skip("entry made before inputs were hashed")
    assert _gen.input_sha256(_gen.CASES[name][0]()) == entry["input_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(TABLE))
def test_fullsize_matches_reference_hash(native_built, name):
    entry = TABLE[name]
    w = _gen.CASES[name][0]()
    with tempfile.TemporaryDirectory() as tmp:
        W.write_fasta(os.path.join(tmp, "in.fa"), w.seqs, width=60)
        if w.boxes:
            W.write_boxes(os.path.join(tmp, "in.boxes"), w.boxes)
        p = subprocess.run([native_built.CLI_PATH] + entry["args"], cwd=tmp, capture_output=True, text=True,
                           timeout=900)
        assert p.returncode == 0, p.stderr
        with open(os.path.join(tmp, "out.motex")) as f:
            out = strip_volatile(f.read())
    assert out.count("\n") == entry["lines"]
    assert hashlib.sha256(out.encode()).hexdigest() == entry["sha256"]
