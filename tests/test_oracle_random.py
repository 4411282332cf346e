"""The CPU port (oracle/_build/motex_port) against the reference itself
(oracle/_ref/motexOMP, built from the reference sources and the shipped
libflasm.so) on the seeded random inputs of the GPU parity tests: whole sets
(alphabets, factor lengths on both sides of the 32- and 64-symbol kernel
boundaries, short sequences, quorum and occurrence bounds) and structured
motifs with one and two gaps, short factors that hit almost everywhere, and
long sequences cut into text chunks.  The GPU tests compare motexGPU with the port
on exactly these inputs; this pins the port to the reference there.  The
reference build is x86-64 only (the shipped libflasm.so), so the test is
skipped where it is absent."""
import os
import random

import pytest

from conftest import ORACLE_DIR
from helpers import run_cli
from test_gpu_random import DENSE_HIT_SHAPES, dense_hit_case, fasta, long_chunk_case, random_case
from test_gpu_random_struct import boxes_text, random_struct_case

REF_OMP = os.path.join(ORACLE_DIR, "_ref", "motexOMP")
THREADS = str(os.cpu_count() or 1)

pytestmark = pytest.mark.skipif(not os.access(REF_OMP, os.X_OK), reason="reference build absent (x86-64 only)")


@pytest.mark.parametrize("seed", range(24))
def test_port_matches_reference_random_whole_set(oracle_port, seed):
    rng = random.Random(1000 + seed)                      # the seeds of test_random_whole_set
    seqs, args = random_case(rng)
    files = {"in.fa": fasta(seqs)}
    r = run_cli(REF_OMP, None, args + ["-t", THREADS], files=files)
    o = run_cli(oracle_port, None, args + ["-t", THREADS], files=files)
    assert r[0] == o[0] == 0, r[2] + o[2]
    assert r[1] == o[1]


@pytest.mark.parametrize("seed", range(16))
def test_port_matches_reference_random_structured(oracle_port, seed):
    rng = random.Random(5000 + seed)                      # the seeds of test_random_structured
    seqs, boxes, args = random_struct_case(rng)
    files = {"in.fa": fasta(seqs), "in.boxes": boxes_text(boxes)}
    r = run_cli(REF_OMP, None, args + ["-t", THREADS], files=files)
    o = run_cli(oracle_port, None, args + ["-t", THREADS], files=files)
    assert r[0] == o[0] == 0, r[2] + o[2]
    assert r[1] == o[1]


def _same(port, files, args):
    r = run_cli(REF_OMP, None, args + ["-t", THREADS], files=files)
    o = run_cli(port, None, args + ["-t", THREADS], files=files)
    assert r[0] == o[0] == 0, r[2] + o[2]
    assert r[1] == o[1]


@pytest.mark.parametrize("kind,l,e", DENSE_HIT_SHAPES)
def test_port_matches_reference_dense_hits(oracle_port, kind, l, e):
    _same(oracle_port, *dense_hit_case(kind, l, e))


@pytest.mark.parametrize("d", [0, 1])
def test_port_matches_reference_long_chunks(oracle_port, d):
    _same(oracle_port, *long_chunk_case(d))
