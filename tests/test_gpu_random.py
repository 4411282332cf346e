"""Whole-set GPU runs (motex_gpu_run through the motexGPU CLI) against the
oracle CLI on seeded random inputs: alphabets, factor lengths on both sides
of the 32- and 64-symbol kernel boundaries, short sequences, quorum and
occurrence bounds, and long sequences that the DP cuts into several chunks."""
import random

import pytest

from motex_gb300 import workloads as W
from helpers import run_cli


def fasta(seqs):
    return "".join(f">s{i}\n{s}\n" for i, s in enumerate(seqs))


def random_case(rng):
    kind = rng.choice(["DNA", "DNA", "PROT", "USR"])
    letters = {"DNA": "ACGT" + ("N" if rng.random() < 0.3 else ""), "PROT": W.AMINO20, "USR": "0123456789"}[kind]
    l = rng.choice([3, 6, 8, 10, 12, 15, 20, 24, 30, 32, 33, 48, 70])
    e = rng.randint(0, min(l - 1, 5))
    nseq = rng.randint(2, 30)
    seqs = []
    for _ in range(nseq):
        n = rng.choice([rng.randint(1, l + 3), rng.randint(l, 400), rng.randint(300, 1500)])
        seqs.append("".join(rng.choice(letters) for _ in range(n)))
    motif = "".join(rng.choice(letters) for _ in range(l))
    for i in range(nseq):
        if len(seqs[i]) >= l and rng.random() < 0.5:
            w = list(motif)
            for _ in range(rng.randint(0, e)):
                w[rng.randrange(l)] = rng.choice(letters)
            a = rng.randint(0, len(seqs[i]) - l)
            seqs[i] = seqs[i][:a] + "".join(w) + seqs[i][a + l:]
    d = rng.randint(0, 1)
    q = rng.choice([0, 5, 20, 50])
    args = ["-a", kind, "-i", "in.fa", "-o", "out.motex", "-d", str(d), "-k", str(l), "-e", str(e), "-q", str(q)]
    if rng.random() < 0.3:
        args += ["-n", str(rng.randint(0, 3)), "-N", str(rng.randint(5, 200)), "-Q", str(rng.randint(q, 100))]
    return seqs, args


DENSE_HIT_SHAPES = [("DNA", 4, 3), ("DNA", 4, 2), ("PROT", 4, 3), ("USR", 4, 3), ("DNA", 5, 4), ("PROT", 5, 3)]


def dense_hit_case(kind, l, e):
    """(files, args): short factors with many errors over 9 random sequences."""
    rng = random.Random(77 + l * 10 + e)
    letters = {"DNA": "ACGT", "PROT": W.AMINO20, "USR": "0123456789"}[kind]
    seqs = ["".join(rng.choice(letters) for _ in range(rng.randint(60, 700))) for _ in range(9)]
    args = ["-a", kind, "-i", "in.fa", "-o", "out.motex", "-d", "1", "-k", str(l), "-e", str(e), "-q", "30"]
    return {"in.fa": fasta(seqs)}, args


def long_chunk_case(d):
    """(files, args): 8 x 6000 nt with tandem repeats, long enough that the DP
    cuts every sequence into several text chunks."""
    wl = W.dna_long(seed=31, scale=0.006)
    wl.d, wl.k, wl.e, wl.q = d, 12, 2, 25
    return {"in.fa": fasta(wl.seqs)}, wl.cli("in.fa", "out.motex")


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(24))
def test_random_whole_set(native_built, oracle_port, seed):
    rng = random.Random(1000 + seed)
    seqs, args = random_case(rng)
    files = {"in.fa": fasta(seqs)}
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0, g[2] + o[2]
    assert g[1] == o[1]


@pytest.mark.gpu
@pytest.mark.parametrize("kind,l,e", DENSE_HIT_SHAPES)
def test_short_factors_dense_hits(native_built, oracle_port, kind, l, e):
    """Short factors with many errors hit at nearly every text position:
    the count field of each packed edit-distance lane must hold all 32 hits
    of a text block without carrying into its neighbour."""
    files, args = dense_hit_case(kind, l, e)
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0, g[2] + o[2]
    assert g[1] == o[1]
    assert g[1].count("\n") > 20


@pytest.mark.gpu
@pytest.mark.parametrize("d", [0, 1])
def test_long_sequences_split_across_chunks(native_built, oracle_port, d):
    """Few long sequences: the DP cuts every sequence into several text
    chunks, so presence must be counted once per sequence across chunks."""
    files, args = long_chunk_case(d)
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0
    assert g[1] == o[1] and g[1].count("\n") > 20
