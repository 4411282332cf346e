"""The popc-free form of the one-gap structured Hamming kernel
(k_dp_struct1_hd with GE = e: box 0 and the two box-1 rows as guarded lanes,
each lane's lowest set bit cleared e times), taken when both boxes allow the
same e <= 3 and l0 + 2 b1 + 3 <= 32: motexGPU against the oracle CLI on seeded
inputs with planted structured occurrences, and against the popc form
(MOTEX_STRUCT_NO_CLEAR=1) on 1/10 of config 2's input with quorum 1 %."""
import os
import random
import tempfile

import pytest

from helpers import run_cli
from motex_gb300 import workloads as W


def fasta(seqs):
    return "".join(f">s{i}\n{s}\n" for i, s in enumerate(seqs))


def case(rng):
    letters = rng.choice(["ACGT", "ACGT", "ARNDCQEGHILKMFPSTWYV"])
    kind = "PROT" if len(letters) > 4 else "DNA"
    while True:
        l0, b1 = rng.randint(3, 10), rng.randint(3, 11)
        if l0 + 2 * b1 + 3 <= 32:
            break
    e = rng.randint(0, min(3, min(l0, b1) - 1))
    gmin = rng.randint(0, 8)
    boxes = [(gmin, gmin + rng.randint(0, 6), b1, e)]
    seqs = ["".join(rng.choice(letters) for _ in range(rng.randint(60, 400))) for _ in range(rng.randint(5, 12))]
    p0 = "".join(rng.choice(letters) for _ in range(l0))
    p1 = "".join(rng.choice(letters) for _ in range(b1))
    for i in range(len(seqs)):
        for _ in range(rng.randint(0, 3)):
            occ = list(p0 + "".join(rng.choice(letters) for _ in range(rng.randint(boxes[0][0], boxes[0][1]))) + p1)
            for q in rng.sample(range(len(occ)), rng.randint(0, e)):
                occ[q] = rng.choice(letters)
            if len(occ) <= len(seqs[i]):
                a = rng.randint(0, len(seqs[i]) - len(occ))
                seqs[i] = seqs[i][:a] + "".join(occ) + seqs[i][a + len(occ):]
    args = ["-a", kind, "-i", "in.fa", "-o", "out.motex", "-d", "0", "-k", str(l0), "-e", str(e),
            "-q", str(rng.choice([10, 25])), "-s", "in.boxes"]
    return seqs, boxes, args


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(16))
def test_guarded_struct_hd_vs_oracle(native_built, oracle_port, seed):
    rng = random.Random(9900 + seed)
    seqs, boxes, args = case(rng)
    files = {"in.fa": fasta(seqs), "in.boxes": f"{len(boxes)}\n" + "".join(f"{a}\n{b}\n{c}\n{d}\n" for a, b, c, d in boxes)}
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0, g[2] + o[2]
    assert g[1] == o[1]


@pytest.mark.gpu
def test_guarded_struct_hd_equals_popc_form(native_built, monkeypatch):
    w = W.structured(d=0, scale=0.1)
    w.q = 1
    with tempfile.TemporaryDirectory() as tmp:
        W.write_fasta(os.path.join(tmp, "in.fa"), w.seqs)
        W.write_boxes(os.path.join(tmp, "in.boxes"), w.boxes)
        files = {"in.fa": open(os.path.join(tmp, "in.fa")).read(),
                 "in.boxes": open(os.path.join(tmp, "in.boxes")).read()}
    args = w.cli("in.fa", "out.motex", "in.boxes")
    clr = run_cli(native_built.CLI_PATH, None, args, files=files)
    monkeypatch.setenv("MOTEX_STRUCT_NO_CLEAR", "1")
    pop = run_cli(native_built.CLI_PATH, None, args, files=files)
    assert clr[0] == pop[0] == 0, clr[2] + pop[2]
    assert clr[1] == pop[1]
    assert clr[1].count("\n") > 20
