"""Structured motifs on seeded random inputs: motexGPU against the oracle CLI
for one- and two-gap boxes files, both distances, shapes that take the
packed one-gap kernel, the unpacked one and the box-check kernel.
(-q 0 -n 0 is avoided: the reference reads past sequence ends there.)"""
import random

import pytest

from helpers import run_cli


def fasta(seqs):
    return "".join(f">s{i}\n{s}\n" for i, s in enumerate(seqs))


def boxes_text(boxes):
    return f"{len(boxes)}\n" + "".join(f"{a}\n{b}\n{c}\n{d}\n" for a, b, c, d in boxes)


def random_struct_case(rng):
    letters = rng.choice(["ACGT", "ACGTN", "ARNDCQEGHILKMFPSTWYV"])
    kind = "PROT" if len(letters) > 5 else "DNA"
    ngaps = rng.choice([1, 1, 2])
    l = rng.randint(4, 9)
    e = rng.randint(0, min(2, l - 1))
    boxes = []
    for _ in range(ngaps):
        gmin = rng.randint(0, 6)
        gmax = gmin + rng.randint(0, 4 if ngaps == 2 else 12)
        blen = rng.randint(3, 12)
        boxes.append((gmin, gmax, blen, rng.randint(0, min(2, blen - 1))))
    nseq = rng.randint(4, 12)
    seqs = ["".join(rng.choice(letters) for _ in range(rng.randint(20, 160))) for _ in range(nseq)]
    # plant a structured occurrence (boxes with random gaps) in half of the sequences
    parts = ["".join(rng.choice(letters) for _ in range(l))]
    for gmin, gmax, blen, _ in boxes:
        parts.append("".join(rng.choice(letters) for _ in range(blen)))
    for i in range(nseq):
        if rng.random() < 0.5:
            occ = parts[0]
            for (gmin, gmax, _, _), box in zip(boxes, parts[1:]):
                occ += "".join(rng.choice(letters) for _ in range(rng.randint(gmin, gmax))) + box
            if len(occ) <= len(seqs[i]):
                a = rng.randint(0, len(seqs[i]) - len(occ))
                seqs[i] = seqs[i][:a] + occ + seqs[i][a + len(occ):]
    d = rng.randint(0, 1)
    q = rng.choice([5, 20, 40])
    args = ["-a", kind, "-i", "in.fa", "-o", "out.motex", "-d", str(d), "-k", str(l), "-e", str(e),
            "-q", str(q), "-s", "in.boxes"]
    return seqs, boxes, args


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(16))
def test_random_structured(native_built, oracle_port, seed):
    rng = random.Random(5000 + seed)
    seqs, boxes, args = random_struct_case(rng)
    files = {"in.fa": fasta(seqs), "in.boxes": boxes_text(boxes)}
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0, g[2] + o[2]
    assert g[1] == o[1]
