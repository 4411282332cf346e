"""The block form of the any-gap structured search (k_dp_structN_blk): a warp
owns Pw = 33 - D pattern positions, every lane packs one row of each box in a
register, hit masks of the last blocks sit in a per-warp ring, and chains are
merged only where a box-0 hit occurs.

* seeded random inputs with two and three gaps, and one gap too long for the
  one-gap shared-history kernel, short sequences (chains that would cross a
  sequence end) and gap spans that need several blocks of look-ahead:
  motexGPU against the oracle CLI;
* the reference's example boxes shape on 1/10 of config 2's input: the block
  form against the per-position form of the same search
  (MOTEX_STRUCTN_NO_BLOCK=1), both distances, quorum 1% so that motifs print.
"""
import os
import random
import tempfile

import pytest

from helpers import run_cli
from motex_gb300 import workloads as W


def fasta(seqs):
    return "".join(f">s{i}\n{s}\n" for i, s in enumerate(seqs))


def boxes_text(boxes):
    return f"{len(boxes)}\n" + "".join(f"{a}\n{b}\n{c}\n{d}\n" for a, b, c, d in boxes)


def block_case(rng):
    letters = rng.choice(["ACGT", "ACGT", "ACGTN", "ARNDCQEGHILKMFPSTWYV"])
    kind = "PROT" if len(letters) > 5 else "DNA"
    shape = rng.choice(["two", "two", "three", "long_one"])
    d = rng.randint(0, 1)
    l = rng.randint(4, 8)
    e = rng.randint(0, min(1, l - 1))
    boxes = []
    if shape == "long_one":                      # gap max + box length > 31: the any-gap kernels
        gmin = rng.randint(20, 60)
        boxes.append((gmin, gmin + rng.randint(0, 12), rng.randint(4, 9), rng.randint(0, 1)))
    else:
        for _ in range(2 if shape == "two" else 3):
            gmin = rng.randint(0, 30)
            blen = rng.randint(3, 7)
            boxes.append((gmin, gmin + rng.randint(0, 3), blen, rng.randint(0, min(1, blen - 1))))
    nseq = rng.randint(4, 12)
    seqs = []
    for _ in range(nseq):
        n = rng.randint(15, 60) if rng.random() < 0.3 else rng.randint(60, 400)
        seqs.append("".join(rng.choice(letters) for _ in range(n)))
    parts = ["".join(rng.choice(letters) for _ in range(l))]
    for _, _, blen, _ in boxes:
        parts.append("".join(rng.choice(letters) for _ in range(blen)))
    for i in range(nseq):
        for _ in range(rng.randint(0, 3)):       # planted structured occurrences, some back to back
            occ = parts[0]
            for (gmin, gmax, _, _), box in zip(boxes, parts[1:]):
                occ += "".join(rng.choice(letters) for _ in range(rng.randint(gmin, gmax))) + box
            if len(occ) <= len(seqs[i]):
                a = rng.randint(0, len(seqs[i]) - len(occ))
                seqs[i] = seqs[i][:a] + occ + seqs[i][a + len(occ):]
    q = rng.choice([5, 20, 40])
    args = ["-a", kind, "-i", "in.fa", "-o", "out.motex", "-d", str(d), "-k", str(l), "-e", str(e),
            "-q", str(q), "-s", "in.boxes"]
    return seqs, boxes, args


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(24))
def test_block_random_vs_oracle(native_built, oracle_port, seed):
    rng = random.Random(9100 + seed)
    seqs, boxes, args = block_case(rng)
    files = {"in.fa": fasta(seqs), "in.boxes": boxes_text(boxes)}
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0, g[2] + o[2]
    assert g[1] == o[1]


@pytest.mark.gpu
@pytest.mark.parametrize("d", [0, 1])
def test_block_equals_per_position_form(native_built, monkeypatch, d):
    w = W.structured2(d=d, scale=0.1)
    w.q = 1
    with tempfile.TemporaryDirectory() as tmp:
        W.write_fasta(os.path.join(tmp, "in.fa"), w.seqs)
        W.write_boxes(os.path.join(tmp, "in.boxes"), w.boxes)
        files = {"in.fa": open(os.path.join(tmp, "in.fa")).read(),
                 "in.boxes": open(os.path.join(tmp, "in.boxes")).read()}
    args = w.cli("in.fa", "out.motex", "in.boxes")
    blk = run_cli(native_built.CLI_PATH, None, args, files=files)
    monkeypatch.setenv("MOTEX_STRUCTN_NO_BLOCK", "1")
    per = run_cli(native_built.CLI_PATH, None, args, files=files)
    assert blk[0] == per[0] == 0, blk[2] + per[2]
    assert blk[1] == per[1]
    assert blk[1].count("\n") > 20                 # motifs printed


def wide_case(rng):
    """Shapes only the per-position any-gap kernel takes: a box or box 0
    longer than 32 symbols (64-bit rows), more than 32 structures, or more
    than 8 gaps."""
    shape = rng.choice(["wide_box", "wide_l", "many", "gaps"])
    d = rng.randint(0, 1)
    l, e = rng.randint(5, 8), rng.randint(0, 1)
    if shape == "wide_l":
        l, e = rng.randint(33, 60), rng.randint(2, 6)
    if shape == "wide_box":
        boxes = [(rng.randint(0, 4), 0, rng.randint(33, 64), rng.randint(1, 5))]
        boxes = [(a, a + rng.randint(0, 3), c, dd) for a, _, c, dd in boxes]
        if rng.random() < 0.5:
            boxes.append((1, 3, rng.randint(4, 8), 1))
    elif shape == "wide_l":
        boxes = [(2, 5, rng.randint(6, 12), 1)]
    elif shape == "many":
        boxes = [(0, rng.randint(5, 9), rng.randint(4, 7), 1), (0, rng.randint(5, 9), rng.randint(4, 7), 1)]
    else:
        boxes = [(1, rng.choice([1, 1, 2]), rng.randint(3, 5), 0) for _ in range(rng.randint(9, 12))]
    nseq = rng.randint(4, 8)
    seqs = ["".join(rng.choice("ACGT") for _ in range(rng.randint(80, 300))) for _ in range(nseq)]
    parts = ["".join(rng.choice("ACGT") for _ in range(l))] + ["".join(rng.choice("ACGT") for _ in range(b[2]))
                                                               for b in boxes]
    for i in range(nseq):
        if rng.random() < 0.6:
            occ = parts[0]
            for (gmin, gmax, _, _), box in zip(boxes, parts[1:]):
                occ += "".join(rng.choice("ACGT") for _ in range(rng.randint(gmin, gmax))) + box
            if len(occ) <= len(seqs[i]):
                a = rng.randint(0, len(seqs[i]) - len(occ))
                seqs[i] = seqs[i][:a] + occ + seqs[i][a + len(occ):]
    args = ["-a", "DNA", "-i", "in.fa", "-o", "out.motex", "-d", str(d), "-k", str(l), "-e", str(e),
            "-q", str(rng.choice([20, 40])), "-s", "in.boxes"]
    return seqs, boxes, args


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(16))
def test_wide_and_many_structures_vs_oracle(native_built, oracle_port, seed):
    rng = random.Random(9300 + seed)
    seqs, boxes, args = wide_case(rng)
    files = {"in.fa": fasta(seqs), "in.boxes": boxes_text(boxes)}
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0, g[2] + o[2]
    assert g[1] == o[1]
