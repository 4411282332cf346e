"""Structured edit distance with the SWAR lanes filling the register.

The one-gap block kernel (k_dp_struct1_swar_blk) and the any-gap block kernel
(k_dp_structN_blk) pack box 0 and the box rows as lanes with a guard bit
above each.  When the top lane ends below bit 31 the score fields are updated
by one arithmetic shift of ph - mh; when it ends at bit 31 (lengths summing
to 32 with the guards) that difference needs 33 bits and the kernels keep two
shifts.  Both layouts, against the oracle CLI on seeded inputs with planted
structured occurrences."""
import random

import pytest

from helpers import run_cli


def fasta(seqs):
    return "".join(f">s{i}\n{s}\n" for i, s in enumerate(seqs))


def boxes_text(boxes):
    return f"{len(boxes)}\n" + "".join(f"{a}\n{b}\n{c}\n{d}\n" for a, b, c, d in boxes)


def planted(rng, l, boxes, nseq=8):
    seqs = ["".join(rng.choice("ACGT") for _ in range(rng.randint(150, 400))) for _ in range(nseq)]
    parts = ["".join(rng.choice("ACGT") for _ in range(l))] + \
        ["".join(rng.choice("ACGT") for _ in range(b[2])) for b in boxes]
    for i in range(nseq):
        for _ in range(rng.randint(1, 3)):
            occ = parts[0]
            for (gmin, gmax, _, _), box in zip(boxes, parts[1:]):
                occ += "".join(rng.choice("ACGT") for _ in range(rng.randint(gmin, gmax))) + box
            a = rng.randint(0, len(seqs[i]) - len(occ))
            seqs[i] = seqs[i][:a] + occ + seqs[i][a + len(occ):]
    return seqs


# (l, e, boxes): bits the lanes span = l + sum(1 + row length); the one-gap
# kernel packs box 0 and the box twice (two rows), the any-gap kernel box 0
# and one row per box
SHAPES = [
    (8, 1, [(3, 6, 11, 1)]),                  # one gap, 8 + 1 + 11 + 1 + 11 = 32: top lane at bit 31
    (8, 1, [(3, 6, 10, 1)]),                  # one gap, 30 bits: one-shift update
    (9, 2, [(2, 4, 10, 2)]),                  # one gap, 9 + 1 + 10 + 1 + 10 = 31
    (8, 1, [(1, 3, 11, 1), (2, 4, 11, 2)]),   # two gaps, 8 + 1 + 11 + 1 + 11 = 32
    (8, 1, [(1, 3, 10, 1), (2, 4, 11, 2)]),   # two gaps, 8 + 1 + 10 + 1 + 11 = 31
    (6, 1, [(0, 2, 7, 1), (1, 2, 7, 1), (0, 1, 8, 1)]),   # three gaps, 6+1+7+1+7+1+8 = 31
]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", range(len(SHAPES)))
@pytest.mark.parametrize("seed", range(2))
def test_lane_fill_vs_oracle(native_built, oracle_port, shape, seed):
    l, e, boxes = SHAPES[shape]
    rng = random.Random(9700 + 10 * shape + seed)
    seqs = planted(rng, l, boxes)
    files = {"in.fa": fasta(seqs), "in.boxes": boxes_text(boxes)}
    args = ["-a", "DNA", "-i", "in.fa", "-o", "out.motex", "-d", "1", "-k", str(l), "-e", str(e),
            "-q", "25", "-s", "in.boxes"]
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert g[0] == o[0] == 0, g[2] + o[2]
    assert g[1] == o[1]
    assert g[1].count("\n") > 14                  # motifs printed
