"""The popc-free Hamming form (k_dp_hclr: two or three factors per register
in guarded lanes, the third unguarded and tested by a compare, mismatches
counted by clearing each lane's lowest set bit e times), the default for
Hamming with e <= 3 and 5 <= l <= 12: motexGPU against
the oracle CLI on seeded inputs with planted approximate occurrences, for
DNA and protein, with two and three lanes (MOTEX_DP_CLEAR=2 / 3) and W = 4
and W = 8 register words per thread, and the popc forms (MOTEX_DP_CLEAR=0)
on the same input."""
import random

import pytest

from helpers import run_cli


def fasta(seqs):
    return "".join(f">s{i}\n{s}\n" for i, s in enumerate(seqs))


def case(rng, letters, l, e):
    seqs = ["".join(rng.choice(letters) for _ in range(rng.randint(40, 400))) for _ in range(rng.randint(6, 14))]
    motif = "".join(rng.choice(letters) for _ in range(l))
    for i in range(len(seqs)):
        for _ in range(rng.randint(0, 3)):
            occ = list(motif)
            for q in rng.sample(range(l), rng.randint(0, e)):
                occ[q] = rng.choice(letters)
            if len(seqs[i]) >= l:
                a = rng.randint(0, len(seqs[i]) - l)
                seqs[i] = seqs[i][:a] + "".join(occ) + seqs[i][a + l:]
    return seqs


@pytest.mark.gpu
@pytest.mark.parametrize("l", [5, 8, 10, 12])
@pytest.mark.parametrize("e", [0, 1, 2, 3])
@pytest.mark.parametrize("kind", ["DNA", "PROT"])
def test_guarded_lanes_vs_oracle(native_built, oracle_port, monkeypatch, l, e, kind):
    if e >= l:
        pytest.skip("e < l")
    letters = "ACGT" if kind == "DNA" else "ARNDCQEGHILKMFPSTWYV"
    rng = random.Random(7100 + 100 * l + 10 * e + (kind == "PROT"))
    seqs = case(rng, letters, l, e)
    files = {"in.fa": fasta(seqs)}
    args = ["-a", kind, "-i", "in.fa", "-o", "out.motex", "-d", "0", "-k", str(l), "-e", str(e), "-q", "20"]
    o = run_cli(oracle_port, None, args + ["-t", "8"], files=files)
    assert o[0] == 0, o[2]
    lanes = [nl for nl in (2, 3) if (nl == 2 and 5 <= l <= 12) or (nl == 3 and 6 <= l <= 10)]
    for nl in lanes:
        monkeypatch.setenv("MOTEX_DP_CLEAR", str(nl))
        for w in ("4", "8"):
            monkeypatch.setenv("MOTEX_DP_W", w)
            g = run_cli(native_built.CLI_PATH, None, args, files=files)
            assert g[0] == 0, g[2]
            assert g[1] == o[1], (nl, w, l, e, kind)
    monkeypatch.delenv("MOTEX_DP_W")
    monkeypatch.setenv("MOTEX_DP_CLEAR", "0")
    p = run_cli(native_built.CLI_PATH, None, args, files=files)
    assert p[0] == 0 and p[1] == o[1]
