"""The small-job pipeline (k_mini_prep / DP / k_mini_post: one CTA per job
for every stage around the DP, hash-table factor dedup) against the staged
pipeline (MOTEX_MINI=0: presence, TMA packing, radix-sort dedup, scans) on
seeded random whole-set inputs, bit for bit; a batch of many small jobs
against each job run alone through the staged pipeline; and the inputs
where the dedup table is stressed (every factor equal, l = 1, keys of 62-63
bits) or empty (no sequence as long as a factor).  The golden fixtures from
the reference run through this pipeline too: motexGPU takes it for every
input of at most 131072 symbols."""
import random

import pytest

ALPHABETS = {"DNA": "ACGT", "DNAN": "ACGTN", "PROT": "ARNDCQEGHILKMFPSTWYV", "DIGITS": "0123456789", "BIN": "AC",
             "ONE": "A"}


def random_job(rng, native):
    name = rng.choice(list(ALPHABETS))
    alpha = ALPHABETS[name]
    B = max(2, (len(alpha) - 1).bit_length())
    l = rng.randint(1, min(31, 63 // B))
    e = rng.randint(0, min(l - 1, 4))
    d = rng.randint(0, 1)
    nseq = rng.randint(1, 40)
    seqs = []
    for _ in range(nseq):
        n = rng.choice([rng.randint(1, 12), rng.randint(20, 400), rng.randint(400, 3000)])
        seqs.append("".join(rng.choice(alpha) for _ in range(n)))
    # plant a few near-copies so that some words pass the quorum
    if rng.random() < 0.8:
        w = "".join(rng.choice(alpha) for _ in range(l))
        for i in range(nseq):
            if rng.random() < 0.5 and len(seqs[i]) >= l:
                a = rng.randint(0, len(seqs[i]) - l)
                seqs[i] = seqs[i][:a] + w + seqs[i][a + l:]
    q = rng.choice([0, 5, 20, 50])
    n_min, n_max = rng.choice([(1, 10000), (1, 10000), (2, 40)])
    return seqs, native.make_params(d, l, e, q, 100, n_min, n_max)


def staged(ctx, monkeypatch, seqs, prm):
    monkeypatch.setenv("MOTEX_MINI", "0")
    r = ctx.run(seqs, prm)
    monkeypatch.delenv("MOTEX_MINI")
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(40))
def test_mini_equals_staged(native_built, gpu_ctx, monkeypatch, seed):
    rng = random.Random(7700 + seed)
    seqs, prm = random_job(rng, native_built)
    mini = gpu_ctx.run(seqs, prm)
    ref = staged(gpu_ctx, monkeypatch, seqs, prm)
    assert mini.motifs == ref.motifs
    assert mini.unique_words == ref.unique_words
    assert mini.ref_cells == ref.ref_cells


@pytest.mark.gpu
def test_mini_batch_of_many_jobs(native_built, gpu_ctx, monkeypatch):
    rng = random.Random(7800)
    jobs = [random_job(rng, native_built) for _ in range(60)]
    batch = gpu_ctx.run_batch(jobs)
    alone = [staged(gpu_ctx, monkeypatch, s, p) for s, p in jobs]
    assert [b.motifs for b in batch] == [a.motifs for a in alone]
    assert [b.unique_words for b in batch] == [a.unique_words for a in alone]
    assert sum(len(a.motifs) for a in alone) > 100
    # mixed with a job above the small-job size: both pipelines in one call
    big = ("ACGT" * 40000, native_built.make_params(0, 12, 1, 0))
    mixed = gpu_ctx.run_batch(jobs[:5] + [big] + jobs[5:10])
    assert [m.motifs for m in mixed[:5]] == [a.motifs for a in alone[:5]]
    assert [m.motifs for m in mixed[6:]] == [a.motifs for a in alone[5:10]]
    assert mixed[5].motifs == staged(gpu_ctx, monkeypatch, *big).motifs


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["all_equal", "l1", "key62", "key63", "no_factor", "one_symbol"])
def test_mini_edge_inputs(native_built, gpu_ctx, monkeypatch, case):
    P = native_built.make_params
    if case == "all_equal":                    # every factor has the same key: one table slot
        seqs, prm = ["A" * 5000] * 8, P(1, 10, 2, 0)
    elif case == "l1":
        seqs, prm = ["ACGTTGCA" * 50, "TTTT" * 30, "G"], P(0, 1, 0, 0)
    elif case == "key62":                      # 31 DNA symbols: 62-bit keys
        rng = random.Random(3)
        seqs, prm = ["".join(rng.choice("ACGT") for _ in range(900)) for _ in range(6)], P(1, 31, 3, 0)
        seqs[3] = seqs[0][100:500] + seqs[3][400:]
    elif case == "key63":                      # 21 symbols of 3 bits: 63-bit keys, the largest
        rng = random.Random(4)
        seqs, prm = ["".join(rng.choice("ACGTN") for _ in range(700)) for _ in range(6)], P(0, 21, 4, 0)
        seqs[2] = seqs[1][:300] + seqs[2][300:]
    elif case == "no_factor":                  # no sequence as long as a factor
        seqs, prm = ["ACGT", "ACG", "A"], P(0, 6, 1, 0)
    else:                                      # one symbol: two bit planes all zero
        seqs, prm = ["CCCCCCCC", "CCCC", "CCCCCCCCCCCC"], P(0, 3, 0, 0)
    mini = gpu_ctx.run(seqs, prm)
    ref = staged(gpu_ctx, monkeypatch, seqs, prm)
    assert mini.motifs == ref.motifs
    assert mini.unique_words == ref.unique_words
