"""Word search (motex_gpu_search, the counting loop of the reference's -I
mode, motex.cc:938-1000) against the oracle's per-pair restatement summed
over the sequences, bit-exact: for each word, u = sequences holding its last
l symbols within e errors, v = all such occurrences."""
import ctypes as C
import random

import pytest

from conftest import PORT_LIB


def oracle_search(d, l, e, words, seqs):
    lib = C.CDLL(PORT_LIB)
    us, vs = [], []
    for w in words:
        if len(w) < l:
            us.append(0)
            vs.append(0)
            continue
        x = w[-l:]
        u = v = 0
        for t in seqs:
            if len(t) < l:                           # motex.cc:977-982
                continue
            U = (C.c_uint32 * l)()
            V = (C.c_uint32 * l)()
            lib.oracle_extract_pair(d, l, e, x.encode(), l, t.encode(), len(t), U, V)
            u += U[l - 1]
            v += V[l - 1]
        us.append(u)
        vs.append(v)
    return us, vs


@pytest.mark.gpu
@pytest.mark.parametrize("d", [0, 1])
def test_search_random(native_built, gpu_ctx, oracle_port, d):
    rng = random.Random(300 + d)
    for case in range(30):
        alpha = rng.choice(["ACGT", "ACGTN", "ARNDCQEGHILKMFPSTWYV", "0123456789"])
        l = rng.choice([4, 6, 8, 10, 12, 15, 20, 31, 32, 33, 48])
        e = rng.randint(0, min(l - 1, 4))
        seqs = ["".join(rng.choice(alpha) for _ in range(rng.choice([rng.randint(1, l + 2), rng.randint(l, 600)])))
                for _ in range(rng.randint(1, 25))]
        words = []
        for _ in range(rng.randint(1, 60)):
            kind = rng.random()
            if kind < 0.5 and any(len(s) >= l for s in seqs):
                s = rng.choice([s for s in seqs if len(s) >= l])
                a = rng.randint(0, len(s) - l)
                w = list(s[a:a + l])
                for _ in range(rng.randint(0, e + 1)):
                    w[rng.randrange(l)] = rng.choice(alpha)
                w = "".join(rng.choice(alpha) for _ in range(rng.randint(0, 5))) + "".join(w)
            elif kind < 0.8:
                w = "".join(rng.choice(alpha) for _ in range(rng.randint(l, l + 6)))
            elif kind < 0.9:
                w = "".join(rng.choice(alpha) for _ in range(rng.randint(0, l - 1)))   # too short: 0, 0
            else:
                w = "".join(rng.choice(alpha + "WXZ") for _ in range(l))              # symbols no text holds
            words.append(w)
        prm = native_built.make_params(d, l, e)
        got = gpu_ctx.search(words, seqs, prm)
        assert got == oracle_search(d, l, e, words, seqs), (case, d, l, e)


@pytest.mark.gpu
def test_search_edges(native_built, gpu_ctx):
    prm = native_built.make_params(1, 5, 1)
    assert gpu_ctx.search([], ["ACGTACGT"], prm) == ([], [])
    assert gpu_ctx.search(["ACG"], ["ACGTACGT"], prm) == ([0], [0])        # word shorter than l
    assert gpu_ctx.search(["ACGTA"], ["ACG", "TT"], prm) == ([0], [0])     # every sequence skipped
    u, v = gpu_ctx.search(["ACGTA", "ACGTA"], ["ACGTACGTA", "ACGTA"], prm)
    assert u[0] == u[1] == 2 and v[0] == v[1] > 0                          # duplicates are counted alike
