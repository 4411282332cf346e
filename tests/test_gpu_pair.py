"""Per-pair drop-in (motex_gpu_extract_pair, replacing motifs_extraction_hd/_ed)
against the oracle's restatement of the same wrapper, bit-exact."""
import ctypes as C
import random

import pytest

from conftest import PORT_LIB


def oracle_pair(d, l, e, p, t):
    lib = C.CDLL(PORT_LIB)
    m = len(p)
    U = (C.c_uint32 * m)()
    V = (C.c_uint32 * m)()
    lib.oracle_extract_pair(d, l, e, p.encode(), m, t.encode(), len(t), U, V)
    return list(U), list(V)


ALPHABETS = {"DNA": "ACGT", "DNAN": "ACGTN", "PROT": "ARNDCQEGHILKMFPSTWYV", "USR": "0123456789", "BIN": "AC"}


@pytest.mark.gpu
@pytest.mark.parametrize("d", [0, 1])
def test_pair_random(native_built, gpu_ctx, oracle_port, d):
    rng = random.Random(7 + d)
    for case in range(80):
        alpha = ALPHABETS[rng.choice(list(ALPHABETS))]
        l = rng.choice([1, 2, 5, 8, 12, 15, 20, 28, 29, 31, 32, 33, 40, 64, 65, 90])
        e = rng.randint(0, min(l - 1, 6))
        m = rng.randint(l, l + 150)
        n = rng.randint(1, 400)
        p = "".join(rng.choice(alpha) for _ in range(m))
        t = "".join(rng.choice(alpha) for _ in range(n))
        if n >= l and rng.random() < 0.7:              # plant a few near-copies
            for _ in range(3):
                a = rng.randint(0, m - l)
                b = rng.randint(0, n - l)
                w = list(p[a:a + l])
                for _ in range(rng.randint(0, e)):
                    w[rng.randrange(l)] = rng.choice(alpha)
                t = t[:b] + "".join(w) + t[b + l:]
        prm = native_built.make_params(d, l, e)
        got = gpu_ctx.extract_pair(p, t, prm)
        assert got == oracle_pair(d, l, e, p, t), (case, d, l, e, m, n)


@pytest.mark.gpu
def test_pair_accumulates(native_built, gpu_ctx, oracle_port):
    """u and v are accumulated (+=) like the reference wrappers do."""
    p, t1, t2 = "ACGTACGTTGCA" * 4, "ACGTACGTAA" * 6, "TTGCAACGTA" * 5
    prm = native_built.make_params(1, 6, 1)
    u, v = gpu_ctx.extract_pair(p, t1, prm)
    u, v = gpu_ctx.extract_pair(p, t2, prm, u, v)
    u1, v1 = oracle_pair(1, 6, 1, p, t1)
    u2, v2 = oracle_pair(1, 6, 1, p, t2)
    assert u == [a + b for a, b in zip(u1, u2)] and v == [a + b for a, b in zip(v1, v2)]
