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


def oracle_pair_struct(d, l, e, boxes, p, t):
    lib = C.CDLL(PORT_LIB)
    ng = len(boxes)
    cols = [(C.c_uint * ng)(*[b[i] for b in boxes]) for i in range(4)]
    ns = 1
    for g in boxes:
        ns *= g[1] - g[0] + 1
    U = (C.c_uint32 * (len(p) * ns))()
    V = (C.c_uint32 * (len(p) * ns))()
    lib.oracle_extract_pair_struct(d, l, e, ng, cols[0], cols[1], cols[2], cols[3], p.encode(), len(p),
                                   t.encode(), len(t), U, V)
    return list(U), list(V), ns


@pytest.mark.gpu
@pytest.mark.parametrize("d", [0, 1])
def test_pair_structured(native_built, gpu_ctx, oracle_port, d):
    """structured_motifs_extraction_hd/_ed drop-in: one gap (shared-history
    kernel), a long gap and two gaps (box-check kernel)."""
    rng = random.Random(300 + d)
    # one gap packed in one register (edit distance), one gap that does not fit the
    # packed lanes, a long gap and two gaps (box-check kernel)
    shapes = [((6, 4, 1), ((2, 6, 5, 1),)), ((7, 1, 0), ((20, 26, 6, 1),)),
              ((5, 1, 1), ((1, 3, 5, 1), (2, 3, 4, 0))), ((8, 2, 2), ((4, 9, 7, 2),)),
              ((12, 3, 2), ((2, 5, 12, 2),))]
    for case in range(30):
        (l, _, e), boxes = shapes[case % len(shapes)]
        e = min(e, l - 1)
        m, n = rng.randint(60, 160), rng.randint(60, 200)
        p = "".join(rng.choice("ACGT") for _ in range(m))
        t = "".join(rng.choice("ACGT") for _ in range(n))
        # plant one copy of a structured occurrence of p into t
        a = rng.randint(0, m - 45)
        seg = p[a:a + 45]
        b = rng.randint(0, n - 45)
        t = t[:b] + seg + t[b + 45:]
        U, V, ns = oracle_pair_struct(d, l, e, boxes, p, t)
        prm = native_built.make_params(d, l, e, boxes=boxes)
        got = gpu_ctx.extract_pair(p, t, prm, nb_structs=ns)
        assert got == (U, V), (case, d, l, e, boxes)
        assert sum(V) > 0
