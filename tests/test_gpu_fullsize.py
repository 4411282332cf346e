"""Parity at the benchmark sizes, where the CPU oracle cannot redo the whole
run: size-independent properties of the output, a metamorphic check
(every sequence given twice => same motifs, u and v doubled), and sampled
per-word totals recomputed by the oracle over all sequences."""
import ctypes as C
import random

import pytest

from conftest import PORT_LIB
from motex_gb300 import workloads as W


def _qok(u, n, q, Q):
    r = (u / n) * 100
    return q <= r <= Q


def _check_properties(wl, res):
    n = len(wl.seqs)
    words, last = set(), (-1, -1)
    for seq, pos, k, u, v in res.motifs:
        w = wl.seqs[seq][pos - wl.k + 1: pos + 1]
        assert w not in words
        words.add(w)
        assert (seq, pos) > last
        last = (seq, pos)
        assert 1 <= u <= n and u <= v and wl.n <= v <= wl.N and _qok(u, n, wl.q, wl.Q)
    return words


def _oracle_uv(wl, word):
    lib = C.CDLL(PORT_LIB)
    text = "".join(wl.seqs).encode()
    offs = [0]
    for s in wl.seqs:
        offs.append(offs[-1] + len(s))
    O = (C.c_uint * len(offs))(*offs)
    u, v = C.c_uint(), C.c_uint()
    lib.oracle_word_uv(wl.d, wl.k, wl.e, word.encode(), text, O, len(wl.seqs), wl.k, C.byref(u), C.byref(v))
    return u.value, v.value


def _sampled_oracle(wl, res, rng, n_printed=25, n_random=25):
    printed = {wl.seqs[s][p - wl.k + 1: p + 1]: (u, v) for s, p, _, u, v in res.motifs}
    for w in rng.sample(sorted(printed), min(n_printed, len(printed))):
        assert _oracle_uv(wl, w) == printed[w], w
    for _ in range(n_random):
        s = rng.randrange(len(wl.seqs))
        if len(wl.seqs[s]) < wl.k:
            continue
        p = rng.randrange(wl.k - 1, len(wl.seqs[s]))
        w = wl.seqs[s][p - wl.k + 1: p + 1]
        u, v = _oracle_uv(wl, w)
        passes = _qok(u, len(wl.seqs), wl.q, wl.Q) and wl.n <= v <= wl.N
        assert (w in printed) == passes, w
        if passes:
            assert printed[w] == (u, v)


def _run(native, ctx, wl):
    return ctx.run(wl.seqs, native.make_params(wl.d, wl.k, wl.e, wl.q, wl.Q, wl.n, wl.N, wl.boxes))


@pytest.mark.gpu
def test_dna_ed_full_properties_and_duplication(native_built, gpu_ctx, oracle_port):
    wl = W.dna_ed()                                   # 1200 x U[800,1200], -d 1 -k 15 -e 3 -q 10
    res = _run(native_built, gpu_ctx, wl)
    assert res.ref_cells == sum(map(len, wl.seqs)) ** 2
    words = _check_properties(wl, res)
    assert len(words) > 1000
    _sampled_oracle(wl, res, random.Random(1))
    dup = W.Workload("dup", wl.alphabet, wl.seqs + wl.seqs, wl.d, wl.k, wl.e, wl.q, N=10 ** 9)
    res2 = _run(native_built, gpu_ctx, dup)
    base = _run(native_built, gpu_ctx, W.Workload("b", wl.alphabet, wl.seqs, wl.d, wl.k, wl.e, wl.q, N=10 ** 9))
    assert [(s, p, 2 * u, 2 * v) for s, p, _, u, v in base.motifs] == [(s, p, u, v) for s, p, _, u, v in res2.motifs]


@pytest.mark.gpu
@pytest.mark.parametrize("d", [0, 1])
def test_prot_uneven_full_sampled_oracle(native_built, gpu_ctx, oracle_port, d):
    wl = W.prot_uneven(d=d)                           # 2000 x logU[50,2000] aa, -k 10 -e 2 -q 15
    res = _run(native_built, gpu_ctx, wl)
    _check_properties(wl, res)
    _sampled_oracle(wl, res, random.Random(10 + d))


@pytest.mark.gpu
def test_dna_long_quarter_sampled_oracle(native_built, gpu_ctx, oracle_port):
    wl = W.dna_long(scale=0.25)                       # 8 x 250,000 nt with tandem repeats, -k 20 -e 3 -q 50
    res = _run(native_built, gpu_ctx, wl)
    _check_properties(wl, res)
    _sampled_oracle(wl, res, random.Random(3), n_printed=15, n_random=10)
