"""Seeded workload generators: deterministic and shaped as specified."""
import numpy as np

from motex_gb300 import workloads as W


def test_deterministic():
    assert W.dna_hd_small(seed=1).seqs == W.dna_hd_small(seed=1).seqs
    assert W.prot_uneven(seed=3, scale=0.01).seqs == W.prot_uneven(seed=3, scale=0.01).seqs
    assert W.dna_hd_small(seed=1).seqs != W.dna_hd_small(seed=2).seqs


def test_shapes():
    w = W.dna_hd_small()
    assert len(w.seqs) == 64 and all(len(s) == 500 for s in w.seqs)
    assert (w.d, w.k, w.e, w.q) == (0, 12, 2, 50)
    w = W.dna_ed(scale=0.05)
    assert all(800 <= len(s) <= 1200 for s in w.seqs) and (w.d, w.k, w.e, w.q) == (1, 15, 3, 10)
    gc = np.mean([ (s.count("G") + s.count("C")) / len(s) for s in w.seqs])
    assert 0.36 < gc < 0.44
    w = W.prot_uneven(scale=0.05)
    assert all(50 <= len(s) <= 2000 for s in w.seqs) and set("".join(w.seqs)) <= set(W.AMINO20)
    w = W.dna_long(scale=0.001)
    assert len(w.seqs) == 8 and all(len(s) == 1000 for s in w.seqs)
    s = W.structured(scale=0.01)
    assert s.boxes == ((5, 15, 10, 1),) and (s.k, s.e) == (8, 1)


def test_serve_stream():
    reqs = W.serve_stream(nreq=50)
    ts = [t for t, _ in reqs]
    assert ts == sorted(ts)
    for _, w in reqs:
        assert 8 <= len(w.seqs) <= 256 and w.e < w.k / 3 + 1 and w.q in (10, 25, 50)
        assert w.k <= (12 if w.alphabet == "PROT" else 24)
