"""Text chunks of the edit-distance DP restart their column l + e - 1
positions before the first position they count (build_chunks in
motex_gb300/csrc/motex_gpu.cu): a hit at position j needs an alignment of
cost <= e, whose text part is at most l + e symbols long and so starts no
earlier than j - (l + e) + 1.  Checked here with a Sellers column over whole
texts against chunked runs with that warm-up, and shown tight: one position
less misses hits."""
import random


def sellers(p, t, e, start=0):
    """Hit flags for positions start..len(t)-1, column started fresh at start."""
    l = len(p)
    col = list(range(l + 1))
    out = []
    for c in t[start:]:
        prev = col[:]
        col[0] = 0
        for i in range(1, l + 1):
            col[i] = min(prev[i] + 1, col[i - 1] + 1, prev[i - 1] + (p[i - 1] != c))
        out.append(col[l] <= e)
    return out


def chunked(p, t, e, cuts, warm):
    """Hits of a run cut at `cuts`, each chunk restarted `warm` positions early."""
    bounds = [0] + sorted(cuts) + [len(t)]
    out = []
    for a, b in zip(bounds, bounds[1:]):
        s = max(0, a - warm)
        out += sellers(p, t[:b], e, s)[a - s:]
    return out


def test_warmup_of_l_plus_e_minus_1_is_exact():
    rng = random.Random(5)
    for _ in range(400):
        l = rng.randint(1, 20)
        e = rng.randint(0, min(l - 1, 5))
        alpha = rng.choice(["AC", "ACGT", "ACDEFGHIKLMNPQRSTVWY"])
        t = "".join(rng.choice(alpha) for _ in range(rng.randint(1, 200)))
        p = "".join(rng.choice(alpha) for _ in range(l))
        if rng.random() < 0.5 and len(t) > l:                # plant a copy of the factor
            a = rng.randint(0, len(t) - l)
            t = t[:a] + p + t[a + l:]
        cuts = sorted(rng.sample(range(1, len(t)), min(len(t) - 1, rng.randint(0, 5)))) if len(t) > 1 else []
        assert chunked(p, t, e, cuts, l + e - 1) == sellers(p, t, e), (p, e, cuts)


def test_one_position_less_misses_hits():
    """ACGT with one error occurs as ACXGT (an insertion): five text symbols,
    and every shorter window ending at its T costs 2; a chunk starting at that
    T needs all four earlier positions."""
    p, e = "ACGT", 1
    t = "GGGGACXGTGGGG"
    cut = t.index("ACXGT") + 4                             # the occurrence ends here
    assert sellers(p, t, e)[cut]
    assert chunked(p, t, e, [cut], len(p) + e - 1) == sellers(p, t, e)
    assert chunked(p, t, e, [cut], len(p) + e - 2) != sellers(p, t, e)
