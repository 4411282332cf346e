"""The packed edit-distance register step (dp_swar_body in
motex_gb300/csrc/dp_body.cuh, constants from swar_const in dp.cu) restated
bit for bit in 32-bit arithmetic and checked against a Sellers DP column on
random factors and texts: NL factors share a register in lanes of
S = max(l+1, 6) bits with guard bits above each lane, scores held as
score + K per field, hit counts in S-bit fields drained every 32 positions.
The same check with the narrower stride S = l+1 fails for k = 4 (a block of
32 hits overflows a 5-bit count field into the next lane), which is how that
layout bug was found."""
import random

import pytest

M32 = 0xFFFFFFFF


def sellers_hits(p, t, e):
    """Per text position: min edit distance of p to a suffix of t[..j] <= e."""
    l = len(p)
    col = list(range(l + 1))
    out = []
    for c in t:
        prev = col[:]
        col[0] = 0
        for i in range(1, l + 1):
            col[i] = min(prev[i] + 1, col[i - 1] + 1, prev[i - 1] + (p[i - 1] != c))
        out.append(col[l] <= e)
    return out


def stride(l):
    return max(l + 1, 6)


def lanes(l, S):
    return min(4, (32 - l) // S + 1)


def consts(l, e, NL, S):
    HB = K = SC0 = guards = 0
    for j in range(NL):
        o = j * S
        HB |= 1 << (o + l - 1)
        for g in range(o + l, min(o + S, 32)):
            guards |= 1 << g
        K += ((1 << (l - 1)) - (e + 1)) << o
        SC0 += l << o
    NG = ~guards & M32
    return dict(HB=HB, NG=NG, NGm1=NG & ~HB & M32, K=K, SC0=SC0, FM=(1 << S) - 1)


def swar_counts(pats, text, l, e, S):
    """Hit counts of NL = len(pats) factors in one register over text."""
    NL = len(pats)
    C = consts(l, e, NL, S)
    sh = l - 1
    eq = {}
    for c in set(text):
        x = 0
        for j, p in enumerate(pats):
            for q in range(l):
                if p[q] == c:
                    x |= 1 << (j * S + q)
        eq[c] = (x | (~C["NG"] & M32)) & M32            # Eq = 1 at the guards
    Pv, Mv, sc, cnt = C["NG"], 0, (C["SC0"] + C["K"]) & M32, 0
    counts = [0] * NL
    for k, ch in enumerate(text):
        Eq = eq[ch]
        Xv = Eq | Mv
        s = ((Eq & Pv) + Pv) & M32
        Xh = (s ^ Pv) | Eq
        Ph = (Mv | ~(Xh | Pv)) & M32
        Mhs = Pv & Xh & C["NGm1"]
        mh = Pv & Xh & C["HB"]
        ph = Ph & C["HB"]
        sc = (sc + (ph >> sh) - (mh >> sh)) & M32
        Ph2, Mh2 = (Ph << 1) & M32, (Mhs << 1) & M32
        Pv = (Mh2 | ~(Xv | Ph2)) & M32
        Mv = Ph2 & Xv & C["NG"]
        cnt = (cnt + (((~sc & M32) & C["HB"]) >> sh)) & M32
        if k % 32 == 31 or k == len(text) - 1:               # drain per 32-position block
            for j in range(NL):
                counts[j] += (cnt >> (j * S)) & C["FM"]
            cnt = 0
    return counts


@pytest.mark.parametrize("l", range(4, 16))
def test_packed_lanes_match_sellers(l):
    rng = random.Random(100 + l)
    S = stride(l)
    NL = lanes(l, S)
    assert (NL - 1) * S + l <= 32
    for e in range(0, min(l - 1, 5) + 1):
        for alpha in ("ACGT", "ACDEFGHIKLMNPQRSTVWY"):
            pats = ["".join(rng.choice(alpha) for _ in range(l)) for _ in range(NL)]
            text = "".join(rng.choice(alpha) for _ in range(150))
            assert swar_counts(pats, text, l, e, S) == [sum(sellers_hits(p, text, e)) for p in pats], (l, e, alpha)


def test_narrow_stride_overflows_for_k4():
    """With S = l + 1 = 5 a block of 32 hits does not fit a count field."""
    rng = random.Random(7)
    l, e, S = 4, 3, 5
    pats = ["".join(rng.choice("ACGT") for _ in range(l)) for _ in range(lanes(l, S))]
    text = "".join(rng.choice("ACGT") for _ in range(200))
    assert swar_counts(pats, text, l, e, S) != [sum(sellers_hits(p, text, e)) for p in pats]
