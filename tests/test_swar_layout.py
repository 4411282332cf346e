"""The packed edit-distance register step (dp_swar_body in
motex_gb300/csrc/dp_body.cuh, constants from swar_const in dp.cu) restated
bit for bit in 32-bit arithmetic and checked against a Sellers DP column on
random factors and texts: NL factors share a register in lanes of
S = max(l+1, 6) bits with guard bits above each lane, scores held as
score + K per field with the hit flag at bit h, hit counts drained every 32
positions.
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
    """swar_const: hit bit h = ceil(log2 l) of each score field and 6-bit
    count fields at h for NL = 2, 3; h = l-1 and S-bit count fields at the
    lane base for NL = 4."""
    h = l - 1 if NL == 4 else (l - 1).bit_length()
    HB = HQ = K = SC0 = guards = 0
    for j in range(NL):
        o = j * S
        HB |= 1 << (o + l - 1)
        HQ |= 1 << (o + h)
        for g in range(o + l, min(o + S, 32)):
            guards |= 1 << g
        K += ((1 << h) - (e + 1)) << o
        SC0 += l << o
    NG = ~guards & M32
    return dict(HB=HB, HQ=HQ, NG=NG, NGm1=NG & ~HB & M32, K=K, SC0=SC0, Q=0 if NL == 4 else h,
                FM=(1 << S) - 1 if NL == 4 else 63)


def signed32(x):
    return x - (1 << 32) if x & (1 << 31) else x


def swar_counts(pats, text, l, e, S, one_shift=False):
    """Hit counts of NL = len(pats) factors in one register over text.
    one_shift: the score update of the NL = 2, 4 kernels, ph - mh taken as a
    signed word and moved to the score fields by one arithmetic shift."""
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
        if one_shift:
            sc = (sc + (signed32((ph - mh) & M32) >> sh)) & M32
        else:
            sc = (sc + (ph >> sh) - (mh >> sh)) & M32
        Ph2, Mh2 = (Ph << 1) & M32, (Mhs << 1) & M32
        Pv = (Mh2 | ~(Xv | Ph2)) & M32
        Mv = Ph2 & Xv & C["NG"]
        hits = (~sc & M32) & C["HQ"]
        cnt = (cnt + (hits if NL != 4 else hits >> sh)) & M32   # NL = 2, 3: added in place
        if k % 32 == 31 or k == len(text) - 1:               # drain per 32-position block
            for j in range(NL):
                counts[j] += (cnt >> (j * S + C["Q"])) & C["FM"]
            cnt = 0
    return counts


@pytest.mark.parametrize("l", range(4, 16))
def test_packed_lanes_match_sellers(l):
    rng = random.Random(100 + l)
    S = stride(l)
    NL = lanes(l, S)
    assert (NL - 1) * S + l <= 32
    # e = l - 1: nearly every position is a hit, 32 per block fill a count field
    for e in sorted(set(range(0, min(l - 1, 5) + 1)) | {l - 1}):
        for alpha in ("ACGT", "ACDEFGHIKLMNPQRSTVWY"):
            pats = ["".join(rng.choice(alpha) for _ in range(l)) for _ in range(NL)]
            text = "".join(rng.choice(alpha) for _ in range(150))
            assert swar_counts(pats, text, l, e, S) == [sum(sellers_hits(p, text, e)) for p in pats], (l, e, alpha)


@pytest.mark.parametrize("l", [l for l in range(4, 16) if lanes(l, stride(l)) != 3])
def test_one_shift_score_update_matches_sellers(l):
    """NL = 2, 4 (the lanes' top bit at most 30): one arithmetic shift of
    ph - mh gives the same counts as the two shifts."""
    rng = random.Random(300 + l)
    S = stride(l)
    NL = lanes(l, S)
    assert (NL - 1) * S + l - 1 <= 30
    for e in range(0, min(l - 1, 5) + 1):
        for alpha in ("ACGT", "ACDEFGHIKLMNPQRSTVWY"):
            pats = ["".join(rng.choice(alpha) for _ in range(l)) for _ in range(NL)]
            text = "".join(rng.choice(alpha) for _ in range(150))
            assert swar_counts(pats, text, l, e, S, one_shift=True) == \
                [sum(sellers_hits(p, text, e)) for p in pats], (l, e, alpha)


def test_one_shift_fails_when_the_top_lane_reaches_bit_31():
    """l = 10 packs three lanes with the top one's bit l-1 at bit 31: ph - mh
    needs 33 bits there, so that layout keeps the two shifts."""
    l, S = 10, stride(10)
    NL = lanes(l, S)
    assert NL == 3 and (NL - 1) * S + l - 1 == 31
    rng = random.Random(11)
    bad = 0
    for _ in range(20):
        pats = ["".join(rng.choice("ACGT") for _ in range(l)) for _ in range(NL)]
        text = "".join(rng.choice("ACGT") for _ in range(200))
        ref = [sum(sellers_hits(p, text, 3)) for p in pats]
        assert swar_counts(pats, text, l, 3, S) == ref
        bad += swar_counts(pats, text, l, 3, S, one_shift=True) != ref
    assert bad > 0


def test_narrow_stride_overflows_for_k4():
    """With S = l + 1 = 5 a block of 32 hits does not fit a count field."""
    rng = random.Random(7)
    l, e, S = 4, 3, 5
    pats = ["".join(rng.choice("ACGT") for _ in range(l)) for _ in range(lanes(l, S))]
    text = "".join(rng.choice("ACGT") for _ in range(200))
    assert swar_counts(pats, text, l, e, S) != [sum(sellers_hits(p, text, e)) for p in pats]


# ------------------------------------------------------- packed Hamming lanes

def hswar_counts(pats, text, l, e):
    """dp_hswar_body restated: NL factors of l bits per register (no guards),
    the text window replicated into every lane by one multiply with
    REP = sum 2^(j*l), a masked popc per lane, counts in l-bit fields drained
    every 32 positions.  Symbols are compared as whole codes here (one plane);
    the kernel ORs the XORs of its B planes, which is the same mismatch bit."""
    NL = len(pats)
    REP = sum(1 << (j * l) for j in range(NL))
    FM = (1 << l) - 1
    codes = {c: i for i, c in enumerate(sorted(set(text) | set("".join(pats))))}
    nbits = max(1, (len(codes) - 1).bit_length())
    planes_p = [[0] * NL for _ in range(nbits)]
    for j, p in enumerate(pats):
        for q, ch in enumerate(p):
            for b in range(nbits):
                if (codes[ch] >> b) & 1:
                    planes_p[b][j] |= 1 << (j * l + q)
    cnt, counts = 0, [0] * NL
    for k in range(len(text)):
        x = 0
        if k >= l - 1:
            win = text[k - l + 1:k + 1]
            for b in range(nbits):
                w = sum(((codes[ch] >> b) & 1) << q for q, ch in enumerate(win))
                Y = (w * REP) & M32                       # no carries: the copies do not overlap
                x |= sum(planes_p[b]) ^ Y
            for j in range(NL):
                if bin(x & (FM << (j * l))).count("1") <= e:
                    cnt = (cnt + (1 << (j * l))) & M32
        if k % 32 == 31 or k == len(text) - 1:
            for j in range(NL):
                counts[j] += (cnt >> (j * l)) & FM
            cnt = 0
    return counts


def hamming_hits(p, t, e):
    l = len(p)
    return sum(1 for k in range(l - 1, len(t)) if sum(a != b for a, b in zip(p, t[k - l + 1:k + 1])) <= e)


@pytest.mark.parametrize("l", range(6, 17))
def test_packed_hamming_lanes_match(l):
    rng = random.Random(300 + l)
    NL = 32 // l
    for e in (0, 1, l // 2, l - 1):
        for alpha in ("ACG", "ACDEFGHIKLMNPQRSTVWY"):
            pats = ["".join(rng.choice(alpha) for _ in range(l)) for _ in range(NL)]
            text = "".join(rng.choice(alpha) for _ in range(150))
            assert hswar_counts(pats, text, l, e) == [hamming_hits(p, text, e) for p in pats], (l, e, alpha)


def test_packed_hamming_needs_six_bit_lanes():
    """l = 5 fields hold 31 hits: a block of 32 hits (a repeat that matches at
    every position) overflows; l = 6 fields hold it."""
    text = "A" * 100
    for l, ok in ((5, False), (6, True)):
        pats = ["A" * l] * (32 // l)
        assert (hswar_counts(pats, text, l, 0) == [hamming_hits(p, text, 0) for p in pats]) == ok, l


# ------------------------------- popc-free Hamming: guarded lanes, bit clears

def hclr_counts(pats, text, l, e):
    """dp_hswar_body with E = e (hclr_const in dp_hclr.cu) restated: two or
    three factors of l bits in lanes at 0, S = l+1 (and 2S) with a guard bit
    above each lane but the third, set in the mismatch word; e times
    x = (x & (x - L)) | G clears each lane's lowest set bit; the hits of the
    guarded lanes are ~(x - L) & G (a lane that is zero borrows its guard),
    added into 6-bit count fields at the guards; the third lane's hit is
    x < 2^(2S), counted at bit 0; drained every 32 positions."""
    NL, S = len(pats), l + 1
    assert (NL == 2 and 5 <= l <= 12 or NL == 3 and 6 <= l <= 10) and e <= 3
    G = sum(1 << (j * S + l) for j in range(2))
    L = sum(1 << (j * S) for j in range(NL))
    LIM = 1 << (2 * S)
    codes = {c: i for i, c in enumerate(sorted(set(text) | set("".join(pats))))}
    nbits = max(1, (len(codes) - 1).bit_length())
    fp = [0] * nbits
    for j, p in enumerate(pats):
        for q, ch in enumerate(p):
            for b in range(nbits):
                if (codes[ch] >> b) & 1:
                    fp[b] |= 1 << (j * S + q)
    fp[0] |= G
    cnt, counts = 0, [0] * NL
    for k in range(len(text)):
        if k >= l - 1:
            win = text[k - l + 1:k + 1]
            x = 0
            for b in range(nbits):
                w = sum(((codes[ch] >> b) & 1) << q for q, ch in enumerate(win))
                x |= fp[b] ^ ((w * L) & M32)                # window copies at 0 and S
            for _ in range(e):
                x = ((x & ((x - L) & M32)) | G) & M32
            cnt = (cnt + (~((x - L) & M32) & G)) & M32
            if NL == 3 and x < LIM:
                cnt += 1
        if k % 32 == 31 or k == len(text) - 1:
            for j in range(NL):
                counts[j] += (cnt >> (0 if j == 2 else j * S + l)) & 63
            cnt = 0
    return counts


@pytest.mark.parametrize("l,NL", [(l, 2) for l in range(5, 13)] + [(l, 3) for l in range(6, 11)])
def test_guarded_lane_hamming_matches(l, NL):
    rng = random.Random(500 + 20 * NL + l)
    for e in range(0, min(3, l - 1) + 1):
        for alpha in ("ACGT", "ACDEFGHIKLMNPQRSTVWY"):
            for _ in range(3):
                pats = ["".join(rng.choice(alpha) for _ in range(l)) for _ in range(NL)]
                text = "".join(rng.choice(alpha) for _ in range(150))
                # plant both factors with up to e substitutions
                for p in pats:
                    a = rng.randint(0, len(text) - l)
                    occ = list(p)
                    for q in rng.sample(range(l), rng.randint(0, e)):
                        occ[q] = rng.choice(alpha)
                    text = text[:a] + "".join(occ) + text[a + l:]
                assert hclr_counts(pats, text, l, e) == [hamming_hits(p, text, e) for p in pats], (l, e, alpha)


def test_guarded_lane_hamming_full_blocks():
    """Every position a hit for both lanes (32 per block fill the 6-bit count
    fields), and a lane whose mismatches all sit in its top bit."""
    for l, NL in ((5, 2), (12, 2), (6, 3), (10, 3)):
        text = "A" * 100
        assert hclr_counts(["A" * l] * NL, text, l, 0) == [hamming_hits("A" * l, text, 0)] * NL
        p1 = "A" * (l - 1) + "C"
        pats = ["A" * l] * (NL - 1) + [p1]
        assert hclr_counts(pats, text, l, 1) == [hamming_hits(p, text, 1) for p in pats]


# ------------------------------------- structured lanes of different lengths

def struct_shape(l0, e0, b1, e1):
    """hswar_shape (dp_struct.cu) restated: box 0 and the two box-1 rows as
    lanes of l0, b1, b1 bits with a guard bit above each; score fields shifted
    down from each lane's top bit by the common s = min(l0, b1) - 1; None when
    the register or the field condition does not hold."""
    Ls, es = (l0, b1, b1), (e0, e1, e1)
    offs = (0, l0 + 1, l0 + b1 + 2)
    if offs[2] + b1 > 32:
        return None
    s = min(l0, b1) - 1
    if not 1 <= s <= 30:
        return None
    if any(e + 1 > (1 << s) or L - e - 1 >= (1 << s) for L, e in zip(Ls, es)):
        return None
    return offs, s


def struct_hits(words, text, offs, s, es, check=True, one_shift=False):
    """Per lane, per text position: the top-bit hit test of the packed step.
    one_shift: the score update of the kernels whose top lane ends below bit
    31 (ph - mh as a signed word, one arithmetic shift)."""
    Ls = [len(w) for w in words]
    HB = guards = K = SC0 = 0
    for L, e, o in zip(Ls, es, offs):
        hb = o + L - 1
        HB |= 1 << hb
        if o + L < 32:
            guards |= 1 << (o + L)
        K += ((1 << s) - (e + 1)) << (hb - s)
        SC0 += L << (hb - s)
    NG = ~guards & M32
    NGm1 = NG & ~HB & M32
    eq = {}
    for c in set(text):
        x = 0
        for w, o in zip(words, offs):
            for q, ch in enumerate(w):
                if ch == c:
                    x |= 1 << (o + q)
        eq[c] = (x | guards) & M32
    Pv, Mv, sc = NG, 0, (SC0 + K) & M32
    out = [[] for _ in words]
    for ch in text:
        Eq = eq[ch]
        Xv = Eq | Mv
        s1 = ((Eq & Pv) + Pv) & M32
        Xh = (s1 ^ Pv) | Eq
        Ph = (Mv | ~(Xh | Pv)) & M32
        Mhs = Pv & Xh & NGm1
        mh = Pv & Xh & HB
        ph = Ph & HB
        if one_shift:
            sc = (sc + (signed32((ph - mh) & M32) >> s)) & M32
        else:
            sc = (sc + (ph >> s) - (mh >> s)) & M32
        Ph2, Mh2 = (Ph << 1) & M32, (Mhs << 1) & M32
        Pv = (Mh2 | ~(Xv | Ph2)) & M32
        Mv = Ph2 & Xv & NG
        hits = ~sc & HB
        for i, (L, o) in enumerate(zip(Ls, offs)):
            out[i].append(bool((hits >> (o + L - 1)) & 1))
    return out


def test_structured_lanes_match_sellers():
    rng = random.Random(11)
    done = 0
    while done < 300:
        l0, b1 = rng.randint(2, 14), rng.randint(2, 14)
        e0, e1 = rng.randint(0, l0 - 1), rng.randint(0, b1 - 1)
        shape = struct_shape(l0, e0, b1, e1)
        if shape is None:
            continue
        offs, s = shape
        alpha = rng.choice(["ACGT", "ACDEFGHIKLMNPQRSTVWY"])
        words = ["".join(rng.choice(alpha) for _ in range(L)) for L in (l0, b1, b1)]
        text = "".join(rng.choice(alpha) for _ in range(80))
        got = struct_hits(words, text, offs, s, (e0, e1, e1))
        for w, e, g in zip(words, (e0, e1, e1), got):
            assert g == sellers_hits(w, text, e), (l0, e0, b1, e1)
        done += 1


def test_structured_one_shift_update_matches_sellers():
    """The one-gap and any-gap block kernels take the one-shift score update
    when the top lane ends below bit 31 (sd in hswar_shape / the any-gap
    shape): same hits as the two shifts."""
    rng = random.Random(23)
    done = 0
    while done < 300:
        l0, b1 = rng.randint(2, 14), rng.randint(2, 14)
        e0, e1 = rng.randint(0, l0 - 1), rng.randint(0, b1 - 1)
        shape = struct_shape(l0, e0, b1, e1)
        if shape is None:
            continue
        offs, s = shape
        if offs[2] + b1 - 1 > 30:                   # top lane at bit 31: two shifts
            continue
        alpha = rng.choice(["ACGT", "ACDEFGHIKLMNPQRSTVWY"])
        words = ["".join(rng.choice(alpha) for _ in range(L)) for L in (l0, b1, b1)]
        text = "".join(rng.choice(alpha) for _ in range(80))
        got = struct_hits(words, text, offs, s, (e0, e1, e1), one_shift=True)
        for w, e, g in zip(words, (e0, e1, e1), got):
            assert g == sellers_hits(w, text, e), (l0, e0, b1, e1)
        done += 1


def test_structured_field_condition_is_needed():
    """l0 = 3 gives s = 2: a 12-symbol row with 1 error has l - e - 1 = 10 >= 2^s,
    so score + 2^s - (e+1) passes 2^(s+1) while the score climbs from 0 and the
    top-bit test reads false hits (scores 6-9)."""
    assert struct_shape(3, 1, 12, 1) is None
    words, es = ["AAA", "A" * 12, "A" * 12], (1, 1, 1)
    offs, s = (0, 4, 17), 2
    text = "A" * 12 + "C" * 20
    got = struct_hits(words, text, offs, s, es)
    assert any(g != sellers_hits(w, text, e) for w, e, g in zip(words, es, got))


# ---------------------- one-gap structured Hamming: guarded lanes, bit clears

def brev32(x):
    return int(f"{x & M32:032b}"[::-1], 2)


def struct_hd_guarded_block(words, e, text, k0, codes, nbits):
    """k_dp_struct1_hd's guarded-lane form (GE = e) restated for the 32
    positions k0 .. k0+31 of text: box 0 (l0 symbols) and the two box-1 rows
    (b1 symbols each) as lanes at o0 = 32 - (l0 + 2 b1 + 3), o1, o2 with a
    guard bit above each (the top one at bit 31); the text window's newest
    l_j symbols copied into lane j; e clears of each lane's lowest set bit,
    t = x - L, and lane j's mask bit = bit g_j of t, shifted in by a funnel
    shift per position; after the block the masks are complemented and
    bit-reversed (bit r = a hit ending at position k0 + r)."""
    l0, b1 = len(words[0]), len(words[1])
    o0 = 32 - (l0 + 2 * b1 + 3)
    offs = (o0, o0 + l0 + 1, o0 + l0 + b1 + 2)
    lens = (l0, b1, b1)
    gs = tuple(o + l for o, l in zip(offs, lens))
    assert gs[2] == 31
    G = sum(1 << g for g in gs)
    L = sum(1 << o for o in offs)
    fp = [0] * nbits
    for w, o, ln in zip(words, offs, lens):
        for q, ch in enumerate(w):
            for b in range(nbits):
                if (codes[ch] >> b) & 1:
                    fp[b] |= 1 << (o + q)
    fp[0] |= G
    m = [0, 0, 0]
    for r in range(32):
        k = k0 + r
        x = 0
        for b in range(nbits):
            W = 0                                          # newest symbol at bit 31
            for d in range(32):
                if k - d >= 0 and (codes[text[k - d]] >> b) & 1:
                    W |= 1 << (31 - d)
            Y = 0
            for o, ln in zip(offs, lens):
                Y |= (W >> (32 - ln)) << o
            x |= fp[b] ^ Y
        for _ in range(e):
            x = ((x & ((x - L) & M32)) | G) & M32
        t = (x - L) & M32
        for j, g in enumerate(gs):
            m[j] = ((m[j] << 1) | (((t * (1 << (31 - g))) & M32) >> 31)) & M32
    return [brev32(~mj & M32) for mj in m]


@pytest.mark.parametrize("seed", range(12))
def test_struct_hd_guarded_lanes_match(seed):
    rng = random.Random(800 + seed)
    while True:
        l0, b1 = rng.randint(2, 12), rng.randint(2, 12)
        if l0 + 2 * b1 + 3 <= 32:
            break
    e = rng.randint(0, min(3, min(l0, b1) - 1))
    alpha = rng.choice(["ACGT", "ACDEFGHIKLMNPQRSTVWY"])
    codes = {c: i for i, c in enumerate(sorted(set(alpha)))}
    nbits = max(1, (len(codes) - 1).bit_length())
    words = ["".join(rng.choice(alpha) for _ in range(n)) for n in (l0, b1, b1)]
    text = "".join(rng.choice(alpha) for _ in range(96))
    for w in words:                                    # plant near-occurrences
        a = rng.randint(0, len(text) - len(w))
        occ = list(w)
        for q in rng.sample(range(len(w)), rng.randint(0, e)):
            occ[q] = rng.choice(alpha)
        text = text[:a] + "".join(occ) + text[a + len(w):]
    for k0 in (32, 64):
        got = struct_hd_guarded_block(words, e, text, k0, codes, nbits)
        for j, w in enumerate(words):
            ln = len(w)
            want = 0
            for r in range(32):
                k = k0 + r
                if sum(a != b for a, b in zip(w, text[k - ln + 1:k + 1])) <= e:
                    want |= 1 << r
            assert got[j] == want, (seed, j, l0, b1, e)
