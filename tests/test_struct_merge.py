"""The one-gap structured kernels merge box-0 and box-1 hits in two forms
(motex_gb300/csrc/dp_struct.cu):

* per position (k_dp_struct1): each lane shifts its box-0 hit into a 32-bit
  history word at every text position; when some lane's box-1 row hits, the
  lanes exchange the row hits by ballots and add
  popc(history & gap window) to every pattern gap choice k whose row hit;
* per block (k_dp_struct1_hd, k_dp_struct1_swar_blk): a block of 32
  positions first yields per-lane 32-bit hit masks, box-0 masks join a
  64-bit history word, and one pass visits only the positions where some
  lane's box-1 row hits (OR over the warp) or a sequence ends, reading the
  gap window out of the 64-bit word.

Both are restated here over random hit masks (rows r0 = lane's first row,
r1 = its second, valid-position masks, sequence ends, gap choices that fit)
and must give the same counts, flushed per sequence, for every lane and gap
choice."""
import random

import pytest

M32 = 0xFFFFFFFF
M64 = (1 << 64) - 1


def popc(x):
    return bin(x).count("1")


def per_position(nblk, m0, ma, mb, vm, em, G, gmin, gmax, b1, kvalid, begin, has_r1):
    lo, hi = gmin + b1, gmax + b1
    win = (((2 << hi) - 1) if hi < 31 else M32) & ~((1 << lo) - 1)
    hist = [0] * 32
    cnt = [[0] * G for _ in range(32)]
    flushed = [[0] * G for _ in range(32)]
    for kb in range(nblk):
        counting = kb >= begin
        for r in range(32):
            for L in range(32):
                h0 = (m0[kb][L] >> r) & 1 and (vm[kb] >> r) & 1
                hist[L] = ((hist[L] << 1) | h0) & M32
            Ha = sum(((ma[kb][L] >> r) & 1) << L for L in range(32))
            Hb = sum((((mb[kb][L] >> r) & 1) if has_r1[L] else 0) << L for L in range(32))
            if counting and (Ha | Hb):
                H = (Hb << 32) | Ha
                for L in range(32):
                    g = (H >> L) & ((1 << G) - 1) & kvalid[L]
                    if g:
                        c = popc(hist[L] & win)
                        for k in range(G):
                            if (g >> k) & 1:
                                cnt[L][k] += c
            if (em[kb] >> r) & 1:
                if counting:
                    for L in range(32):
                        for k in range(G):
                            flushed[L][k] += cnt[L][k]
                            cnt[L][k] = 0
                hist = [0] * 32
    return cnt, flushed


def per_block(nblk, m0, ma, mb, vm, em, G, gmin, gmax, b1, kvalid, begin, has_r1):
    lo, hi = gmin + b1, gmax + b1
    wmask = (1 << (hi - lo + 1)) - 1
    X = [0] * 32
    cnt = [[0] * G for _ in range(32)]
    flushed = [[0] * G for _ in range(32)]
    for kb in range(nblk):
        counting = kb >= begin
        rb = [mb[kb][L] if has_r1[L] else 0 for L in range(32)]
        for L in range(32):
            X[L] = (((m0[kb][L] & vm[kb]) << 32) | (X[L] >> 32)) & M64
        R = 0
        if counting:
            for L in range(32):
                R |= ma[kb][L] | rb[L]
        E = em[kb]
        while R | E:
            v = R | E
            r = (v & -v).bit_length() - 1
            bit = 1 << r
            if R & bit:
                Ha = sum(((ma[kb][L] >> r) & 1) << L for L in range(32))
                Hb = sum(((rb[L] >> r) & 1) << L for L in range(32))
                H = (Hb << 32) | Ha
                for L in range(32):
                    g = (H >> L) & ((1 << G) - 1) & kvalid[L]
                    if g:
                        c = popc((X[L] >> (32 + r - hi)) & M32 & wmask)
                        for k in range(G):
                            if (g >> k) & 1:
                                cnt[L][k] += c
            if E & bit:
                if counting:
                    for L in range(32):
                        for k in range(G):
                            flushed[L][k] += cnt[L][k]
                            cnt[L][k] = 0
                for L in range(32):
                    X[L] &= ~((2 << (32 + r)) - 1) & M64     # box-0 ends of the finished sequence
            R &= ~bit
            E &= ~bit
    return cnt, flushed


@pytest.mark.parametrize("seed", range(6))
def test_block_merge_equals_per_position(seed):
    rng = random.Random(1000 + seed)
    for _ in range(50):
        G = rng.randint(1, 12)
        gmin = rng.randint(0, 8)
        gmax = gmin + G - 1
        b1 = rng.randint(1, 31 - gmax)                 # gap max + box length <= 31
        nblk = rng.randint(1, 6)
        begin = rng.randint(0, 1)
        dens = rng.choice([0.02, 0.1, 0.3])

        def masks():
            return [[sum((rng.random() < dens) << i for i in range(32)) for _ in range(32)] for _ in range(nblk)]

        m0, ma, mb = masks(), masks(), masks()
        vm = [rng.getrandbits(32) | rng.choice([0, M32]) for _ in range(nblk)]
        em = [sum((rng.random() < 0.03) << i for i in range(32)) for _ in range(nblk)]
        kvalid = [rng.getrandbits(G) for _ in range(32)]
        has_r1 = [L + 1 < G for L in range(32)]
        args = (nblk, m0, ma, mb, vm, em, G, gmin, gmax, b1, kvalid, begin, has_r1)
        assert per_position(*args) == per_block(*args), (G, gmin, gmax, b1)
