"""The autotuner's key and cache file, on the CPU: entries read from the file
MOTEX_TUNE_CACHE names are keyed by (bit planes B, factor length l, errors e,
distance d), and a line that does not parse or names a launch shape the DP
kernels do not implement is skipped instead of reaching a launch (a zero
factors-per-register count would divide by zero when the grid is sized).
Lines carry an optional eighth field, the Hamming form (1: guarded lanes with
lowest-bit clears, for e <= 3 and 5 <= l <= 12)."""
import json
import os
import subprocess
import sys

from conftest import ROOT

CACHE_LINES = [
    "2 15 3 1 8 2 8",      # DNA edit distance, k 15: packed 2 lanes, valid
    "5 10 2 1 4 3 4",      # protein edit distance, k 10: 3 lanes, valid
    "5 10 2 0 8 3 4",      # protein Hamming, k 10: packed 3 lanes, unroll 4, valid
    "2 20 3 0 8 1 32",     # DNA Hamming, k 20: 1 lane, full unroll, valid
    "2 12 2 0 8 0 4",      # NL = 0: rejected
    "2 13 2 0 6 1 4",      # W = 6: rejected
    "2 14 2 0 8 1 16",     # UR = 16: rejected
    "5 11 2 0 8 3 4",      # NL = 3 is not the packed count (2) for l = 11: rejected
    "5 12 2 0 8 2 8",      # packed Hamming with unroll 8: rejected
    "2 9 1 1 8 2 32",      # packed edit distance with full unroll: rejected
    "2 40 3 0 8 1 4",      # l > 32 is never tuned: rejected
    "2 8 8 1 8 3 4",       # e >= l: rejected
    "7 8 1 1 8 1 4",       # 7 bit planes: rejected
    "2 16 2 1 8 1",        # six fields: rejected
    "2 17 2 1 8 1 4 9",    # Hamming form 9: rejected
    "2 17 2 1 8 1 4 1 7",  # nine fields: rejected
    "2 9 2 0 8 2 4 1",     # DNA Hamming, k 9, e 2: guarded lanes (form 1), valid
    "5 10 1 0 4 2 4 1",    # protein Hamming, k 10, e 1: guarded lanes, valid
    "2 13 1 0 8 2 4 1",    # guarded lanes need l <= 12: rejected
    "2 10 4 0 8 2 4 1",    # guarded lanes need e <= 3: rejected
    "2 11 2 0 8 2 8 1",    # guarded lanes with unroll 8: rejected
    "2 11 2 1 8 2 4 1",    # guarded lanes for edit distance: rejected
    "2 11 3 0 8 3 4 1",    # three guarded lanes need l <= 10: rejected
    "2 8 2 0 8 3 4 1",     # DNA Hamming, k 8, e 2: three guarded lanes, valid
    "2 5 1 0 8 3 4 1",     # three guarded lanes need l >= 6: rejected
    "2 11 1 0 8 2 4 2",    # form 2: rejected
    "garbage line",
    "2 18 2 1 4 1 8",      # valid, after the bad lines
    "2 18 2 1 8 1 4",      # a later valid line for the same key wins
]

QUERIES = [(2, 15, 3, 1), (5, 10, 2, 1), (5, 10, 2, 0), (2, 20, 3, 0), (2, 12, 2, 0), (2, 13, 2, 0),
           (2, 14, 2, 0), (5, 11, 2, 0), (5, 12, 2, 0), (2, 9, 1, 1), (2, 40, 3, 0), (2, 8, 8, 1),
           (7, 8, 1, 1), (2, 16, 2, 1), (2, 17, 2, 1), (2, 18, 2, 1), (2, 15, 3, 0), (3, 15, 3, 1),
           (2, 9, 2, 0), (5, 10, 1, 0), (2, 13, 1, 0), (2, 10, 4, 0), (2, 11, 2, 0), (2, 11, 2, 1),
           (2, 11, 3, 0), (2, 11, 1, 0), (2, 8, 2, 0), (2, 5, 1, 0)]

EXPECTED = {(2, 15, 3, 1): [8, 2, 8], (5, 10, 2, 1): [4, 3, 4], (5, 10, 2, 0): [8, 3, 4],
            (2, 20, 3, 0): [8, 1, 32], (2, 18, 2, 1): [8, 1, 4],
            # a negative NL reports the guarded-lane form
            (2, 9, 2, 0): [8, -2, 4], (5, 10, 1, 0): [4, -2, 4], (2, 8, 2, 0): [8, -3, 4]}


def test_tune_cache_keys_and_validation(native_built, tmp_path):
    cache = tmp_path / "tune.txt"
    cache.write_text("\n".join(CACHE_LINES) + "\n")
    # a fresh process: the cache file is read once per process, at the first lookup
    code = ("import json, sys; sys.path.insert(0, %r); from motex_gb300 import native; "
            "print(json.dumps([native.tune_lookup(*q) for q in %r]))" % (ROOT, QUERIES))
    env = dict(os.environ, MOTEX_TUNE_CACHE=str(cache))
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)
    assert p.returncode == 0, p.stderr
    got = dict(zip(QUERIES, json.loads(p.stdout.strip().splitlines()[-1])))
    for q in QUERIES:
        assert got[q] == EXPECTED.get(q), q


def test_tune_lookup_without_cache(native_built):
    env = {k: v for k, v in os.environ.items() if k != "MOTEX_TUNE_CACHE"}
    code = ("import sys; sys.path.insert(0, %r); from motex_gb300 import native; "
            "print(native.tune_lookup(2, 15, 3, 1))" % ROOT)
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip().splitlines()[-1] == "None"
