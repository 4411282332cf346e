"""The oracle (CPU restatement) against the reference's own outputs.

* golden fixtures: outputs of the reference MoTeX itself (its sources
  compiled with g++, linked to the shipped libflasm.so), regenerated by
  tests/golden/make_golden.py;
* the restated flasm against the shipped libflasm.so (x86-64 only);
* the edit-distance / Hamming cores against brute force on small cases.
"""
import ctypes as C
import os
import platform
import random
import subprocess

import pytest

from conftest import ORACLE_DIR, PORT_LIB, ROOT, golden_cases, mode_cases
from helpers import (expected_smile, load_case, load_mode_case, read_smile, run_cli, run_outputs,
                     same_but_pvalues)


@pytest.mark.parametrize("name", golden_cases())
def test_port_matches_reference_golden(oracle_port, name):
    d, args, expected = load_case(name)
    rc, out, err = run_cli(oracle_port, d, args, extra=["-t", "4"])
    assert rc == 0, err
    assert out == expected


@pytest.mark.parametrize("name", [n for n in golden_cases() if expected_smile(n) is not None])
def test_port_smile_matches_reference_golden(oracle_port, name):
    """-S: the SMILE-like file (functions.cc:1262-1591) of the reference itself."""
    d, args, expected = load_case(name)
    rc, out, smile, err = read_smile(d, oracle_port, args, extra=["-t", "4"])
    assert rc == 0, err
    assert out == expected
    assert smile == expected_smile(name)


@pytest.mark.parametrize("name", mode_cases())
def test_port_modes_match_reference_golden(oracle_port, name):
    """-b/-u/-S/-U and -I: every output file of the reference itself.  Built
    on x86-64, as the fixtures were, the port's long double p-values match
    to the last printed digit."""
    d, args, expected = load_mode_case(name)
    rc, got, err = run_outputs(oracle_port, d, args, list(expected), extra=["-t", "4"])
    assert rc == 0, err
    for o, text in expected.items():
        if platform.machine() in ("x86_64", "AMD64"):
            assert got[o] == text, o
        else:
            assert same_but_pvalues(got[o], text) is None, o


def test_golden_set_is_complete():
    names = set(golden_cases())
    for needed in ("dna_hd_64x500", "dna_ed_24seq", "prot_hd_20seq", "prot_ed_20seq", "struct_planted_hd",
                   "struct_planted_ed", "quorum_boundary_q29", "dna_with_N_ed", "short_seqs_ed",
                   "long_factor_k70_ed", "q0_n0_all_words", "caps_Q60_n2_N40", "struct3_box40_ed",
                   "struct3_box40_hd", "struct_l40_ed", "struct9_gaps_ed", "struct2_64structs_ed",
                   "dna_hd_k8_e3", "dna_hd_k5_e0", "short_factor_k5_e3_dna_hd"):
        assert needed in names
    assert {"bg_dna_hd_smile", "bg_prot_ed", "bg_struct_hd_smile", "bg_struct2_ed", "fore_dna_hd",
            "fore_prot_ed"} <= set(mode_cases())
    smile = {n for n in names if expected_smile(n) is not None}
    assert {"prot_hd_20seq", "usr_hd", "struct_planted_hd", "struct2_planted_ed"} <= smile


def _difftest_binary():
    b = os.path.join(ORACLE_DIR, "_ref", "flasm_difftest")
    if not os.path.exists(b):
        # exit status 2: the reference sources are not on this host
        r = subprocess.run([os.path.join(ORACLE_DIR, "build_ref.sh")], capture_output=True, text=True)
        assert r.returncode in (0, 2), r.stdout + r.stderr
    return b


@pytest.mark.skipif(platform.machine() != "x86_64", reason="the shipped libflasm.so is x86-64 only")
def test_flasm_port_vs_shipped_library():
    b = _difftest_binary()
    if not os.path.exists(b):
        pytest.skip("reference tree not available on this host")
    for seed, mode in ((11, []), (12, ["edge"])):
        p = subprocess.run([b, "1500", str(seed)] + mode, capture_output=True, text=True, timeout=300)
        assert p.returncode == 0 and p.stdout.startswith("OK"), p.stdout + p.stderr


# ---------------------------------------------------------------- brute force

def _ed_end(w, t, i):
    """min_s EditDistance(w, t[s..i]) (empty t-factor allowed)."""
    l = len(w)
    col = list(range(l + 1))
    best = col[l]
    for ch in t[: i + 1]:
        nxt = [0] * (l + 1)
        for p in range(1, l + 1):
            nxt[p] = min(col[p - 1] + (w[p - 1] != ch), col[p] + 1, nxt[p - 1] + 1)
        col = nxt
    return col[l]


def brute_pair(d, l, e, p, t):
    """u/v contributions of one (pattern p, text t) pair, flasm contract."""
    m = len(p)
    u, v = [0] * m, [0] * m
    for j in range(l - 1, m):
        w = p[j - l + 1: j + 1]
        hits = 0
        if d == 0:
            for i in range(l - 1, len(t)):
                if sum(a != b for a, b in zip(w, t[i - l + 1: i + 1])) <= e:
                    hits += 1
        else:
            for i in range(len(t)):
                if _ed_end(w, t, i) <= e:
                    hits += 1
        u[j] += hits > 0
        v[j] += hits
    return u, v


def port_pair(d, l, e, p, t):
    lib = C.CDLL(PORT_LIB)
    m = len(p)
    U = (C.c_uint32 * m)()
    V = (C.c_uint32 * m)()
    lib.oracle_extract_pair(d, l, e, p.encode(), m, t.encode(), len(t), U, V)
    return list(U), list(V)


@pytest.mark.parametrize("d", [0, 1])
def test_port_pair_vs_bruteforce(oracle_port, d):
    rng = random.Random(100 + d)
    for _ in range(60):
        sigma = rng.choice([2, 4, 20])
        alpha = "ACGTNRDQEHIKLMFPSWYV"[:sigma]
        l = rng.randint(1, 7)
        e = rng.randint(0, l - 1)
        p = "".join(rng.choice(alpha) for _ in range(rng.randint(l, 18)))
        t = "".join(rng.choice(alpha) for _ in range(rng.randint(1, 22)))
        assert port_pair(d, l, e, p, t) == brute_pair(d, l, e, p, t), (d, l, e, p, t)
