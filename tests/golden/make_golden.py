"""Regenerate the golden fixtures under tests/golden/cases/.

Each case is a seeded input (FASTA, optional boxes file) plus the CLI
switches; its expected output is produced by the reference MoTeX itself:
the unmodified reference sources compiled by oracle/build_ref.sh and linked
with the libflasm.so shipped in the reference (x86-64 only).  The restated
oracle (oracle/_build/motex_port) is run on every case as well and must give
the identical file; a mismatch aborts the script.

Cases listed in SMILE_CASES also run with ``-S out.smile`` and store the
SMILE-like file as expected.smile.  The background cases (-b, with -u and
optionally -S/-U) and the word-search cases (-I) of mode_cases() carry extra
inputs -- a background file made by the reference from other seeded
sequences, or the unmatched-motif file of such a run -- kept byte for byte
(the reference finds N and Q in a background header by line number), and
list their output files in case.json ("outputs"; the expected copy of X is
expected.X, with out.motex -> expected.motex and out.smile -> expected.smile).

The two non-deterministic header lines (``# Rundate:`` and ``# Run on ...``)
and the SMILE file's ``User time:`` line are removed from stored outputs.  Cases run with relative paths (in.fa,
in.boxes, out.motex) from the case directory, so the header's file lines are
reproducible.

usage: python tests/golden/make_golden.py [--only NAME ...]   (needs the reference
tree and an x86-64 host; run oracle/build_ref.sh and make -C oracle first;
--only rebuilds the named cases and keeps the others)
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from motex_gb300 import workloads as W  # noqa: E402

CASES_DIR = os.path.join(HERE, "cases")
REF = os.path.join(ROOT, "oracle", "_ref")
PORT = os.path.join(ROOT, "oracle", "_build", "motex_port")


SMILE_CASES = {"dna_hd_64x500", "prot_hd_20seq", "prot_ed_20seq", "usr_hd", "dna_with_N_ed",
               "quorum_boundary_q29", "short_seqs_ed", "struct_planted_hd", "struct_planted_ed",
               "struct2_planted_ed", "struct_long_gap_hd"}


def strip_volatile(text: str) -> str:
    return "".join(l for l in text.splitlines(True)
                   if not l.startswith(("# Rundate:", "# Run on ", "User time:")))


def expected_name(output):
    return "expected." + (output[4:] if output.startswith("out.") else output)


def run_outputs(binary, args, cwd, outputs):
    """Returns (rc, {output name: stripped text or None})."""
    p = subprocess.run([binary] + args, cwd=cwd, capture_output=True, text=True)
    got = {}
    for name in outputs:
        path = os.path.join(cwd, name)
        got[name] = None
        if os.path.exists(path):
            with open(path) as f:
                got[name] = strip_volatile(f.read())
            os.remove(path)
    return p.returncode, got


def run_cli(binary, args, cwd):
    """Returns (rc, main output, SMILE output or None)."""
    p = subprocess.run([binary] + args, cwd=cwd, capture_output=True, text=True)
    outs = []
    for name in ("out.motex", "out.smile"):
        path = os.path.join(cwd, name)
        outs.append(None)
        if os.path.exists(path):
            with open(path) as f:
                outs[-1] = strip_volatile(f.read())
            os.remove(path)
    return p.returncode, outs[0], outs[1]


# --------------------------------------------------------------- case inputs

def planted_structured(seed, nseq, length, d):
    """Random DNA with a planted 2-box structured motif (8-mer, gap 5-15,
    10-mer; <= 1 substitution per box) in half of the sequences."""
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, W.DNA, length) for _ in range(nseq)]
    b0, b1 = W._rand_seq(rng, W.DNA, 8), W._rand_seq(rng, W.DNA, 10)

    def copy():
        gap = W._rand_seq(rng, W.DNA, int(rng.integers(5, 16)))
        return (W._substitute(rng, b0, W.DNA, int(rng.integers(2))) + gap +
                W._substitute(rng, b1, W.DNA, int(rng.integers(2))))
    W._plant(rng, seqs, copy, 0.5)
    return W.Workload("planted_structured", "DNA", seqs, d=d, k=8, e=1, q=30,
                      boxes=((5, 15, 10, 1),))


def planted_structured2(seed, nseq, length, d):
    """A planted 3-box structured motif (6-mer, gap 3-5, 7-mer, gap 2-3,
    6-mer; <= 1 substitution per box) in 60% of the sequences: two gaps."""
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, W.DNA, length) for _ in range(nseq)]
    b0, b1, b2 = (W._rand_seq(rng, W.DNA, n) for n in (6, 7, 6))

    def copy():
        g1 = W._rand_seq(rng, W.DNA, int(rng.integers(3, 6)))
        g2 = W._rand_seq(rng, W.DNA, int(rng.integers(2, 4)))
        return (W._substitute(rng, b0, W.DNA, int(rng.integers(2))) + g1 +
                W._substitute(rng, b1, W.DNA, int(rng.integers(2))) + g2 +
                W._substitute(rng, b2, W.DNA, int(rng.integers(2))))
    W._plant(rng, seqs, copy, 0.6)
    return W.Workload("planted_structured2", "DNA", seqs, d=d, k=6, e=1, q=25,
                      boxes=((3, 5, 7, 1), (2, 3, 6, 1)))


def planted_long_gap(seed, nseq, length, d):
    """One gap of 20-30 symbols between a 7-mer and an 8-mer: a gap longer
    than the box-0 hit history of the one-gap kernel."""
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, W.DNA, length) for _ in range(nseq)]
    b0, b1 = W._rand_seq(rng, W.DNA, 7), W._rand_seq(rng, W.DNA, 8)

    def copy():
        gap = W._rand_seq(rng, W.DNA, int(rng.integers(20, 31)))
        return (W._substitute(rng, b0, W.DNA, int(rng.integers(2))) + gap +
                W._substitute(rng, b1, W.DNA, int(rng.integers(2))))
    W._plant(rng, seqs, copy, 0.5)
    return W.Workload("planted_long_gap", "DNA", seqs, d=d, k=7, e=1, q=30,
                      boxes=((20, 30, 8, 1),))


def planted_boxes(seed, nseq, length, d, k, e, boxes, q=30, frac=0.6):
    """Random DNA with a planted structured motif of the given boxes (a
    k-mer, then per gap a random gap of gmin..gmax symbols and a box of
    blen symbols; <= 1 substitution per box) in `frac` of the sequences."""
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, W.DNA, length) for _ in range(nseq)]
    parts = [W._rand_seq(rng, W.DNA, k)] + [W._rand_seq(rng, W.DNA, b[2]) for b in boxes]

    def copy():
        occ = W._substitute(rng, parts[0], W.DNA, int(rng.integers(2)))
        for (gmin, gmax, _, _), box in zip(boxes, parts[1:]):
            occ += W._rand_seq(rng, W.DNA, int(rng.integers(gmin, gmax + 1)))
            occ += W._substitute(rng, box, W.DNA, int(rng.integers(2)))
        return occ
    W._plant(rng, seqs, copy, frac)
    return W.Workload("planted_boxes", "DNA", seqs, d=d, k=k, e=e, q=q, boxes=tuple(boxes))


def quorum_boundary(seed):
    """100 sequences; one 10-mer planted exactly in 29 of them and run with
    q=29: (29/100)*100 evaluates below 29 in IEEE double, so the reference
    rejects it although 29% of the sequences hold it."""
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, W.DNA, 40) for _ in range(100)]
    motif = W._rand_seq(rng, W.DNA, 10)
    for i in rng.choice(100, size=29, replace=False):
        pos = int(rng.integers(0, 31))
        seqs[i] = seqs[i][:pos] + motif + seqs[i][pos + 10:]
    return W.Workload("quorum_boundary", "DNA", seqs, d=0, k=10, e=0, q=29)


def with_n(seed, d):
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, "ACGTN", int(rng.integers(60, 140)), [0.24, 0.24, 0.24, 0.24, 0.04])
            for _ in range(16)]
    return W.Workload("dna_with_N", "DNA", seqs, d=d, k=6, e=1, q=20)


def short_seqs(seed, d):
    rng = np.random.default_rng(seed)
    lens = [3, 80, 5, 120, 9, 60, 10, 11, 200, 7]
    seqs = [W._rand_seq(rng, W.DNA, n) for n in lens]
    return W.Workload("short_seqs", "DNA", seqs, d=d, k=10, e=2, q=10)


def usr(seed, d):
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, "0123456789", int(rng.integers(50, 150))) for _ in range(12)]
    return W.Workload("usr_digits", "USR", seqs, d=d, k=5, e=1, q=25)


def long_factor(seed, d, k, e, nseq=6, length=220):
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, W.DNA, length) for _ in range(nseq)]
    src = seqs[0][10:10 + k]
    for i in range(1, nseq, 2):
        c = W._edit(rng, src, W.DNA, int(rng.integers(e + 1))) if d else \
            W._substitute(rng, src, W.DNA, int(rng.integers(e + 1)))
        seqs[i] = seqs[i][:30] + c + seqs[i][30 + len(c):]
    return W.Workload(f"long_factor_k{k}", "DNA", seqs, d=d, k=k, e=e, q=30)


def raw_fasta_text(seed):
    """Multi-line records, lower case, an empty record and a header-only record."""
    rng = np.random.default_rng(seed)
    seqs = [W._rand_seq(rng, W.DNA, int(rng.integers(40, 90))) for _ in range(6)]
    txt = ""
    for i, s in enumerate(seqs):
        if i == 2:
            txt += ">empty record\n\n"
        if i == 4:
            txt += ">header only\n"
        body = s.lower() if i % 2 else s
        txt += f">s{i} description\n" + "\n".join(body[p:p + 25] for p in range(0, len(body), 25)) + "\n"
    return txt


def cases():
    """(name, workload, extra CLI tokens, raw FASTA text or None)"""
    out = []
    out.append(("dna_hd_64x500", W.dna_hd_small(seed=1), [], None))
    out.append(("dna_ed_24seq", W.dna_ed(seed=2, scale=0.02), [], None))
    out.append(("dna_hd_24seq", W.dna_ed(seed=2, scale=0.02, d=0), [], None))
    out.append(("prot_hd_20seq", W.prot_uneven(seed=3, scale=0.01, d=0), [], None))
    out.append(("prot_ed_20seq", W.prot_uneven(seed=3, scale=0.01, d=1), [], None))
    out.append(("dna_long_8x2000", W.dna_long(seed=4, scale=0.002), [], None))
    out.append(("struct_hd_dna_ed_12seq", W.structured(seed=2, scale=0.01, d=0), [], None))
    out.append(("struct_ed_dna_ed_12seq", W.structured(seed=2, scale=0.01, d=1), [], None))
    out.append(("struct_planted_hd", planted_structured(11, 16, 150, 0), [], None))
    out.append(("struct_planted_ed", planted_structured(11, 16, 150, 1), [], None))
    out.append(("struct2_planted_hd", planted_structured2(22, 14, 160, 0), [], None))
    out.append(("struct2_planted_ed", planted_structured2(22, 14, 160, 1), [], None))
    out.append(("struct_long_gap_hd", planted_long_gap(23, 12, 150, 0), [], None))
    out.append(("struct_long_gap_ed", planted_long_gap(23, 12, 150, 1), [], None))
    out.append(("quorum_boundary_q29", quorum_boundary(12), [], None))
    out.append(("dna_with_N_hd", with_n(13, 0), [], None))
    out.append(("dna_with_N_ed", with_n(13, 1), [], None))
    out.append(("short_seqs_hd", short_seqs(14, 0), [], None))
    out.append(("short_seqs_ed", short_seqs(14, 1), [], None))
    out.append(("usr_hd", usr(15, 0), [], None))
    out.append(("usr_ed", usr(15, 1), [], None))
    w = W.dna_ed(seed=16, scale=0.01, d=0)
    w.k, w.e, w.q = 6, 1, 0
    w.n = 0
    out.append(("q0_n0_all_words", w, [], None))
    w = W.prot_uneven(seed=17, scale=0.008, d=1)
    w.k, w.e, w.q, w.Q, w.n, w.N = 5, 1, 10, 60, 2, 40
    out.append(("caps_Q60_n2_N40", w, [], None))
    out.append(("long_factor_k40_hd", long_factor(18, 0, 40, 6), [], None))
    out.append(("long_factor_k40_ed", long_factor(18, 1, 40, 6), [], None))
    out.append(("long_factor_k70_hd", long_factor(19, 0, 70, 9), [], None))
    out.append(("long_factor_k70_ed", long_factor(19, 1, 70, 5, nseq=4, length=160), [], None))
    w = W.Workload("raw_fasta", "DNA", [], d=0, k=5, e=1, q=30)
    out.append(("raw_fasta_hd", w, [], raw_fasta_text(20)))
    w = W.dna_ed(seed=21, scale=0.005, d=0)
    w.k, w.e, w.q = 7, 1, 20
    out.append(("flag_L_ignored", w, ["-L", "1"], None))
    # 4-mers with 2-3 errors hit at nearly every position: a packed lane's hit
    # count for a 32-position block must not carry into its neighbour
    w = W.dna_ed(seed=24, scale=0.006, d=1)
    w.k, w.e, w.q = 4, 3, 30
    out.append(("short_factor_k4_e3_dna_ed", w, [], None))
    w = W.prot_uneven(seed=25, scale=0.004, d=1)
    w.k, w.e, w.q = 4, 2, 30
    out.append(("short_factor_k4_e2_prot_ed", w, [], None))
    # structured shapes beyond 32-symbol rows, 32 structures and 8 gaps
    box40 = ((2, 5, 40, 4), (1, 4, 6, 1), (3, 6, 7, 1))               # 3 gaps, 64 structures, a 40-symbol box
    out.append(("struct3_box40_hd", planted_boxes(26, 10, 260, 0, 8, 1, box40), [], None))
    out.append(("struct3_box40_ed", planted_boxes(26, 10, 260, 1, 8, 1, box40), [], None))
    out.append(("struct_l40_hd", planted_boxes(27, 10, 220, 0, 40, 4, ((3, 6, 10, 1),)), [], None))
    out.append(("struct_l40_ed", planted_boxes(27, 10, 220, 1, 40, 4, ((3, 6, 10, 1),)), [], None))
    gaps9 = tuple([(1, 1, 4, 0)] * 7 + [(1, 2, 4, 0), (2, 3, 5, 1)])  # 9 gaps, 4 structures
    out.append(("struct9_gaps_hd", planted_boxes(28, 10, 200, 0, 5, 0, gaps9), [], None))
    out.append(("struct9_gaps_ed", planted_boxes(28, 10, 200, 1, 5, 0, gaps9), [], None))
    many = ((0, 7, 6, 1), (0, 7, 6, 1))                                # 2 gaps, 64 structures
    out.append(("struct2_64structs_ed", planted_boxes(29, 10, 220, 1, 6, 1, many), [], None))
    # popc-free Hamming: three guarded lanes (k 8, e 3), two lanes at the
    # smallest k (5, e 0), and 5-mers with 3 mismatches, which hit at nearly
    # every position (full 6-bit count fields per 32-position block)
    w = W.dna_ed(seed=30, scale=0.01, d=0)
    w.k, w.e, w.q = 8, 3, 40
    out.append(("dna_hd_k8_e3", w, [], None))
    w = W.dna_ed(seed=31, scale=0.01, d=0)
    w.k, w.e, w.q = 5, 0, 30
    out.append(("dna_hd_k5_e0", w, [], None))
    w = W.dna_ed(seed=32, scale=0.006, d=0)
    w.k, w.e, w.q = 5, 3, 30
    out.append(("short_factor_k5_e3_dna_hd", w, [], None))
    return out


# ------------------------------------------------------- background and -I

def _mixed_background(rng_seed, fg_seqs, alphabet, n_new, length_range, keep):
    """Background sequences: `keep` of the foreground sequences (so some
    motifs match) and n_new fresh random ones."""
    rng = np.random.default_rng(rng_seed)
    new = [W._rand_seq(rng, alphabet, int(rng.integers(*length_range))) for _ in range(n_new)]
    return list(fg_seqs[:keep]) + new


def mode_cases():
    """(name, fg workload, bg sequences, background quorum, extra switches
    for the foreground run, kind) with kind "b" (background run) or "I"
    (search the unmatched motifs of that background run in the background
    sequences, every motif printed: -q 0 -n 0)."""
    out = []
    # sequence lengths stay clear of 440-500: in the reference's -I mode a
    # sequence copy of that size takes the memory of the closed FASTA stream
    # it still reads the motif file's header through (motex.cc:902)
    w = W.dna_ed(seed=2, scale=0.01, d=0)
    w.k, w.e, w.q = 10, 1, 25
    bgd = _mixed_background(51, w.seqs, W.DNA, 10, (600, 1000), 6)
    out.append(("bg_dna_hd_smile", w, bgd, 10, ["-S", "out.smile", "-U", "un.smile"], "b"))
    out.append(("fore_dna_hd", w, bgd, 10, [], "I"))
    w = W.prot_uneven(seed=3, scale=0.01, d=1)
    w.k, w.e, w.q = 6, 1, 10
    w.seqs = [q for q in w.seqs if not 440 <= len(q) <= 500]
    bgp = _mixed_background(52, w.seqs, W.AMINO20, 14, (80, 440), 10)
    out.append(("bg_prot_ed", w, bgp, 10, [], "b"))
    out.append(("fore_prot_ed", w, bgp, 10, [], "I"))
    ws = planted_structured(11, 16, 150, 0)
    out.append(("bg_struct_hd_smile", ws, _mixed_background(53, ws.seqs, W.DNA, 12, (100, 200), 9), 20,
                ["-S", "out.smile", "-U", "un.smile"], "b"))
    ws2 = planted_structured2(22, 14, 160, 1)
    out.append(("bg_struct2_ed", ws2, _mixed_background(54, ws2.seqs, W.DNA, 10, (120, 200), 8), 15, [], "b"))
    return out


def build_mode_case(name, w, bg_seqs, bg_q, extra, kind):
    d = os.path.join(CASES_DIR, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    boxes = "in.boxes" if w.boxes else None
    fg_args = w.cli("in.fa", "out.motex", boxes)
    bg_args = list(fg_args)
    bg_args[bg_args.index("-i") + 1] = "bg.fa"
    bg_args[bg_args.index("-o") + 1] = "bg.motex"
    bg_args[bg_args.index("-q") + 1] = str(bg_q)
    ref_bin = os.path.join(REF, "motexCPU")
    with tempfile.TemporaryDirectory() as tmp:
        W.write_fasta(os.path.join(tmp, "in.fa"), w.seqs, width=60)
        W.write_fasta(os.path.join(tmp, "bg.fa"), bg_seqs, width=60)
        if w.boxes:
            W.write_boxes(os.path.join(tmp, "in.boxes"), w.boxes)
        subprocess.run([ref_bin] + bg_args, cwd=tmp, check=True, capture_output=True)
        b_args = fg_args + ["-b", "bg.motex", "-u", "un.motex"]
        if kind == "b":
            args = b_args + extra
            outputs = ["out.motex", "un.motex"] + (["out.smile", "un.smile"] if "-U" in extra else [])
            keep = ["in.fa", "bg.motex"] + (["in.boxes"] if w.boxes else [])
        else:
            # the unmatched motifs of a background run, searched in the background sequences
            subprocess.run([ref_bin] + b_args, cwd=tmp, check=True, capture_output=True)
            os.replace(os.path.join(tmp, "un.motex"), os.path.join(tmp, "fg.in"))
            os.replace(os.path.join(tmp, "bg.fa"), os.path.join(tmp, "in.fa"))
            args = list(fg_args)
            args[args.index("-q") + 1] = "0"
            args += ["-n", "0", "-I", "fg.in"] + extra
            outputs = ["out.motex"]
            keep = ["in.fa", "fg.in"]
        for f in keep:
            shutil.copy(os.path.join(tmp, f), d)
        rc, ref_out = run_outputs(ref_bin, args, tmp, outputs)
        rc2, port_out = run_outputs(PORT, args + ["-t", str(os.cpu_count())], tmp, outputs)
    if rc != 0 or any(v is None for v in ref_out.values()):
        sys.exit(f"make_golden: reference failed on {name} (rc={rc})")
    if rc2 != rc or port_out != ref_out:
        sys.exit(f"make_golden: oracle/_build/motex_port disagrees with the reference on {name}")
    for o, text in ref_out.items():
        with open(os.path.join(d, expected_name(o)), "w") as f:
            f.write(text)
    with open(os.path.join(d, "case.json"), "w") as f:
        json.dump({"args": args, "reference": "motexCPU", "outputs": outputs}, f, indent=1)
    print(f"{name:28s} kind={kind} " + " ".join(f"{o}={t.count(chr(10))}" for o, t in ref_out.items()) + " ok")


def main():
    only = set(sys.argv[sys.argv.index("--only") + 1:]) if "--only" in sys.argv else None
    if not os.path.exists(os.path.join(REF, "motexCPU")):
        sys.exit("make_golden: oracle/_ref/motexCPU missing (run oracle/build_ref.sh on x86-64)")
    if not os.path.exists(PORT):
        sys.exit("make_golden: oracle/_build/motex_port missing (run make -C oracle)")
    os.makedirs(CASES_DIR, exist_ok=True)
    for name, w, extra, raw in cases():
        if only is not None and name not in only:
            continue
        d = os.path.join(CASES_DIR, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        if raw is not None:
            with open(os.path.join(d, "in.fa"), "w") as f:
                f.write(raw)
        else:
            W.write_fasta(os.path.join(d, "in.fa"), w.seqs, width=60)
        if w.boxes:
            W.write_boxes(os.path.join(d, "in.boxes"), w.boxes)
        args = w.cli("in.fa", "out.motex", "in.boxes" if w.boxes else None) + extra
        if name in SMILE_CASES:
            args += ["-S", "out.smile"]
        big = w.total_len ** 2 * (len(w.boxes) + 1) > 3e8
        ref_bin = os.path.join(REF, "motexOMP" if big else "motexCPU")
        ref_args = args + (["-t", str(os.cpu_count())] if big else [])
        with tempfile.TemporaryDirectory() as tmp:
            for f in os.listdir(d):
                shutil.copy(os.path.join(d, f), tmp)
            rc, ref_out, ref_smile = run_cli(ref_bin, ref_args, tmp)
            rc2, port_out, port_smile = run_cli(PORT, args + ["-t", str(os.cpu_count())], tmp)
        if rc != 0 or ref_out is None or (name in SMILE_CASES and ref_smile is None):
            sys.exit(f"make_golden: reference failed on {name} (rc={rc})")
        if rc2 != rc or port_out != ref_out or port_smile != ref_smile:
            sys.exit(f"make_golden: oracle/_build/motex_port disagrees with the reference on {name}")
        with open(os.path.join(d, "expected.motex"), "w") as f:
            f.write(ref_out)
        if ref_smile is not None:
            with open(os.path.join(d, "expected.smile"), "w") as f:
                f.write(ref_smile)
        with open(os.path.join(d, "case.json"), "w") as f:
            json.dump({"args": args, "reference": os.path.basename(ref_bin),
                       "motifs": ref_out.count("\n") - ref_out.count("#") - 3}, f, indent=1)
        print(f"{name:28s} seqs={len(w.seqs) if raw is None else 'raw':>5} "
              f"lines={ref_out.count(chr(10)):6d} ok")
    for case in mode_cases():
        if only is None or case[0] in only:
            build_mode_case(*case)


if __name__ == "__main__":
    main()
