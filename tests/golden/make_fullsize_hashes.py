"""Pin the full-size workloads to the reference itself.

For each workload below, the seeded input is generated (the same
generators the benchmark and the GPU tests use), the reference MoTeX built by
oracle/build_ref.sh (motexOMP, all host threads) is run on it, and the
SHA-256 and line count of its output file -- without the two volatile header
lines -- are stored in tests/golden/fullsize.json.  The outputs are too large
to commit (dna_ed prints 441,205 motifs); tests/test_gpu_fullsize_ref.py
regenerates each input, runs motexGPU with the same switches and compares the
hash.  Each reference run takes from minutes to about an hour on 8 cores;
entries are written as they finish, and existing ones are kept unless named
with --redo.

usage: python tests/golden/make_fullsize_hashes.py [--only NAME ...] [--redo]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from motex_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "fullsize.json")
REF = os.path.join(ROOT, "oracle", "_ref", "motexOMP")

def _q(w, q):
    """The workload with quorum q percent instead of its own."""
    w.q = q
    return w


# name -> (workload factory, description)
CASES = {
    "dna_ed": (lambda: W.dna_ed(), "dna_ed: DNA 1200 x U[800,1200], -d 1 -k 15 -e 3 -q 10"),
    "prot_uneven_d0": (lambda: W.prot_uneven(d=0), "prot_uneven: PROT 2000 x logU[50,2000], -d 0 -k 10 -e 2 -q 15"),
    "prot_uneven_d1": (lambda: W.prot_uneven(d=1), "prot_uneven: PROT 2000 x logU[50,2000], -d 1 -k 10 -e 2 -q 15"),
    "dna_long_tenth": (lambda: W.dna_long(scale=0.1),
                       "dna_long at 1/10 length: DNA 8 x 100 knt with tandem repeats, -d 0 -k 20 -e 3 -q 50"),
    "structured_d0": (lambda: W.structured(d=0), "structured motifs on dna_ed's input: -k 8 -e 1 -s (5-15, 10, 1), -d 0"),
    "structured_d1": (lambda: W.structured(d=1), "structured motifs on dna_ed's input: -k 8 -e 1 -s (5-15, 10, 1), -d 1"),
    "structured_d1_quarter": (lambda: W.structured(d=1, scale=0.25),
                              "structured motifs on dna_ed's input at 1/4 (300 sequences): -k 8 -e 1 -s (5-15, 10, 1), "
                              "-d 1"),
    "structured2_d0_quarter": (lambda: W.structured2(d=0, scale=0.25),
                               "two-gap structured motifs on dna_ed's input at 1/4 (300 sequences): -k 8 -e 1 "
                               "-s (16-17, 6, 1; 15-16, 7, 2), -d 0"),
    "structured2_d1_quarter": (lambda: W.structured2(d=1, scale=0.25),
                               "two-gap structured motifs on dna_ed's input at 1/4 (300 sequences): -k 8 -e 1 "
                               "-s (16-17, 6, 1; 15-16, 7, 2), -d 1"),
    "dna_long_quarter": (lambda: W.dna_long(scale=0.25),
                         "dna_long at 1/4 length: DNA 8 x 250 knt with tandem repeats, -d 0 -k 20 -e 3 -q 50"),
    "structured_d0_quarter_q1": (lambda: _q(W.structured(d=0, scale=0.25), 1),
                                 "structured motifs on dna_ed's input at 1/4 (300 sequences), quorum 1% so that "
                                 "motifs print: -k 8 -e 1 -q 1 -s (5-15, 10, 1), -d 0"),
    "structured_d1_quarter_q1": (lambda: _q(W.structured(d=1, scale=0.25), 1),
                                 "structured motifs on dna_ed's input at 1/4 (300 sequences), quorum 1% so that "
                                 "motifs print: -k 8 -e 1 -q 1 -s (5-15, 10, 1), -d 1"),
    "structured2_d0_quarter_q1": (lambda: _q(W.structured2(d=0, scale=0.25), 1),
                                  "two-gap structured motifs on dna_ed's input at 1/4 (300 sequences), quorum 1%: "
                                  "-k 8 -e 1 -q 1 -s (16-17, 6, 1; 15-16, 7, 2), -d 0"),
    "structured2_d1_quarter_q1": (lambda: _q(W.structured2(d=1, scale=0.25), 1),
                                  "two-gap structured motifs on dna_ed's input at 1/4 (300 sequences), quorum 1%: "
                                  "-k 8 -e 1 -q 1 -s (16-17, 6, 1; 15-16, 7, 2), -d 1"),
    "structured2_d0": (lambda: W.structured2(d=0),
                       "two-gap structured motifs on dna_ed's input: -k 8 -e 1 -s (16-17, 6, 1; 15-16, 7, 2), -d 0"),
    "structured2_d1": (lambda: W.structured2(d=1),
                       "two-gap structured motifs on dna_ed's input: -k 8 -e 1 -s (16-17, 6, 1; 15-16, 7, 2), -d 1"),
}


def strip_volatile(text: str) -> str:
    return "".join(l for l in text.splitlines(True)
                   if not l.startswith(("# Rundate:", "# Run on ", "User time:")))


def input_sha256(w) -> str:
    """SHA-256 of a workload's input (sequences, one per line, and the boxes)."""
    h = hashlib.sha256()
    for seq in w.seqs:
        h.update(seq.encode())
        h.update(b"\n")
    if w.boxes:
        h.update(repr(tuple(tuple(g) for g in w.boxes)).encode())
    return h.hexdigest()


def run_case(name):
    w = CASES[name][0]()
    with tempfile.TemporaryDirectory() as tmp:
        W.write_fasta(os.path.join(tmp, "in.fa"), w.seqs, width=60)
        boxes = None
        if w.boxes:
            boxes = "in.boxes"
            W.write_boxes(os.path.join(tmp, boxes), w.boxes)
        args = w.cli("in.fa", "out.motex", boxes)
        t0 = time.time()
        subprocess.run([REF] + args + ["-t", str(os.cpu_count())], cwd=tmp, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        secs = time.time() - t0
        with open(os.path.join(tmp, "out.motex")) as f:
            text = strip_volatile(f.read())
    return {"args": args, "description": CASES[name][1], "input_sha256": input_sha256(w),
            "sha256": hashlib.sha256(text.encode()).hexdigest(),
            "lines": text.count("\n"), "reference": "motexOMP", "threads": os.cpu_count(),
            "reference_seconds": round(secs, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--redo", action="store_true")
    a = ap.parse_args()
    if not os.path.exists(REF):
        sys.exit("make_fullsize_hashes: oracle/_ref/motexOMP missing (run oracle/build_ref.sh on x86-64)")
    table = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for name in a.only or list(CASES):
        if name in table and not a.redo:
            continue
        entry = run_case(name)
        # re-read before writing: several runs may fill the table side by side
        table = json.load(open(OUT)) if os.path.exists(OUT) else {}
        table[name] = entry
        with open(OUT + ".tmp", "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(OUT + ".tmp", OUT)
        print(name, table[name]["lines"], table[name]["reference_seconds"], "s", flush=True)


if __name__ == "__main__":
    main()
