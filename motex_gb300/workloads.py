"""Seeded synthetic inputs for the word-based motif-extraction workloads.

Each generator returns a list of sequences (``str``) and the CLI switches the
workload runs with.  No public dataset is named for this path; the shapes,
length distributions, compositions and planted motifs below stand in for
real inputs.  Every generator is a pure function of its seed (numpy PCG64).

Workloads (sizes as run by ``bench.py`` and the tests):

* ``dna_hd_small``   64 x 500 nt iid ACGT, one 12-mer planted with 0-2
  substitutions in 50% of sequences; ``-d 0 -k 12 -e 2 -q 50``.
* ``dna_ed``         1200 x U[800,1200] nt, GC 40%, three 15-mers planted with
  0-3 edits (sub/ins/del equiprobable) in 20/40/60% of sequences;
  ``-d 1 -k 15 -e 3 -q 10``.  ``dna_ed_k20``: the same with 20-mers and
  ``-k 20 -e 4`` (factors of one 32-bit word, past the packed lanes).
* ``prot_uneven``    2000 x logU[50,2000] aa over 20 amino acids with
  Dirichlet(5) frequencies, five 10-mers planted with 0-2 substitutions in
  U[15,50]% of sequences; ``-k 10 -e 2 -q 15`` with ``-d 0`` and ``-d 1``.
* ``dna_long``       8 x 1,000,000 nt uniform background plus tandem repeats
  (unit 2-6, 20-200 copies, 1% per-base mutation) over 5% of each sequence;
  ``-d 0 -k 20 -e 3 -q 50``.
* ``structured``     boxes ``1 / 5 15 10 1`` with ``-k 8 -e 1`` on dna_ed's
  input.
* ``structured2``    two gaps (``2 / 16 17 6 1 / 15 16 7 2``) with ``-k 8 -e 1``
  on dna_ed's input.
* ``serve_stream``   extraction requests with Poisson arrivals.

``scale`` shrinks a workload (fewer / shorter sequences) for parity tests
at sizes the CPU oracle finishes in seconds.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

DNA = "ACGT"
AMINO20 = "ARNDCQEGHILKMFPSTWYV"


@dataclass
class Workload:
    name: str
    alphabet: str            # "DNA" | "PROT" | "USR"
    seqs: list
    d: int
    k: int
    e: int
    q: int
    Q: int = 100
    n: int = 1
    N: int = 10000
    boxes: tuple = ()        # ((gmin, gmax, blen, berr), ...)
    extra: dict = field(default_factory=dict)

    def cli(self, fasta: str, out: str, boxes_file: str | None = None) -> list:
        a = ["-a", self.alphabet, "-i", fasta, "-o", out, "-d", str(self.d),
             "-k", str(self.k), "-e", str(self.e), "-q", str(self.q)]
        if self.Q != 100:
            a += ["-Q", str(self.Q)]
        if self.n != 1:
            a += ["-n", str(self.n)]
        if self.N != 10000:
            a += ["-N", str(self.N)]
        if self.boxes:
            a += ["-s", boxes_file]
        return a

    @property
    def total_len(self) -> int:
        return sum(len(s) for s in self.seqs)


def write_fasta(path: str, seqs, width: int = 0) -> None:
    with open(path, "w") as f:
        for i, s in enumerate(seqs):
            f.write(f">seq{i}\n")
            if width:
                for p in range(0, len(s), width):
                    f.write(s[p:p + width] + "\n")
            else:
                f.write(s + "\n")


def write_boxes(path: str, boxes) -> None:
    with open(path, "w") as f:
        f.write(f"{len(boxes)}\n")
        for g in boxes:
            f.write("\n".join(str(x) for x in g) + "\n")


def _rand_seq(rng, alphabet: str, n: int, p=None) -> str:
    idx = rng.choice(len(alphabet), size=n, p=p)
    return np.frombuffer(alphabet.encode(), dtype=np.uint8)[idx].tobytes().decode()


def _substitute(rng, w: str, alphabet: str, nsub: int) -> str:
    w = list(w)
    for pos in rng.choice(len(w), size=min(nsub, len(w)), replace=False):
        w[pos] = alphabet[rng.integers(len(alphabet))]
    return "".join(w)


def _edit(rng, w: str, alphabet: str, nedit: int) -> str:
    w = list(w)
    for _ in range(nedit):
        kind = rng.integers(3)
        if kind == 0 and w:                       # substitution
            w[rng.integers(len(w))] = alphabet[rng.integers(len(alphabet))]
        elif kind == 1:                           # insertion
            w.insert(int(rng.integers(len(w) + 1)), alphabet[rng.integers(len(alphabet))])
        elif w:                                   # deletion
            del w[rng.integers(len(w))]
    return "".join(w)


def _plant(rng, seqs, motif_copy, frac: float) -> None:
    nsel = int(round(frac * len(seqs)))
    for i in rng.choice(len(seqs), size=nsel, replace=False):
        c = motif_copy()
        s = seqs[i]
        if len(c) > len(s):
            continue
        pos = int(rng.integers(len(s) - len(c) + 1))
        seqs[i] = s[:pos] + c + s[pos + len(c):]


def dna_hd_small(seed: int = 1, scale: float = 1.0) -> Workload:
    rng = np.random.default_rng(seed)
    nseq = max(4, int(64 * scale))
    seqs = [_rand_seq(rng, DNA, 500) for _ in range(nseq)]
    motif = _rand_seq(rng, DNA, 12)
    _plant(rng, seqs, lambda: _substitute(rng, motif, DNA, int(rng.integers(3))), 0.5)
    return Workload("dna_hd_small", "DNA", seqs, d=0, k=12, e=2, q=50)


def dna_ed(seed: int = 2, scale: float = 1.0, d: int = 1, k: int = 15, e: int = 3) -> Workload:
    rng = np.random.default_rng(seed)
    nseq = max(4, int(round(1200 * scale)))
    p = [0.3, 0.2, 0.2, 0.3]                      # A C G T, GC = 40%
    seqs = [_rand_seq(rng, DNA, int(rng.integers(800, 1201)), p) for _ in range(nseq)]
    for frac in (0.2, 0.4, 0.6):
        motif = _rand_seq(rng, DNA, k)
        _plant(rng, seqs, lambda: _edit(rng, motif, DNA, int(rng.integers(e + 1))), frac)
    name = "dna_ed" if (k, e) == (15, 3) else f"dna_ed_k{k}"
    return Workload(name, "DNA", seqs, d=d, k=k, e=e, q=10)


def prot_uneven(seed: int = 3, scale: float = 1.0, d: int = 0) -> Workload:
    rng = np.random.default_rng(seed)
    nseq = max(4, int(round(2000 * scale)))
    freqs = rng.dirichlet([5.0] * 20)
    lens = np.exp(rng.uniform(math.log(50), math.log(2000), size=nseq)).astype(int)
    seqs = [_rand_seq(rng, AMINO20, int(n), freqs) for n in lens]
    for _ in range(5):
        motif = _rand_seq(rng, AMINO20, 10, freqs)
        frac = float(rng.uniform(0.15, 0.50))
        _plant(rng, seqs, lambda: _substitute(rng, motif, AMINO20, int(rng.integers(3))), frac)
    return Workload("prot_uneven", "PROT", seqs, d=d, k=10, e=2, q=15)


def dna_long(seed: int = 4, scale: float = 1.0) -> Workload:
    rng = np.random.default_rng(seed)
    nseq = 8
    length = max(200, int(1_000_000 * scale))
    alpha = np.frombuffer(DNA.encode(), dtype=np.uint8)
    seqs = []
    for _ in range(nseq):
        s = alpha[rng.integers(4, size=length)].copy()
        covered, target = 0, int(0.05 * length)
        while covered < target:
            unit = alpha[rng.integers(4, size=int(rng.integers(2, 7)))]
            copies = int(rng.integers(20, 201))
            rep = np.tile(unit, copies)
            mut = rng.random(rep.size) < 0.01
            rep[mut] = alpha[rng.integers(4, size=int(mut.sum()))]
            rep = rep[: max(1, min(rep.size, length // 4))]
            pos = int(rng.integers(0, length - rep.size + 1))
            s[pos:pos + rep.size] = rep
            covered += rep.size
        seqs.append(s.tobytes().decode())
    return Workload("dna_long", "DNA", seqs, d=0, k=20, e=3, q=50)


def dna_satellite(seed: int = 6, scale: float = 1.0) -> Workload:
    """Satellite-like DNA: 64 sequences of ~1 Mnt, each an exact tandem copy
    of one random 4096-nt unit from a random phase.  Only ~4k distinct words
    exist, so the DP is short and the HBM-bound stages (packing, the dedup
    sort of every factor, scans, compaction) carry a real share of the run:
    the workload their bandwidth is measured on."""
    rng = np.random.default_rng(seed)
    unit = _rand_seq(rng, DNA, 4096)
    length = max(8192, int(1_000_000 * scale))
    reps = length // len(unit) + 2
    seqs = []
    for _ in range(64):
        a = int(rng.integers(len(unit)))
        seqs.append((unit * reps)[a:a + length])
    return Workload("dna_satellite", "DNA", seqs, d=0, k=12, e=1, q=50)


def structured(seed: int = 2, scale: float = 1.0, d: int = 1) -> Workload:
    w = dna_ed(seed, scale, d=d)
    w.name = "structured"
    w.k, w.e = 8, 1
    w.boxes = ((5, 15, 10, 1),)
    return w


def structured2(seed: int = 2, scale: float = 1.0, d: int = 0) -> Workload:
    """Two gaps, the shape of the reference's example boxes file (gap 16-17,
    box 6 with 1 error; gap 15-16, box 7 with 2 errors) after a k 8 e 1 first
    box, on dna_ed's input."""
    w = dna_ed(seed, scale, d=d)
    w.name = "structured2"
    w.k, w.e = 8, 1
    w.boxes = ((16, 17, 6, 1), (15, 16, 7, 2))
    return w


def serve_stream(seed: int = 5, nreq: int = 2000, rate_hz: float = 200.0,
                 max_seqs: int = 256, max_len: int = 2000):
    """Poisson arrivals of extraction requests (arrival time in s, Workload)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for r in range(nreq):
        t += float(rng.exponential(1.0 / rate_hz))
        prot = bool(rng.integers(2))
        alphabet, letters = ("PROT", AMINO20) if prot else ("DNA", DNA)
        nseq = int(rng.integers(8, max_seqs + 1))
        lens = np.exp(rng.uniform(math.log(200), math.log(max_len), size=nseq)).astype(int)
        seqs = [_rand_seq(rng, letters, int(n)) for n in lens]
        k = int(rng.integers(8, (12 if prot else 24) + 1))
        e_hi = max(1, min(4, (k - 1) // 3))
        e = int(rng.integers(1, e_hi + 1))
        d = int(rng.integers(2))
        q = int(rng.choice([10, 25, 50]))
        out.append((t, Workload(f"req{r}", alphabet, seqs, d=d, k=k, e=e, q=q)))
    return out
