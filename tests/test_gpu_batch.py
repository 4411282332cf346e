"""Batched uneven-size extraction (motex_gpu_run_batch, one persistent DP
launch per kernel class) and graph replay of repeated executions: every
result must equal the same job run alone, bit for bit."""
import pytest

from motex_gb300 import workloads as W


def _jobs(native):
    out = []
    for wl in (W.dna_ed(seed=41, scale=0.02), W.prot_uneven(seed=42, scale=0.01, d=0),
               W.prot_uneven(seed=43, scale=0.015, d=1), W.dna_hd_small(seed=44, scale=0.25),
               W.structured(seed=45, scale=0.01, d=1), W.dna_ed(seed=46, scale=0.005, d=0)):
        out.append((wl.seqs, native.make_params(wl.d, wl.k, wl.e, wl.q, wl.Q, wl.n, wl.N, wl.boxes)))
    # factor longer than 32 (generic kernel) and a protein job with a low quorum
    wl = W.dna_ed(seed=47, scale=0.004, d=1)
    out.append((wl.seqs, native.make_params(1, 40, 4, 10)))
    wl = W.prot_uneven(seed=48, scale=0.01, d=1)
    out.append((wl.seqs, native.make_params(1, 6, 1, 5)))
    return out


@pytest.mark.gpu
def test_batch_equals_alone(native_built, gpu_ctx):
    jobs = _jobs(native_built)
    alone = [gpu_ctx.run(seqs, prm).motifs for seqs, prm in jobs]
    batch = gpu_ctx.run_batch(jobs)
    assert [b.motifs for b in batch] == alone
    assert sum(len(m) for m in alone) > 50
    # a second batch in a different order reuses the pooled jobs
    rev = gpu_ctx.run_batch(jobs[::-1])
    assert [b.motifs for b in rev] == alone[::-1]


@pytest.mark.gpu
def test_batch_guarded_lane_hamming_classes(native_built, gpu_ctx):
    """Several Hamming jobs of one kernel class run one persistent launch of
    the popc-free form (two lanes for DNA k 12, three for protein k 10 and
    k 8); each must equal the same job run alone."""
    jobs = []
    for s in range(4):
        wl = W.dna_hd_small(seed=60 + s, scale=0.1)
        jobs.append((wl.seqs, native_built.make_params(0, 12, 2, 10)))
    for s in range(3):
        wl = W.prot_uneven(seed=70 + s, scale=0.01, d=0)
        jobs.append((wl.seqs, native_built.make_params(0, 10, 2, 10)))
        jobs.append((wl.seqs, native_built.make_params(0, 8, 1, 20)))
    alone = [gpu_ctx.run(seqs, prm).motifs for seqs, prm in jobs]
    batch = gpu_ctx.run_batch(jobs)
    assert [b.motifs for b in batch] == alone
    assert sum(len(m) for m in alone) > 10


@pytest.mark.gpu
def test_repeated_execute_replays_identically(native_built, gpu_ctx):
    wl = W.prot_uneven(seed=49, scale=0.02, d=1)
    prm = native_built.make_params(wl.d, wl.k, wl.e, wl.q)
    gpu_ctx.load(wl.seqs, prm)
    runs = []
    for _ in range(4):                       # run, capture, replay, replay
        gpu_ctx.execute()
        runs.append(gpu_ctx.fetch())
    assert all(r.motifs == runs[0].motifs for r in runs)
    assert all(r.launches == runs[1].launches for r in runs[1:])
    assert runs[0].launches > 10
    # a new load after replays starts from scratch
    wl2 = W.prot_uneven(seed=50, scale=0.01, d=0)
    r2 = gpu_ctx.run(wl2.seqs, native_built.make_params(wl2.d, wl2.k, wl2.e, wl2.q))
    assert r2.motifs == gpu_ctx.run(wl2.seqs, native_built.make_params(wl2.d, wl2.k, wl2.e, wl2.q)).motifs
