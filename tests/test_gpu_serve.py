"""Serving loop (motex_srv_*): requests of different sizes, alphabets and
parameters served by continuous batching give the same result as the same
request run alone; admission respects the memory budget; waits are bounded
on the host; a bad request fails alone without taking its batch down."""
import threading
import time

import pytest

from motex_gb300 import workloads as W


def _requests(native, n, seed):
    out = []
    for _, wl in W.serve_stream(seed=seed, nreq=n, max_seqs=32, max_len=500):
        out.append((wl.seqs, native.make_params(wl.d, wl.k, wl.e, wl.q)))
    return out


@pytest.mark.gpu
def test_served_equals_alone(native_built, gpu_ctx):
    reqs = _requests(native_built, 40, 7)
    alone = [gpu_ctx.run(s, p).motifs for s, p in reqs]
    with native_built.Server(max_batch=8, workers=2) as srv:
        ids = [srv.submit(s, p) for s, p in reqs]
        got = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert [g[0].motifs for g in got] == alone
    assert st["completed"] == 40 and st["failed"] == 0
    assert st["batches"] < 40 and st["max_batch_seen"] > 1
    assert all(g[1]["latency_ms"] >= g[1]["run_ms"] >= 0 for g in got)


@pytest.mark.gpu
def test_concurrent_submitters_and_tight_budget(native_built, gpu_ctx):
    reqs = _requests(native_built, 24, 8)
    alone = [gpu_ctx.run(s, p).motifs for s, p in reqs]
    # a budget that holds only a few requests at a time
    with native_built.Server(hbm_budget=64 << 20, max_batch=16, workers=2) as srv:
        got = [None] * len(reqs)

        def client(k):
            for i in range(k, len(reqs), 3):
                rid = srv.submit(*reqs[i])
                got[i] = srv.wait(rid)[0].motifs

        th = [threading.Thread(target=client, args=(k,)) for k in range(3)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        st = srv.stats()
    assert got == alone
    assert st["in_use_bytes"] == 0 and st["completed"] == len(reqs)


@pytest.mark.gpu
def test_admission_timeouts_and_errors(native_built):
    big = W.dna_ed(seed=9, scale=0.2)
    prm = native_built.make_params(1, 15, 3, 10)
    with native_built.Server(hbm_budget=1 << 20, max_batch=4, workers=1) as srv:
        with pytest.raises(native_built.MotexError) as ei:
            srv.submit(big.seqs, prm)                       # can never fit 1 MiB
        assert ei.value.code == -2
    with native_built.Server(max_batch=4, workers=1) as srv:
        rid = srv.submit(big.seqs, prm)
        with pytest.raises(native_built.MotexError) as ei:
            srv.wait(rid, timeout_ms=0)                      # still running: bounded host wait
        assert ei.value.code == -5
        res, tm = srv.wait(rid)
        assert len(res.motifs) > 0
        with pytest.raises(native_built.MotexError) as ei:
            srv.wait(rid, timeout_ms=0)                      # already collected
        assert ei.value.code == -7
        # a request with e >= k fails alone; its batch-mates still succeed
        small = W.dna_ed(seed=10, scale=0.01)
        good = srv.submit(small.seqs, native_built.make_params(1, 8, 1, 20))
        bad = srv.submit(small.seqs, native_built.make_params(1, 8, 8, 20))
        good2 = srv.submit(small.seqs, native_built.make_params(0, 8, 1, 20))
        assert len(srv.wait(good)[0].motifs) > 0
        with pytest.raises(native_built.MotexError) as ei:
            srv.wait(bad)
        assert ei.value.code == -1
        assert len(srv.wait(good2)[0].motifs) > 0
