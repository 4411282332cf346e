"""Failure detection on the device, without a GPU fault: the packer stages its
input tiles into shared memory with TMA bulk copies and waits for each on an
mbarrier with a bounded number of try_wait polls.  MOTEX_PACK_WAIT_POLLS=0
makes every such wait give up at once.  The copies themselves are valid and
land, and the kernel drains them before its CTAs exit, so nothing faults or
hangs; the run must come back promptly with MOTEX_ETIMEOUT, and the same
context must then extract bit-exactly (checked against the oracle)."""
import os
import tempfile
import time

import pytest

from motex_gb300 import workloads as W

import __graft_entry__ as entry


def _gpu_rows(wl, got):
    return [(wl.seqs[s][p - wl.k + 1: p + 1], u, v) for s, p, _, u, v in got.motifs]


@pytest.mark.gpu
@pytest.mark.parametrize("d", [0, 1])
def test_staging_wait_gives_up_then_context_recovers(native_built, oracle_port, monkeypatch, d):
    wl = W.dna_ed(seed=11, scale=0.05, d=d)            # 60 sequences, several staged tiles per CTA
    wl.k, wl.e, wl.q = 10, 1, 10
    prm = native_built.make_params(d, wl.k, wl.e, wl.q)
    # the staged pipeline (the small-job pipeline packs without TMA staging)
    monkeypatch.setenv("MOTEX_MINI", "0")
    ctx = native_built.Context(0)
    try:
        monkeypatch.setenv("MOTEX_PACK_WAIT_POLLS", "0")
        t0 = time.time()
        with pytest.raises(native_built.MotexError) as ei:
            ctx.run(wl.seqs, prm)
        assert ei.value.code == -5, str(ei.value)          # MOTEX_ETIMEOUT
        assert "staging wait gave up" in str(ei.value)
        assert "drain" not in str(ei.value)                # the copies in flight landed
        assert time.time() - t0 < 30
        monkeypatch.delenv("MOTEX_PACK_WAIT_POLLS")
        got = ctx.run(wl.seqs, prm)                         # same context, normal limit
    finally:
        ctx.close()
    with tempfile.TemporaryDirectory() as tmp:
        ref = entry._port_output(wl, tmp)
    assert _gpu_rows(wl, got) == ref
    assert len(ref) > 0
