"""bench.py's CPU-baseline sample is bounded by symbols: on a workload of a
few very long sequences it must not start from whole sequences (a run that
is quadratic in 16 M symbols never ends).  A fake CPU run whose time grows
with the square of the symbols stands in for the real one."""
import bench
from motex_gb300 import workloads as W


def test_sample_is_bounded_in_symbols(monkeypatch):
    calls = []

    def fake_run(binary, wl, seqs, threads, timeout=600):
        n = sum(map(len, seqs))
        calls.append(n)
        secs = (n / 50_000.0) ** 2            # 50k symbols per second squared
        return n * n, secs

    monkeypatch.setattr(bench, "cpu_run", fake_run)
    wl = W.Workload("long", "DNA", ["ACGT" * 250_000] * 16, d=0, k=12, e=1, q=50)   # 16 x 1 Mnt
    sample, desc = bench.cpu_sample("x", wl, 8, target_s=12.0)
    assert calls[0] <= 20_000                               # the first probe is small
    assert all(b <= 2 * a for a, b in zip(calls, calls[1:]))  # and grows geometrically
    total = sum(map(len, sample))
    assert 100_000 < total < 300_000                        # ~sqrt(12) x 50k symbols
    assert "the last cut to" in desc and "of 16 sequences" in desc


def test_sample_takes_whole_set_when_cheap(monkeypatch):
    monkeypatch.setattr(bench, "cpu_run", lambda b, wl, seqs, t, timeout=600: (1, 0.001))
    wl = W.Workload("small", "DNA", ["ACGTACGTAC"] * 5, d=0, k=4, e=0, q=50)
    sample, desc = bench.cpu_sample("x", wl, 8)
    assert sample == wl.seqs


def test_reference_arm_line(monkeypatch):
    """The reference arm reports the same config keys as the GPU arm, n_gpus as
    launched, and its e2e as its own value (no host-device copies)."""
    import argparse
    monkeypatch.setattr(bench, "cpu_binary", lambda: ("x", "port"))
    monkeypatch.setattr(bench, "cpu_run", lambda b, wl, seqs, t, timeout=600: (bench.ref_cells(wl, seqs), 0.5))
    args = argparse.Namespace(workload="dna_hd_small", scale=1.0, steps=2, warmup=1)
    line = bench.run_reference(args, 2)
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    cfg = line["config"]
    for key in ("workload", "scale", "alphabet", "num_seqs", "total_len", "d", "k", "e", "q", "ref_cells", "parallelism"):
        assert key in cfg, key
    assert cfg["ref_cells"] == 32000 * 32000                 # 64 x 500 nt, every sequence searched
    # the GPU arm builds its config with the same function: identical keys
    gpu_cfg = bench.workload_config(args, bench.WORKLOADS["dna_hd_small"](1.0), 2, "flushed")
    assert set(cfg) == set(gpu_cfg)
    assert {k: v for k, v in cfg.items() if k != "l2"} == {k: v for k, v in gpu_cfg.items() if k != "l2"}
    assert line["e2e"]["value"] == line["value"] == line["cpu_baseline"]["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_kernel_names_follow_the_tuned_form():
    """The bench line names the DP kernel the engine runs: the default for the
    workload, or the form of the autotuner's entry (a negative lane count is
    the popc-free Hamming form)."""
    ed = W.dna_ed(scale=0.01)
    hd_small = W.dna_hd_small(scale=0.1)
    prot_hd = W.prot_uneven(d=0, scale=0.01)
    assert bench.dp_kernel_name(ed) == "k_dp_swar_ed (NL=2)"
    assert bench.dp_kernel_name(hd_small) == "k_dp_hclr (NL=2)"          # k 12: two lanes
    assert bench.dp_kernel_name(prot_hd) == "k_dp_hclr (NL=3)"           # k 10: three lanes
    assert bench.tuned_kernel_name(prot_hd, (8, -3, 4)) == "k_dp_hclr (NL=3) W=8 NL=3 UR=4"
    assert bench.tuned_kernel_name(prot_hd, (8, 3, 4)) == "k_dp_hswar (NL=3) W=8 NL=3 UR=4"
    assert bench.tuned_kernel_name(hd_small, (4, 1, 8)) == "k_dp_fast W=4 NL=1 UR=8"
    assert bench.tuned_kernel_name(ed, (8, 2, 4)) == "k_dp_swar_ed (NL=2) W=8 NL=2 UR=4"
