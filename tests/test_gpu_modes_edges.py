"""Edge inputs of the background (-b) and word-search (-I) modes: motexGPU
and the oracle built on the same host write the same files and exit the same
way (the reference's own behaviour on these inputs is undefined or aborts;
each case names what it does)."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import strip_volatile

FA = "".join(f">s{i}\n{s}\n" for i, s in enumerate([
    "ACGTACGTTAGCATCGATCGGATCGATCGTAGCTAGCTAGCATCG",
    "TTGACGTACGTTAGCATCGAAAACCGGTTAGCATCGATCGGATCA",
    "GGGACGTACGTTAGCTTCGATCGGATCGCCCCAAAATTTTGGGGA",
    "ACGTTGCAACGTACGTTAGCATCGATCGTAGCATCGTT",
]))
BASE = ["-a", "DNA", "-i", "in.fa", "-o", "out.motex", "-d", "1", "-k", "6", "-e", "1", "-q", "25"]
HEADER = ("####################################\n# Program: MoTeX\n# Rundate: x\n# Input file: bg.fa\n"
          "# Output file: bg.motex\n# For 10 input sequences\n#     d = 1\n#     q = {q}\n#     l = 6\n"
          "#     e = 1\n# Run on 1 proc(s) in 0.1 secs\n####################################\n\n")


def run_both(native_built, oracle_port, args, files, outputs):
    res = []
    for binary, extra in ((native_built.CLI_PATH, []), (oracle_port, ["-t", "2"])):
        with tempfile.TemporaryDirectory() as tmp:
            for name, text in files.items():
                with open(os.path.join(tmp, name), "w") as f:
                    f.write(text)
            p = subprocess.run([binary] + args + extra, cwd=tmp, capture_output=True, text=True, timeout=300)
            got = {}
            for o in outputs:
                path = os.path.join(tmp, o)
                got[o] = strip_volatile(open(path).read()) if os.path.exists(path) else None
            res.append((p.returncode, got, p.stderr))
    return res


@pytest.mark.gpu
def test_background_without_quorum(native_built, oracle_port):
    """A background made with -q 0: the reference's assert aborts; both exit 1."""
    files = {"in.fa": FA, "bg.motex": HEADER.format(q=0) + "ACGTAC 3 10 0.300000 4\n\n"}
    (g_rc, g, g_err), (o_rc, o, o_err) = run_both(native_built, oracle_port, BASE + ["-b", "bg.motex", "-u", "un.motex"],
                                                files, ["out.motex", "un.motex"])
    assert g_rc == o_rc == 1
    assert "no quorum" in g_err and "no quorum" in o_err


@pytest.mark.gpu
def test_background_missing_file(native_built, oracle_port):
    """The files get their headers, the error is printed, the exit status stays 0."""
    (g_rc, g, g_err), (o_rc, o, o_err) = run_both(native_built, oracle_port, BASE + ["-b", "nope.motex", "-u", "un.motex"],
                                                {"in.fa": FA}, ["out.motex", "un.motex"])
    assert g_rc == o_rc == 0
    assert g == o and g["out.motex"].startswith("####")
    assert "cannot open file" in g_err


@pytest.mark.gpu
def test_background_matches_and_repeats(native_built, oracle_port):
    """Matched, unmatched and a background key listed twice (its last row wins)."""
    rows = "ACGTAC 3 10 0.300000 4\nCGTACG 2 10 0.200000 2\nACGTAC 5 10 0.500000 7\nTTTTTT 1 10 0.100000 1\n\n"
    files = {"in.fa": FA, "bg.motex": HEADER.format(q=20) + rows + "#A total of 4 valid motifs were extracted.\n"}
    args = BASE + ["-b", "bg.motex", "-u", "un.motex", "-S", "o.smile", "-U", "u.smile"]
    (g_rc, g, _), (o_rc, o, _) = run_both(native_built, oracle_port, args, files,
                                          ["out.motex", "un.motex", "o.smile", "u.smile"])
    assert g_rc == o_rc == 0
    assert g == o
    assert " 0.500000 7 " in g["out.motex"]          # the repeated key took its last row
    assert g["u.smile"].count("\n") < g["o.smile"].count("\n")


@pytest.mark.gpu
@pytest.mark.parametrize("motifs,expect_lines", [
    ("ACGTAC 3 4 0.750000 4\nGGGGGG 1 4 0.250000 1\n\n", 2),       # header skipped up to its blank line
    ("TTACGTAC 3 4 0.750000 4\nAC 1 4 0.250000 1\n\n", 2),          # longer than k (last factor), shorter (0, 0)
])
def test_word_search_file_forms(native_built, oracle_port, motifs, expect_lines):
    files = {"in.fa": FA, "fg.in": HEADER.format(q=20) + motifs}
    args = BASE[:-2] + ["-q", "0", "-n", "0", "-I", "fg.in"]
    (g_rc, g, g_err), (o_rc, o, _) = run_both(native_built, oracle_port, args, files, ["out.motex"])
    assert g_rc == o_rc == 0, g_err
    assert g == o
    assert sum(1 for l in g["out.motex"].splitlines() if l and not l.startswith("#")) == expect_lines


@pytest.mark.gpu
def test_word_search_without_header_reads_nothing(native_built, oracle_port):
    """A bare motif list: everything before the first blank line is taken as header."""
    files = {"in.fa": FA, "fg.in": "ACGTAC 3 4 0.750000 4\n\n"}
    args = BASE[:-2] + ["-q", "0", "-n", "0", "-I", "fg.in"]
    (g_rc, g, _), (o_rc, o, _) = run_both(native_built, oracle_port, args, files, ["out.motex"])
    assert g_rc == o_rc == 0 and g == o
    assert "#A total of 0 valid motifs were extracted." in g["out.motex"]


@pytest.mark.gpu
def test_word_search_malformed_line(native_built, oracle_port):
    files = {"in.fa": FA, "fg.in": HEADER.format(q=20) + "ACGTAC 3 4\n\n"}
    args = BASE + ["-I", "fg.in"]
    (g_rc, _, g_err), (o_rc, _, o_err) = run_both(native_built, oracle_port, args, files, ["out.motex"])
    assert g_rc == o_rc == 1
    assert "not in the correct format" in g_err and "not in the correct format" in o_err
