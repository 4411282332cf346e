"""motexGPU rejects bad switches and inputs exactly like the reference CLI
(messages of motex.cc:98-201 and the FASTA reader at motex.cc:225-300),
before any GPU work -- so these run without a GPU."""
import os

import pytest

from helpers import run_cli

FA = ">a\nACGTACGTAC\n>b\nACGTTTGCAA\n"
BASE = ["-a", "DNA", "-i", "in.fa", "-o", "out.motex", "-d", "0", "-k", "5", "-e", "1", "-q", "50"]


def _set(args, flag, val):
    a = list(args)
    a[a.index(flag) + 1] = val
    return a


CASES = [
    ("e_ge_k", _set(BASE, "-e", "5"), FA),
    ("q_gt_100", _set(BASE, "-q", "101"), FA),
    ("Q_gt_100", BASE + ["-Q", "101"], FA),
    ("d_is_2", _set(BASE, "-d", "2"), FA),
    ("bad_alphabet", _set(BASE, "-a", "RNA"), FA),
    ("not_fasta", BASE, "ACGT\n"),
    ("unexpected_char", BASE, ">a\nACGU\n"),
    ("carriage_return", BASE, ">a\r\nACGT\r\n"),
    ("missing_file", _set(BASE, "-i", "nope.fa"), FA),
    ("bad_number", _set(BASE, "-k", "x"), FA),
]


@pytest.mark.parametrize("name,args,fasta", CASES, ids=[c[0] for c in CASES])
def test_rejections_match_oracle(native_built, oracle_port, name, args, fasta):
    g = run_cli(native_built.CLI_PATH, None, args, files={"in.fa": fasta})
    o = run_cli(oracle_port, None, args, files={"in.fa": fasta})
    assert g[0] == o[0] == 1
    assert g[1] is None and o[1] is None
    if name != "bad_number":
        assert g[2] == o[2]


def test_missing_mandatory_switches(native_built):
    rc, out, err = run_cli(native_built.CLI_PATH, None, ["-a", "DNA", "-i", "in.fa"], files={"in.fa": FA})
    assert rc == 1 and out is None


@pytest.mark.parametrize("boxes", ["", "x\n", "1\n5\n", "1\n5\n15\n10\n"], ids=["empty", "not_int", "short", "no_err"])
def test_bad_boxes_file(native_built, oracle_port, boxes):
    args = BASE + ["-s", "in.boxes"]
    files = {"in.fa": FA, "in.boxes": boxes}
    g = run_cli(native_built.CLI_PATH, None, args, files=files)
    o = run_cli(oracle_port, None, args, files=files)
    assert g[0] == o[0] == 1
    assert g[2] == o[2]


COMBOS = [
    ("u_without_b", ["-u", "un.txt"]),
    ("U_without_b", ["-U", "un.smile"]),
    ("b_without_u", ["-b", "bg.motex"]),
    ("b_U_without_S", ["-b", "bg.motex", "-u", "un.txt", "-U", "un.smile"]),
    ("b_with_I", ["-b", "bg.motex", "-u", "un.txt", "-I", "un.in"]),
    ("s_with_I", ["-s", "in.boxes", "-I", "un.in"]),
]


@pytest.mark.parametrize("name,extra", COMBOS, ids=[c[0] for c in COMBOS])
def test_option_combinations_match_oracle(native_built, oracle_port, name, extra):
    """The reference's checks of -b/-u/-U/-S/-I/-s combinations (motex.cc:147-201)."""
    files = {"in.fa": FA, "in.boxes": "1\n1\n2\n3\n0\n"}
    g = run_cli(native_built.CLI_PATH, None, BASE + extra, files=files)
    o = run_cli(oracle_port, None, BASE + extra, files=files)
    assert g[0] == o[0] == 1
    assert g[2] == o[2] and "Error" in g[2]
