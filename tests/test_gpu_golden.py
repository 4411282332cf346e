"""motexGPU writes the reference's own output (golden fixtures) byte for byte,
apart from the two volatile header lines."""
import pytest

from conftest import golden_cases, mode_cases
from helpers import (expected_smile, load_case, load_mode_case, read_smile, run_cli, run_outputs,
                     same_but_pvalues)


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
def test_motexgpu_matches_reference(native_built, name):
    d, args, expected = load_case(name)
    rc, out, err = run_cli(native_built.CLI_PATH, d, args)
    assert rc == 0, err
    assert out == expected


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in golden_cases() if expected_smile(n) is not None])
def test_motexgpu_smile_matches_reference(native_built, name):
    """-S writes the reference's SMILE-like file byte for byte (bar the user-time line)."""
    d, args, expected = load_case(name)
    rc, out, smile, err = read_smile(d, native_built.CLI_PATH, args)
    assert rc == 0, err
    assert out == expected
    assert smile == expected_smile(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", mode_cases())
def test_motexgpu_modes_match_reference(native_built, oracle_port, name):
    """-b/-u/-S/-U and -I (the word search runs on the GPU): the reference's
    files line for line, the p-value column within its long double rounding
    (the fixtures come from an x86-64 build); and identical to the oracle
    built on this host, whose long double arithmetic is the same."""
    d, args, expected = load_mode_case(name)
    rc, got, err = run_outputs(native_built.CLI_PATH, d, args, list(expected))
    assert rc == 0, err
    rc2, port, err2 = run_outputs(oracle_port, d, args, list(expected), extra=["-t", "8"])
    assert rc2 == 0, err2
    for o, text in expected.items():
        assert got[o] is not None, o
        assert same_but_pvalues(got[o], text) is None, (o, same_but_pvalues(got[o], text))
        assert got[o] == port[o], o
