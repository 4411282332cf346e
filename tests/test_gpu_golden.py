"""motexGPU writes the reference's own output (golden fixtures) byte for byte,
apart from the two volatile header lines."""
import pytest

from conftest import golden_cases
from helpers import expected_smile, load_case, read_smile, run_cli


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
