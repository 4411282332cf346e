"""motexGPU writes the reference's own output (golden fixtures) byte for byte,
apart from the two volatile header lines."""
import pytest

from conftest import golden_cases
from helpers import load_case, run_cli


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
def test_motexgpu_matches_reference(native_built, name):
    d, args, expected = load_case(name)
    rc, out, err = run_cli(native_built.CLI_PATH, d, args)
    assert rc == 0, err
    assert out == expected
