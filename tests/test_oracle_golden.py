"""The CPU oracle against the reference's own outputs (golden fixtures)."""
import pytest

from conftest import golden_cases, load_golden, run_cli


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_oracle_matches_reference(name, oracle, golden_inputs, tmp_path):
    g = golden_inputs[name]
    rec, oc, st, _ = run_cli(oracle["cli"], g["args"], g["db"], g["skip"], str(tmp_path))
    grec, goc, gst = load_golden(name)
    assert rec.shape == grec.shape
    assert (rec == grec).all()
    assert oc == goc
    assert st == gst
