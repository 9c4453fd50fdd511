"""CUDA path against the reference's own outputs (golden fixtures), bit for bit."""
import pytest

from conftest import golden_cases, load_golden, run_cli


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_gpu_matches_reference(name, built, golden_inputs, tmp_path):
    g = golden_inputs[name]
    rec, oc, st, log = run_cli(built["cli"], g["args"], g["db"], g["skip"], str(tmp_path))
    grec, goc, gst = load_golden(name)
    assert rec.shape == grec.shape, log[-2000:]
    assert (rec == grec).all()
    assert oc == goc
    assert st == gst
