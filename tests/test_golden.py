"""Golden fixtures (tests/golden, written by tests/golden/make_golden.py from the oracle).

CPU: the oracle reproduces every fixture exactly (it has not drifted).
GPU: the library, given the fixture's inputs through the C-ABI, reproduces the spins bit for
bit (Ising; the FP32 Heisenberg state), E and M within 1e-12 relative (the reductions sum in
another order), and S(q) within the structure-factor tolerance (|S_a|/N 3e-4 absolute,
|S|^2/N^2 1e-3 of the largest value).
"""
import numpy as np
import pytest

from tests.golden import golden


@pytest.mark.parametrize("name", golden.SWEEP_CASES)
def test_oracle_reproduces_sweep_fixture(name):
    fix = golden.load(name)
    got = golden.oracle_sweeps(fix)
    np.testing.assert_array_equal(got["spins"], fix["spins"])
    np.testing.assert_array_equal(got["E"], fix["E"])
    np.testing.assert_array_equal(got["M"], fix["M"])


@pytest.mark.parametrize("name", golden.SQ_CASES)
def test_oracle_reproduces_sq_fixture(name):
    fix = golden.load(name)
    got = golden.oracle_sq(fix)
    np.testing.assert_array_equal(got["sq"], fix["sq"])
    np.testing.assert_array_equal(got["comp"], fix["comp"])


def test_fixtures_cover_the_kernel_paths():
    """The cases run the general and the simple-cubic kernels of both models, both proposal
    kinds, overrelaxation, the field, both anisotropies and a staggered magnetisation."""
    metas = {n: golden.load(n)["meta"] for n in golden.SWEEP_CASES}
    assert {m["model"] for m in metas.values()} == {golden.MODEL_ISING, golden.MODEL_XYZ}
    assert any(m["angle"] for m in metas.values()) and any(not m["angle"] for m in metas.values())
    assert any(op == "ovrr" for m in metas.values() for op, _ in m["schedule"])
    assert any(m["sia"] for m in metas.values())
    assert "sia_local" in golden.load("pyro3_xyz_angle_local_sia")
    assert np.any(golden.load("sc8x4x4_ising_staggered")["stgg"] < 0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden.SWEEP_CASES)
def test_gpu_reproduces_sweep_fixture(name):
    fix = golden.load(name)
    got, fast = golden.gpu_sweeps(fix)
    # the simple-cubic cases with an even first side run the fast kernels
    assert fast == (1 if name.startswith("sc8") else 0)
    np.testing.assert_array_equal(got["spins"], fix["spins"])
    np.testing.assert_allclose(got["E"], fix["E"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(got["M"], fix["M"], rtol=1e-12, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden.SQ_CASES)
def test_gpu_reproduces_sq_fixture(name):
    fix = golden.load(name)
    got = golden.gpu_sq(fix)
    np.testing.assert_allclose(got["comp"], fix["comp"], atol=3e-4, rtol=0)
    np.testing.assert_allclose(got["sq"], fix["sq"], atol=1e-3 * fix["sq"].max(), rtol=0)
