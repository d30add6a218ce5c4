"""The oracle against the committed golden fixtures (tests/golden/).

The fixtures hold small seeded inputs and the oracle's outputs for them,
written by tests/golden/make_golden.py.  Recomputing them here catches any
change in the oracle's arithmetic; the GPU tests in test_gpu_golden.py
compare the CUDA paths against the same files."""
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def generator():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


GEN = generator()


@pytest.mark.parametrize("name", sorted(GEN.cases()))
def test_oracle_reproduces_golden(name):
    want = load(name)
    got = GEN.cases()[name]()
    assert set(got) == set(want)
    for key, ref in want.items():
        val = np.asarray(got[key])
        assert val.shape == ref.shape, key
        if key in ("strings",):  # column 9 is exp(-chi2 / 2) through libm
            cols = [c for c in range(ref.shape[1]) if c != 9]
            assert np.array_equal(val[:, cols], ref[:, cols]), key
            np.testing.assert_allclose(val[:, 9], ref[:, 9], rtol=1e-14)
        elif name.startswith(("green", "spectrum")) and val.dtype.kind in "fc":
            # libm sin / cos in the phases and twiddles
            np.testing.assert_allclose(val, ref, rtol=1e-13, atol=1e-13 * np.max(np.abs(ref)), err_msg=key)
        else:
            assert np.array_equal(val, ref), key


def test_golden_inputs_are_nontrivial():
    d = load("defects_8")
    assert d["counts"][0] > 0 and d["counts"][1] > 0 and len(d["strings"]) == d["counts"][0]
    g = load("green_ref_8")
    assert np.any(g["acc"] != 0) and g["nt"] > 0
    g = load("green_degrade1_ref_16")
    assert g["acc"].shape == (4, 8, 8, 8) and g["phi0"].shape == (16, 16, 16) and np.any(g["acc"] != 0)
    lf = load("leapfrog_uij_ref_6")
    assert not np.array_equal(lf["phi"], lf["phi0"])
