"""The oracle against the reference's own outputs, when they exist.

``tests/golden/make_reference_golden.py`` runs the reference (JaxPM) on the
inputs of the oracle's fixtures wherever JAX, jax_cosmo and jaxdecomp
import, and writes ``tests/golden/reference_jaxpm.npz``.  Neither machine
this project is built and tested on has JAX, so the file is absent there and
these tests skip: the oracle is then held by analytic known answers and its
own frozen fixtures (``tests/test_oracle.py``).  With the file present they
pin the oracle to the reference: CIC paint and read (absolute and relative
mode) to float32 rounding, pm_forces to 1e-5 relative L2 in float64, LPT
fields and the five-step FastPM state to 1e-4 (the growth tables are
integrated differently), and the growth functions to 1e-4."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2
from oracle import cic, cosmology as cm, fourier as fo

PATH = os.path.join(GOLDEN, "reference_jaxpm.npz")

pytestmark = pytest.mark.skipif(not os.path.exists(PATH),
                                reason="no reference outputs: JAX is not importable where "
                                       "this project is tested (make_reference_golden.py)")


@pytest.fixture(scope="module")
def ref():
    return np.load(PATH)


def test_cic_against_reference(ref, golden):
    d = golden("cic.npz")
    for tag in ("cube", "rect"):
        np.testing.assert_allclose(d[f"{tag}_paint64"], ref[f"{tag}_paint64"], rtol=1e-12,
                                   atol=1e-12)
        np.testing.assert_allclose(d[f"{tag}_read32"], ref[f"{tag}_read32"], rtol=1e-6,
                                   atol=1e-6)
        np.testing.assert_allclose(d[f"{tag}_rel_paint32"], ref[f"{tag}_rel_paint32"],
                                   rtol=1e-6, atol=1e-6)
        rd = cic.cic_read_dx(d[f"{tag}_mesh"], d[f"{tag}_disp"])
        np.testing.assert_allclose(rd, ref[f"{tag}_rel_read32"], rtol=1e-6, atol=1e-6)


def test_pm_forces_against_reference(ref, golden):
    d = golden("pm_forces16.npz")
    assert rel_l2(d["forces64"], ref["forces64"]) < 1e-5
    assert rel_l2(d["forces64_rsplit"], ref["forces64_rsplit"]) < 1e-5
    assert rel_l2(d["forces32"], ref["forces32"]) < 1e-5


def test_lpt_and_fastpm_against_reference(ref, golden):
    d = golden("sim16.npz")
    for key in ("dx1", "p1", "f1", "dx2", "p2", "f2"):
        assert rel_l2(d[key], ref[key]) < 1e-4, key
    lat = cic.lattice((16,) * 3).reshape(-1, 3)
    assert rel_l2(d["final_pos"] - lat, ref["final_pos"] - lat) < 1e-4
    assert rel_l2(d["final_vel"], ref["final_vel"]) < 1e-4


def test_growth_against_reference(ref):
    c = cm.Cosmology()
    a = ref["a"]
    for name, fn in (("growth_factor", cm.growth_factor), ("growth_rate", cm.growth_rate),
                     ("Gf", cm.Gf), ("dGfa", cm.dGfa), ("gp", cm.gp)):
        np.testing.assert_allclose(fn(c, a), ref[name], rtol=1e-4, err_msg=name)
