"""Rmtxop chains with matrix products (needs a GB300): the products run on
the GPU (double sums of single-precision products, rounded to single
precision, as util/rmatrix.c:806-838 rmx_multiply computes them); every
recorded chain equals the reference rmtxop's output (tests/golden/
rmtxop_chains.npz) to within the rounding of the last single-precision
product."""
import numpy as np
import pytest

from test_host import ROOT, rmtxop_chain

pytestmark = pytest.mark.gpu


def test_rmtxop_chains_with_products():
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib, rmtx
    _lib.lib()
    g = np.load(ROOT / "tests" / "golden" / "rmtxop_chains.npz")
    for i, chain in enumerate(g["chains"]):
        chain = str(chain)
        a = rmtx.read_rmatrix(rmtxop_chain(gb, g, chain)())
        assert a.shape == g[f"out{i}"].shape, chain
        np.testing.assert_allclose(a, g[f"out{i}"], rtol=3e-7, atol=0, err_msg=chain)


def test_rmtxop_product_errors():
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib
    _lib.lib()
    g = np.load(ROOT / "tests" / "golden" / "rmtxop_chains.npz")
    with pytest.raises(gb.GbError, match="mismatched dimensions"):
        rmtxop_chain(gb, g, "A . D").result()
    with pytest.raises(gb.GbError, match="components do not match"):
        rmtxop_chain(gb, g, "A . -t E").result()
