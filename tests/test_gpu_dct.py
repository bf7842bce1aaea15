"""dctimestep's product on the GPU against FP64 (needs a GB300).

R[m,n,c] = sum_k DC[m,k,c] * S[k,n,c] (util/cmatrix.c:421-474).  The
operands are daylight-coefficient-like: lognormal DC with 30% exact zeros,
a lognormal sky with a sun-patch spike per daylight hour and half of the
hours dark (all-zero columns).  Error bounds, relative to an FP64 product of
the same float32 operands, over every non-zero output:
  FP16X3 (pre-scaled fp16 split, the drop-in's form)  max 1e-5, mean 1e-6
  BF16X3 (bf16 split)                                  max 3e-5, mean 3e-6
  FP16   (pre-scaled, one product)                     max 4e-3
  FP32   (CUDA cores)                                  max 1e-5
"""
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import _lib
    _lib.lib()
    return gb


def dc_pair(rng, M, K, N, sun=True):
    dc = rng.lognormal(-6, 2, (M, K, 3)).astype(np.float32)
    dc[rng.random((M, K)) < 0.3] = 0
    sky = rng.lognormal(2, 1, (K, N, 3)).astype(np.float32)
    if sun:
        cols = np.arange(N)
        sky[rng.integers(0, K, N), cols, :] = np.exp(rng.uniform(np.log(1e4), np.log(1e6), N))[:, None]
    sky[:, rng.random(N) < 0.5] = 0
    ref = np.stack([dc[..., c].astype(np.float64) @ sky[..., c].astype(np.float64) for c in range(3)], -1)
    return dc, sky, ref


BOUNDS = {"fp16x3": (1e-5, 1e-6), "bf16x3": (3e-5, 3e-6), "fp16": (4e-3, 1e-3), "fp32": (1e-5, 1e-6)}


@pytest.mark.parametrize("mode", ["fp16x3", "bf16x3", "fp16"])
@pytest.mark.parametrize("M,K,N", [(300, 333, 700), (2100, 700, 2100), (520, 2306, 1000), (131, 150, 1003)])
def test_tensor_core_forms_vs_fp64(gb, mode, M, K, N):
    """Sizes that are not multiples of the 128 x 256 x 32 tiles; the second
    has more tiles than SMs and a partial row-tile group, the third the
    Reinhart MF:4 patch count of the annual workload, the fourth an odd
    column count (rows not 16-byte aligned: zero columns stored float by
    float)."""
    dc, sky, ref = dc_pair(np.random.default_rng(M + K), M, K, N)
    out = gb.dctimestep_array(dc, sky, mode=mode)
    nz = ref != 0
    np.testing.assert_array_equal(out[~nz], 0.0)
    rel = np.abs(out[nz] - ref[nz]) / np.abs(ref[nz])
    mx, mean = BOUNDS[mode]
    assert rel.max() <= mx and rel.mean() <= mean, (rel.max(), rel.mean())


def test_fp32_fp64_against_reference_program(gb):
    g = golden("dct_small.npz")
    r64 = gb.dctimestep_array(g["dc"], g["sky"], mode="fp64")
    np.testing.assert_allclose(r64, g["out"], rtol=1e-6, atol=1e-30)
    for mode in ("fp32", "fp16x3"):
        r = gb.dctimestep_array(g["dc"], g["sky"], mode=mode)
        np.testing.assert_allclose(r, g["out"], rtol=1e-5, atol=1e-7 * np.abs(g["out"]).max())


def test_zero_rows_and_columns_skipped(gb):
    """All-zero rows of DC and all-zero columns of the sky give exact zeros
    (cm_multiply's skip); a row or column holding only a negative zero
    counts as non-zero there, as the byte comparison does, and still gives
    zero; rows and columns of mixed sign are scaled by their magnitudes."""
    rng = np.random.default_rng(7)
    M, K, N = 700, 300, 900
    dc, sky, _ = dc_pair(rng, M, K, N)
    dc[::3] = 0
    dc[1, :, :] = 0
    dc[1, 5, 1] = -0.0
    sky[:, 2:N:4] = 0
    sky[:, 3, :] = 0
    sky[7, 3, 2] = -0.0
    dc[10] *= -1
    sky[:, 11] *= -1
    ref = np.stack([dc[..., c].astype(np.float64) @ sky[..., c].astype(np.float64) for c in range(3)], -1)
    for mode in ("fp16x3", "bf16x3", "fp16"):
        out = gb.dctimestep_array(dc, sky, mode=mode)
        assert (out[::3] == 0).all() and (out[:, 2:N:4] == 0).all() and (out[1] == 0).all()
        assert (out[:, 3] == 0).all()
        nz = ref != 0
        rel = np.abs(out[nz] - ref[nz]) / np.abs(ref[nz])
        assert rel.max() <= BOUNDS[mode][0], (mode, rel.max())
    # nothing non-zero at all
    out = gb.dctimestep_array(np.zeros((5, 4, 3), np.float32), sky[:4], mode="fp16x3")
    assert (out == 0).all()


def test_wide_dynamic_range_rows(gb):
    """Rows and columns whose magnitudes differ by 1e30 from one another:
    each is scaled by its own power of two, so none leaves the FP16 range."""
    rng = np.random.default_rng(3)
    M, K, N = 260, 200, 300
    dc, sky, _ = dc_pair(rng, M, K, N, sun=False)
    dc *= np.float32(10.0) ** rng.integers(-15, 15, (M, 1, 1)).astype(np.float32)
    sky *= np.float32(10.0) ** rng.integers(-15, 15, (1, N, 1)).astype(np.float32)
    ref = np.stack([dc[..., c].astype(np.float64) @ sky[..., c].astype(np.float64) for c in range(3)], -1)
    out = gb.dctimestep_array(dc, sky, mode="fp16x3")
    nz = ref != 0
    rel = np.abs(out[nz] - ref[nz]) / np.abs(ref[nz])
    assert rel.max() <= 1e-5, rel.max()


@pytest.mark.parametrize("mode", ["fp16x3", "fp16"])
def test_clusters_of_two_equal_single_ctas(gb, mode):
    """Row tiles paired in clusters of two CTAs, each copying half of the
    shared column tile into both, give the same bits as one CTA per tile
    (GB_DCT_CLUSTER=1); a single row tile (M <= 128) runs without
    clusters and meets the same bounds."""
    dc, sky, ref = dc_pair(np.random.default_rng(5), 700, 500, 900)
    pair = gb.dctimestep_array(dc, sky, mode=mode)
    os.environ["GB_DCT_CLUSTER"] = "1"
    try:
        single = gb.dctimestep_array(dc, sky, mode=mode)
    finally:
        del os.environ["GB_DCT_CLUSTER"]
    np.testing.assert_array_equal(pair, single)
    dc, sky, ref = dc_pair(np.random.default_rng(6), 100, 500, 900)
    out = gb.dctimestep_array(dc, sky, mode=mode)
    nz = ref != 0
    np.testing.assert_array_equal(out[~nz], 0.0)
    rel = np.abs(out[nz] - ref[nz]) / np.abs(ref[nz])
    mx, mean = BOUNDS[mode]
    assert rel.max() <= mx and rel.mean() <= mean, (rel.max(), rel.mean())


def test_pipeline_wait_limit_returns_error(gb):
    """A pipeline wait limit of 1 ns (GB_DCT_WAIT_NS) makes the first wait
    that is not met at once run out: the kernel records the error, drains
    its copies and products, frees its tensor memory, and the call returns
    GB_ECUDA.  The next call, with the normal limit, is correct."""
    from pyradiance_gb300 import _lib
    dc, sky, ref = dc_pair(np.random.default_rng(11), 600, 900, 800)
    os.environ["GB_DCT_WAIT_NS"] = "1"
    try:
        with pytest.raises(_lib.GbError) as e:
            gb.dctimestep_array(dc, sky, mode="fp16x3")
        assert e.value.code == -4
        assert "wait expired" in str(e.value)
    finally:
        del os.environ["GB_DCT_WAIT_NS"]
    out = gb.dctimestep_array(dc, sky, mode="fp16x3")
    nz = ref != 0
    rel = np.abs(out[nz] - ref[nz]) / np.abs(ref[nz])
    assert rel.max() <= 1e-5
