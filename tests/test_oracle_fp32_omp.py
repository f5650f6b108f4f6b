"""The CPU baseline build of the oracle (FP32 blending, OpenMP tile-parallel
draws): the same fragments and integer A-buffers as the FP64 checker, and
images within FP32 rounding of it. It is timed by bench.py beside the
single-threaded FP64 oracle; it never checks the engine."""
import numpy as np
import pytest

import parity_util as pu
import oracle as orc
import vk_order_independent_transparency_gb300 as oit

CASES = [(orc.LINKEDLIST, 0, 100, 8), (orc.LOOP64, 0, 60, 8), (orc.SIMPLE, oit.OIT_AA_MSAA_4X, 100, 4),
         (orc.INTERLOCK, oit.OIT_AA_MSAA_8X, 100, 8), (orc.SPINLOCK, 0, 70, 4), (orc.LOOP, oit.OIT_AA_SUPER_4X, 100, 4),
         (orc.WEIGHTED, 0, 100, 8), (orc.LINKEDLIST, oit.OIT_AA_SSAA_4X, 100, 4)]


def _frame(variant, alg, aa, pct, L, W=96, H=72):
    v, i, tpo, sd = pu.scene(60, W, H, seed=11, radius_min=0.05, radius_max=0.25)
    fr = orc.render(alg, W, H, sd, v, i, tpo, pct, oit_layers=L, nodes_per_pixel=8, aa_type=aa, variant=variant)
    img, lin = fr.composite()
    return fr, img


@pytest.mark.parametrize('alg,aa,pct,L', CASES)
def test_fp32_omp_matches_checker(alg, aa, pct, L):
    import os
    orc.build()
    if not os.path.exists(orc.LIB_PATHS['fp32_omp']):
        pytest.skip('the oracle baseline build needs OpenMP')
    f64, img64 = _frame('fp64', alg, aa, pct, L)
    f32, img32 = _frame('fp32_omp', alg, aa, pct, L)
    assert f32.fragment_count() == f64.fragment_count() > 0
    if alg == orc.LOOP64:
        np.testing.assert_array_equal(f32.buffer(orc.BUF_ABUFFER), f64.buffer(orc.BUF_ABUFFER))
    if alg == orc.LINKEDLIST:
        # node numbers follow the threads' allocation order: compare the lists
        a64, a32 = f64.buffer(orc.BUF_AUX), f32.buffer(orc.BUF_AUX)
        assert pu.walk_lists(f32.buffer(orc.BUF_ABUFFER), a32) == pu.walk_lists(f64.buffer(orc.BUF_ABUFFER), a64)
    if alg in (orc.SIMPLE, orc.INTERLOCK, orc.SPINLOCK, orc.LOOP):
        np.testing.assert_array_equal(f32.buffer(orc.BUF_AUX), f64.buffer(orc.BUF_AUX))
    d = np.abs(img32.astype(np.int32) - img64.astype(np.int32))
    assert d.max() <= 2, d.max()  # FP32 vs FP64 blending before the sRGB8 encode
    assert (d > 1).mean() < 1e-3
