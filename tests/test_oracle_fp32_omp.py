"""The CPU baseline build of the oracle (FP32 blending, OpenMP tile-parallel
draws): the same fragments and integer A-buffers as the FP64 oracle, and
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
def test_fp32_omp_matches_fp64_oracle(alg, aa, pct, L):
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


@pytest.mark.parametrize('alg', [orc.LOOP64, orc.INTERLOCK, orc.WEIGHTED])
def test_fp32_omp_same_result_on_any_thread_count(alg, tmp_path):
    """Each pixel belongs to one thread's tile and sees its fragments in
    primitive order: 1, 3 and 8 threads give the same images and k-buffers."""
    import hashlib
    import os
    import subprocess
    import sys
    orc.build()
    if not os.path.exists(orc.LIB_PATHS['fp32_omp']):
        pytest.skip('the oracle baseline build needs OpenMP')
    here = os.path.dirname(os.path.abspath(__file__))
    code = (
        "import sys, hashlib; sys.path[:0] = [%r, %r, %r]\n"
        "import oracle as orc, parity_util as pu\n"
        "v, i, tpo, sd = pu.scene(80, 120, 90, seed=4, radius_min=0.05, radius_max=0.25)\n"
        "fr = orc.render(%d, 120, 90, sd, v, i, tpo, 80, oit_layers=4, aa_type=4 if %d == orc.INTERLOCK else 0,"
        " variant='fp32_omp')\n"
        "img, _ = fr.composite()\n"
        "h = hashlib.sha256(img.tobytes() + (fr.buffer(orc.BUF_ABUFFER).tobytes() if %d != orc.WEIGHTED else b''))\n"
        "print(h.hexdigest(), fr.fragment_count())\n" % (os.path.join(here, '..', 'oracle'), here,
                                                      os.path.join(here, '..'), alg, alg, alg))
    outs = set()
    for n in (1, 3, 8):
        env = dict(os.environ, OMP_NUM_THREADS=str(n))
        r = subprocess.run([sys.executable, '-c', code], env=env, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.add(r.stdout.strip().splitlines()[-1])
    assert len(outs) == 1, outs
