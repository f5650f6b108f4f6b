"""Golden fixtures of the reference's test sequence (tests/golden/, written by
tests/golden/make_golden.py): the oracle must reproduce them bit for bit, the
engine within 1 LSB with the same fragment counts."""
import os

import numpy as np
import pytest

from vk_order_independent_transparency_gb300 import sequence as sq

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, 'golden', 'sequence_64x40.npz'))
W, H = int(GOLD['width']), int(GOLD['height'])
NAMES = [str(n) for n in GOLD['names']]
CASES = dict(sq.cases())


def gold(name):
    k = NAMES.index(name)
    return GOLD['images'][k], int(GOLD['fragments'][k])


def test_fixture_covers_sequence():
    assert NAMES == [n for n, _ in sq.cases()]
    assert GOLD['images'].shape == (len(NAMES), H, W, 4)


@pytest.mark.parametrize('name', NAMES)
def test_oracle_matches_golden(name):
    import oracle as orc
    st = CASES[name]
    v, i, tpo = sq.scene(st)
    kw = sq.state_kwargs(st)
    kw.pop('interlock_is_ordered')
    fr = orc.render(st.algorithm, W, H, sq.camera(W, H), v, i, tpo, st.percentTransparent, **kw)
    img, _ = fr.composite()
    ref, frags = gold(name)
    assert fr.fragment_count() == frags
    np.testing.assert_array_equal(img, ref)


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_engine_matches_golden(name):
    """Where the linked-list pool overflows (MSAA at this size: about one pixel
    per sphere, so four to eight times the fragments of 1x), which fragments
    get a node depends on allocation order, as in the reference; the engine
    allocates per tile, the oracle frame-wide. There each pixel keeps a
    primitive-order prefix of its fragments, and the oracle replays the
    engine's per-pixel prefix lengths instead of using the fixture."""
    import parity_util as pu
    st = CASES[name]
    v, i, tpo = sq.scene(st)
    kw = sq.state_kwargs(st)
    g = pu.render_gpu(st.algorithm, W, H, v, i, tpo, sq.camera(W, H), st.percentTransparent, **kw)
    g['renderer'].close()
    assert g['error'] == 0
    ref, n = gold(name)
    assert g['fragments'] == n
    msaa, sample_shading, sup = sq.aa_settings(st.aaType)
    lists = W * H * sup * sup * (msaa if sample_shading else 1)
    if st.algorithm == sq.OIT_LINKEDLIST and n > st.linkedListAllocatedPerElement * lists:
        import oracle as orc
        assert g['counter'][0] == n
        heads = g['aux'][:lists]
        limit = np.array([len(x) for x in pu.walk_lists(g['abuf'], heads)], np.uint32)
        assert limit.sum() == st.linkedListAllocatedPerElement * lists - 1  # every node but the terminator
        kw.pop('interlock_is_ordered')
        fr = orc.Frame(st.algorithm, W, H, **{k: kw[k] for k in ('oit_layers', 'nodes_per_pixel', 'aa_type',
                                                                  'tail_blend', 'alpha_min', 'alpha_width')})
        fr.set_ll_store_limit(limit)
        fr.begin()
        fr.clear_transparent()
        fr.draw_transparent(sq.camera(W, H), v, i, 0, i.shape[0])
        ref, _ = fr.composite()
    d = np.abs(g['image'].astype(np.int32) - ref.astype(np.int32))
    assert d.max() <= 1, 'differs by %d LSB' % d.max()
