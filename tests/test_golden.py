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
    st = CASES[name]
    v, i, tpo = sq.scene(st)
    mesh = sq.DeviceMesh(v, i)
    with sq.Renderer(sq.engine_state(st, W, H)) as r:
        r.update_scene(sq.camera(W, H))
        r.render_frame(mesh, tpo, st.percentTransparent)
        img = r.output()
        assert r.get_error() == 0
        frags = r.fragment_count()
    ref, n = gold(name)
    assert frags == n
    d = np.abs(img.astype(np.int32) - ref.astype(np.int32))
    assert d.max() <= 1, 'differs by %d LSB' % d.max()
