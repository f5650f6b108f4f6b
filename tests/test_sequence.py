"""The reference's test sequence (test.py:13-51): 93 cases at 800x512, each
rendered through the engine and checked against the oracle with the same
bit-exact and colour comparisons as the parity suite; plus the headless image
dump (main.cpp:884-896) as PNG."""
import os

import numpy as np
import pytest

import parity_util as pu
from vk_order_independent_transparency_gb300 import sequence as sq

W, H = 800, 512
CASES = sq.cases()
NAMES = [n for n, _ in CASES]


def test_case_list():
    assert len(CASES) == 9 + 7 * 2 * 6
    assert len(set(NAMES)) == len(NAMES)
    assert NAMES[:9] == ['init', 'interlock_unordered', 'opaque', 'opaque_msaa4', 'opaque_ssaa4', '3objects',
                         'lowsubdiv', 'scaleMin', 'scaleWidth']
    st = dict(CASES)
    assert st['init'] == sq.State()
    assert (st['init'].algorithm, st['init'].oitLayers, st['init'].linkedListAllocatedPerElement,
            st['init'].numObjects, st['init'].subdiv) == (4, 8, 10, 1024, 16)
    assert st['interlock_unordered'].interlockIsOrdered == 0 and st['interlock_unordered'].algorithm == 5
    assert st['opaque_ssaa4'].percentTransparent == 0 and st['opaque_ssaa4'].aaType == 2
    assert st['loop64_notail_msaa8'] == sq.State(algorithm=3, tailBlend=0, aaType=4)
    assert st['weighted_tail_ssaa8'] == sq.State(algorithm=6, tailBlend=1, aaType=5)


def test_scene_parameters():
    st = sq.State(numObjects=64)
    v, i, tpo = sq.scene(st)
    assert tpo == 2 * 16 * (2 * 16 - 2)
    pos = v[:, :3].reshape(64, -1, 3)
    centre = pos.mean(axis=1)
    radius = np.linalg.norm(pos - centre[:, None], axis=2).max(axis=1)
    base = 8.0 * 0.9 / 16.0
    assert (radius >= base * 0.1 * 0.999).all() and (radius <= base * 1.0 * 1.001).all()
    assert (np.abs(centre) <= 4.0).all()
    rgb = v[:, 6:9]
    raw = sq.make_scene(64, seed=3625, radius_min=base * 0.1, radius_max=base, half_extent=4.0)[0][:, 6:9]
    np.testing.assert_array_equal(rgb, raw * raw)


def test_png_round_trip(tmp_path):
    img = np.random.default_rng(5).integers(0, 256, (37, 53, 4), dtype=np.uint8)
    path = os.path.join(str(tmp_path), 'x.png')
    sq.write_png(path, img)
    np.testing.assert_array_equal(sq.read_png(path), img)


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_case_parity(name):
    st = dict(CASES)[name]
    v, i, tpo = sq.scene(st)
    sd = sq.camera(W, H)
    kw = sq.state_kwargs(st)
    g = pu.render_gpu(st.algorithm, W, H, v, i, tpo, sd, st.percentTransparent, **kw)
    o = pu.render_oracle(st.algorithm, W, H, v, i, tpo, sd, st.percentTransparent, **kw)
    ss = sq.aa_settings(st.aaType)[2]
    pu.check_pair(st.algorithm, g, o, W, H, st.oitLayers, st.aaType, ss)
    g['renderer'].close()


@pytest.mark.gpu
def test_sequence_dump(tmp_path):
    out = str(tmp_path)
    sq.main(['--out', out, '--width', '160', '--height', '96'])
    assert sorted(os.listdir(out)) == sorted(n + '.png' for n in NAMES)
    st = dict(CASES)['loop64_tail_msaa4']
    np.testing.assert_array_equal(sq.read_png(os.path.join(out, 'loop64_tail_msaa4.png')),
                                  sq.render_case(st, 160, 96))
