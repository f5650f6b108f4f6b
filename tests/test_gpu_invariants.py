"""Invariants of the engine's own A-buffers at full size, checked on the
host (the race and bounds checks a sanitizer would give, restated as facts
every correct frame satisfies): linked lists are acyclic and disjoint and hold
min(fragments, capacity - 1) nodes, counted by the counter; Loop64 k-buffers
are sorted with empty keys only at the end; Simple keeps min(count, L)."""
import numpy as np
import pytest

import vk_order_independent_transparency_gb300 as oit

pytestmark = pytest.mark.gpu
W, H = 1920, 1080


def _frame(alg, **kw):
    v, i, tpo = oit.make_scene(1024, seed=2, radius_min=0.03, radius_max=0.1)
    with oit.Renderer(oit.make_state(alg, W, H, **kw)) as r:
        r.update_scene(oit.make_camera(W, H))
        r.render_frame(oit.DeviceMesh(v, i), tpo, 100)
        assert r.get_error() == 0
        return {'abuf': r.read_buffer(oit.OIT_BUF_ABUFFER), 'aux': r.read_buffer(oit.OIT_BUF_AUX),
                'counter': r.read_buffer(oit.OIT_BUF_COUNTER), 'frags': r.fragment_count()}


@pytest.mark.parametrize('npp', [1, 2, 8])
def test_linked_lists_acyclic_disjoint_counted(npp):
    g = _frame(oit.OIT_LINKEDLIST, oit_layers=8, nodes_per_pixel=npp)
    cap = npp * W * H
    pool = g['abuf'].reshape(-1, 4).astype(np.int64)
    assert pool.shape[0] == cap
    assert int(g['counter'][0]) == g['frags']  # the counter counts overflowed fragments too
    nxt = pool[:, 3]
    cur = g['aux'].astype(np.int64)
    assert ((cur >= 0) & (cur < cap)).all()
    seen = np.zeros(cap, np.int64)
    steps = 0
    while (cur != 0).any():
        live = cur[cur != 0]
        np.add.at(seen, live, 1)
        cur = np.where(cur != 0, nxt[cur], 0)
        assert ((cur >= 0) & (cur < cap)).all()
        steps += 1
        assert steps <= cap  # a cycle would never end
    assert seen[0] == 0 and seen.max() <= 1  # every node in at most one list, once
    assert int(seen.sum()) == min(g['frags'], cap - 1)


def test_loop64_kbuffers_sorted():
    L = 16
    g = _frame(oit.OIT_LOOP64, oit_layers=L)
    keys = g['abuf'].view(np.uint64).reshape(L, W * H)
    empty = keys == np.uint64(0xFFFFFFFFFFFFFFFF)
    assert (keys[1:] >= keys[:-1]).all()  # ascending, so the empty keys close each list
    n = (~empty).sum(0)
    assert not (empty[:-1] & ~empty[1:]).any()
    assert n.max() == L and int(n.sum()) <= g['frags']


def test_simple_keeps_first_l():
    L = 8
    g = _frame(oit.OIT_SIMPLE, oit_layers=L)
    aux = g['aux'].astype(np.int64)
    assert int(aux.sum()) == g['frags']
    rec = g['abuf'].reshape(L, W * H, 2)
    depth_set = rec[:, :, 1] != 0
    stored = np.minimum(aux, L)
    assert (depth_set.sum(0) <= stored).all()  # nothing past the pixel's count is written
