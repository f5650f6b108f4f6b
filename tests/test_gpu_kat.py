"""The reference README's traces (README.md:45, 53-66, 72, 80, 86-96) on the
GPU: four viewport-covering quads at depths 0.4, 0.2, 0.1, 0.3 (fragments
c4, c2, c1, c3), drawn in the trace's arrival order with identity matrices
(clip space = the scene), OIT_LAYERS = 2. The fragments are told apart by
depth (their colour is shaded); every A-buffer also equals the oracle's on
the same mesh, and the image is within 1 LSB of it."""
import numpy as np
import pytest

import parity_util as pu
import vk_order_independent_transparency_gb300 as oit

pytestmark = pytest.mark.gpu

Z = {1: 0.1, 2: 0.2, 3: 0.3, 4: 0.4}
COL = {1: (0.80, 0.10, 0.10, 0.50), 2: (0.10, 0.70, 0.20, 0.40), 3: (0.20, 0.30, 0.90, 0.60),
       4: (0.60, 0.60, 0.05, 0.30)}


def zbits(k):
    return int(np.float32(Z[k]).view(np.uint32))


def quads(seq, xs=None):
    """Fragment k of `seq` as a quad over NDC x in xs[j] (default the whole
    viewport), all y, at depth Z[k], normal +z, colour COL[k]; two triangles
    per quad, so an 'object' is one quad."""
    v, idx = [], []
    for j, k in enumerate(seq):
        x0, x1 = xs[j] if xs else (-1.0, 1.0)
        base = len(v)
        for x, y in ((x0, -1.0), (x1, -1.0), (x1, 1.0), (x0, 1.0)):
            v.append([x, y, Z[k], 0.0, 0.0, 1.0, *COL[k]])
        idx += [[base, base + 1, base + 2], [base, base + 2, base + 3]]
    return np.array(v, np.float32), np.array(idx, np.uint32)


def identity_scene():
    sd = oit.OitSceneData()
    for j in range(4):
        sd.proj_view_matrix[5 * j] = 1.0
        sd.view_matrix[5 * j] = 1.0
    return sd


def run(alg, W, H, seq, xs=None, **kw):
    v, i = quads(seq, xs)
    sd = identity_scene()
    kw = dict(dict(oit_layers=2, nodes_per_pixel=8), **kw)
    g = pu.render_gpu(alg, W, H, v, i, 2, sd, 100, **kw)
    o = pu.render_oracle(alg, W, H, v, i, 2, sd, 100, **kw)
    assert g['error'] == 0
    # a quad covers every pixel, or (xs) one pixel
    assert g['fragments'] == o['fragments'] == len(seq) * (1 if xs else W * H)
    return g, o


def same_state(g, o, keys):
    for k in keys:
        np.testing.assert_array_equal(g[k], o[k], err_msg=k)
    pu.compare_images(g, o)


def test_simple_first_k():
    """README.md:45: the first two arrivals (c4, c2) are stored; c1, c3 tail blended."""
    g, o = run(oit.OIT_SIMPLE, 1, 1, [4, 2, 1, 3])
    rec = g['abuf'].reshape(-1, 2)  # {rgba8, depth} per layer (P = 1)
    assert [int(rec[0, 1]), int(rec[1, 1])] == [zbits(4), zbits(2)]
    assert int(g['aux'][0]) == 4
    same_state(g, o, ('abuf', 'aux'))


def test_linked_list_pool():
    """README.md:53-66: two pixels, a 4-node pool (nodes 1..3 usable), arrivals
    c4 -> pixel 0, c1 -> pixel 1, c2 -> pixel 0, c3 -> pixel 0 (overflows)."""
    xs = [(-1.0, 0.0), (0.0, 1.0), (-1.0, 0.0), (-1.0, 0.0)]
    g, o = run(oit.OIT_LINKEDLIST, 2, 1, [4, 1, 2, 3], xs, nodes_per_pixel=2)
    pool = g['abuf'].reshape(-1, 4)  # {rgba8, depth, mask, next}
    assert [int(x) for x in pool[1, 1:]] == [zbits(4), 0, 0]
    assert [int(x) for x in pool[2, 1:]] == [zbits(1), 0, 0]
    assert [int(x) for x in pool[3, 1:]] == [zbits(2), 0, 1]
    assert [int(x) for x in g['aux'][:2]] == [3, 2]
    assert int(g['counter'][0]) == 4  # the overflowed fragment is counted too
    same_state(g, o, ('abuf', 'aux', 'counter'))


def test_loop32():
    """README.md:72: depths 0.1 and 0.2 kept in order; c4 and c3 tail blended."""
    g, o = run(oit.OIT_LOOP, 1, 1, [4, 2, 1, 3])
    assert [int(x) for x in g['abuf'][:2]] == [zbits(1), zbits(2)]
    same_state(g, o, ('abuf',))


def test_loop64():
    """README.md:80: keys (0.1, c1), (0.2, c2) kept in order; c4 then c3 tail blended."""
    g, o = run(oit.OIT_LOOP64, 1, 1, [4, 2, 1, 3])
    keys = g['abuf'].view(np.uint64)
    assert [int(k) >> 32 for k in keys[:2]] == [zbits(1), zbits(2)]
    same_state(g, o, ('abuf',))


@pytest.mark.parametrize('alg', [oit.OIT_SPINLOCK, oit.OIT_INTERLOCK])
def test_spinlock_trace(alg):
    """README.md:86-96: critical sections in the order c3, c2, c4, c1: c1 and c2
    end up stored, the furthest evicted depth is 0.3, four fragments counted."""
    g, o = run(alg, 1, 1, [3, 2, 4, 1])
    rec = g['abuf'].reshape(-1, 2)
    assert sorted([int(rec[0, 1]), int(rec[1, 1])]) == [zbits(1), zbits(2)]
    assert int(g['auxdepth'][0]) == zbits(3)
    assert int(g['aux'][0]) == 4
    same_state(g, o, ('abuf', 'aux', 'auxdepth'))
