"""The arrival-order linked-list COLOR pass (OIT_FLAG_ARRIVAL_ORDER).

The reference's GPU runs the linked-list fragment shader for all fragments in
parallel: list order is arrival order, and a fragment that finds the pool full
is blended into the colour target in arrival order. The engine's arrival mode
does the same with HBM atomics (node counter, head exchange) and per-pixel
spinlocks, so its lists are not reproducible node for node. What is checked:
every pixel's list holds exactly the fragments the oracle's primitive-order
list holds (as a multiset; all of them when the pool does not overflow, the
counter counting every fragment), and the image equals the oracle's composite
of the GPU's own lists (and, on overflow, of the GPU's own tail-blended colour
target) within 1 LSB -- the oracle run on the GPU's capture order. With lists
no longer than OIT_LAYERS and no pool overflow the image also equals the
primitive-order one within 1 LSB.
"""
import numpy as np
import pytest

import oracle as orc
import parity_util as pu

pytestmark = pytest.mark.gpu


def arrival_kw(**kw):
    import vk_order_independent_transparency_gb300 as oit
    return dict(kw, flags=kw.get('flags', 0) | oit.OIT_FLAG_ARRIVAL_ORDER)


def list_sets(g, o, P):
    gl = pu.walk_lists(g['abuf'], g['aux'][:P])
    ol = pu.walk_lists(o['abuf'], o['aux'][:P])
    return gl, ol


def replay_image(g, W, H, L, npp, aa=0, tail=True):
    """The oracle's composite of the GPU's pool, heads, counter and colour
    target (opaque colour or background, plus any tail blends): the
    reference's composite on the GPU's arrival order."""
    fr = orc.Frame(orc.LINKEDLIST, W, H, oit_layers=L, nodes_per_pixel=npp, aa_type=aa, tail_blend=tail)
    fr.begin()
    fr.clear_transparent()
    fr.load_state(g['abuf'], g['aux'], g['counter'])
    fr.load_color(g['color'].astype(np.float64))
    img, _ = fr.composite()
    return img


@pytest.mark.parametrize('aa,percent,L', [(0, 100, 32), (0, 60, 8), (3, 100, 16), (0, 100, 4)])
def test_arrival_lists_hold_the_oracle_fragments(engine, aa, percent, L):
    W, H, npp = 128, 96, 64
    v, i, tpo, sd = pu.scene(48, W, H, seed=31, radius_min=0.05, radius_max=0.2)
    kw = dict(oit_layers=L, nodes_per_pixel=npp, aa_type=aa)
    g = pu.render_gpu(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, percent, **arrival_kw(**kw))
    o = pu.render_oracle(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, percent, **kw)
    ss = 2 if aa == 3 else 1
    P = W * H * ss * ss
    assert g['error'] == 0
    assert g['fragments'] == o['fragments'] == int(g['counter'][0]) == int(o['counter'][0])
    if percent < 100:
        np.testing.assert_array_equal(g['depth'][:P], o['depth'][:P])
    gl, ol = list_sets(g, o, P)
    longest = 0
    for a, b in zip(gl, ol):
        assert sorted(a) == sorted(b)
        longest = max(longest, len(b))
    d = np.abs(g['image'].astype(np.int32) - replay_image(g, W, H, L, npp, aa).astype(np.int32))
    assert d.max() <= 1
    if longest <= L:
        pu.compare_images(g, o)


def test_arrival_pool_overflow(engine):
    """A pool of one node per pixel: the stored nodes are a subset of each
    pixel's fragments, the counter still counts them all, and the rest were
    tail-blended in arrival order under the pixel locks (no lock gave up)."""
    W, H, L, npp = 128, 96, 4, 1
    v, i, tpo, sd = pu.scene(48, W, H, seed=9, radius_min=0.1, radius_max=0.25)
    g = pu.render_gpu(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, 100,
                      **arrival_kw(oit_layers=L, nodes_per_pixel=npp))
    full = pu.render_oracle(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, 100, oit_layers=L, nodes_per_pixel=64)
    P = W * H
    assert g['error'] == 0
    assert g['fragments'] > P and int(g['counter'][0]) == g['fragments'] == full['fragments']
    gl, ol = list_sets(g, full, P)
    stored = 0
    for a, b in zip(gl, ol):
        rest = list(b)
        for e in a:
            rest.remove(e)  # each stored node is one of the pixel's fragments
        stored += len(a)
    assert stored == P - 1  # nodes 1 .. P-1
    d = np.abs(g['image'].astype(np.int32) - replay_image(g, W, H, L, npp).astype(np.int32))
    assert d.max() <= 1


def test_arrival_lock_wait_times_out(engine):
    """A tail-blend lock that nothing releases (held from the start of the
    pass by the testing hook): the fragments that must blend at that pixel
    give up after their bounded spin, the frame reports OIT_DEVERR_TIMEOUT
    instead of hanging, the rest of the frame equals the oracle's composite of
    the GPU's own lists and colour target, and the next frame, with the lock
    released, renders without an error."""
    W, H, L, npp = 96, 72, 4, 1  # 2.8 fragments per pixel: about two thirds tail-blend
    v, i, tpo, sd = pu.scene(64, W, H, seed=9, radius_min=0.15, radius_max=0.3)
    P = W * H
    r = engine.Renderer(engine.make_state(engine.OIT_LINKEDLIST, W, H,
                                          **arrival_kw(oit_layers=L, nodes_per_pixel=npp)))
    mesh = engine.DeviceMesh(v, i)
    r.update_scene(sd)
    r.render_frame(mesh, tpo, 100)
    g = pu.collect(r, engine.OIT_LINKEDLIST)
    assert g['error'] == 0
    full = pu.render_oracle(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, 100, oit_layers=L, nodes_per_pixel=64)
    gl, ol = list_sets(g, full, P)
    # a pixel that lost 3 to 5 fragments to tail blending: its tail fragments
    # meet the held lock on the next frame too, and only a few wait there
    lost = np.array([len(b) - len(a) for a, b in zip(gl, ol)])
    some = np.nonzero((lost >= 3) & (lost <= 5))[0]
    px = int(some[0]) if some.size else int(np.argmax(lost))
    assert lost[px] >= 3
    r.debug_hold_arrival_lock(px)
    r.render_frame(mesh, tpo, 100)
    g = pu.collect(r, engine.OIT_LINKEDLIST)
    assert g['error'] & engine.OIT_DEVERR_TIMEOUT
    d = np.abs(g['image'].astype(np.int32) - replay_image(g, W, H, L, npp).astype(np.int32))
    assert d.max() <= 1
    r.debug_hold_arrival_lock(-1)
    r.render_frame(mesh, tpo, 100)
    g = pu.collect(r, engine.OIT_LINKEDLIST)
    assert g['error'] == 0
    with pytest.raises(engine.OitError):
        r.debug_hold_arrival_lock(P)


def test_arrival_unsupported_states(engine):
    import ctypes
    for alg, aa, fmt in ((engine.OIT_LOOP64, 0, 0), (engine.OIT_SIMPLE, 0, 0), (engine.OIT_LINKEDLIST, 1, 0),
                         (engine.OIT_LINKEDLIST, 2, 0), (engine.OIT_LINKEDLIST, 0, engine.OIT_RECORD_RGBA32F)):
        st = engine.make_state(alg, 64, 64, aa_type=aa, record_format=fmt, flags=engine.OIT_FLAG_ARRIVAL_ORDER)
        ctx = ctypes.c_void_p()
        assert engine.library().oit_create(ctypes.byref(st), ctypes.byref(ctx)) == engine.OIT_ERR_UNSUPPORTED


def test_arrival_graph_replay_and_batch(engine):
    """Arrival-order frames replayed from a CUDA graph and rendered in a batch
    beside primitive-order views: lists of at most OIT_LAYERS nodes, so each
    image equals the primitive-order frame's within 1 LSB."""
    W, H, L = 160, 120, 32
    v, i, tpo, sd = pu.scene(40, W, H, seed=12, radius_min=0.05, radius_max=0.2)
    ref = pu.render_gpu(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, 100, oit_layers=L, nodes_per_pixel=32)
    r = engine.Renderer(engine.make_state(engine.OIT_LINKEDLIST, W, H, oit_layers=L, nodes_per_pixel=32,
                                          flags=engine.OIT_FLAG_ARRIVAL_ORDER | engine.OIT_FLAG_CUDA_GRAPH))
    mesh = engine.DeviceMesh(v, i)
    r.update_scene(sd)
    for _ in range(3):
        r.render_frame(mesh, tpo, 100)
        g = pu.collect(r, engine.OIT_LINKEDLIST)
        assert g['error'] == 0 and g['fragments'] == ref['fragments']
        pu.compare_images(g, ref)
    other = engine.Renderer(engine.make_state(engine.OIT_LOOP64, W, H, oit_layers=8))
    other.update_scene(sd)
    ref64 = pu.render_gpu(engine.OIT_LOOP64, W, H, v, i, tpo, sd, 100, oit_layers=8)['image']
    r2 = engine.Renderer(engine.make_state(engine.OIT_LINKEDLIST, W, H, oit_layers=L, nodes_per_pixel=32,
                                           flags=engine.OIT_FLAG_ARRIVAL_ORDER | engine.OIT_FLAG_HALF_COLOR))
    r2.update_scene(sd)
    for cfg in ({'multi_view': 0}, {'multi_view': 1}):
        batch = engine.Batch(parallel_streams=2)
        batch.set_raster_config(cfg)
        batch.set_views([(r2, mesh, tpo, 100), (other, mesh, tpo, 100)])
        for _ in range(3):
            batch.render()
            pu.compare_images({'image': r2.output()}, ref)
            np.testing.assert_array_equal(other.output(), ref64)
            assert r2.get_error() == 0
