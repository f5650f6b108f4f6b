"""A frame whose (tile, triangle) pairs outgrow the bins sized on earlier
frames is still rendered completely.

Bins are sized from the pair counts of earlier frames, so a replayed CUDA
graph can meet more pairs than its bins hold (the scene grew behind the same
mesh pointer, or the camera moved closer). The reference never loses a
triangle (the hardware rasteriser has no bins). Here the pairs of the first
triangles fill the bins, the raster walks the tile lists for those and tests
every later triangle by its bbox, so the image and A-buffer equal those of a
frame rendered with bins large enough; OIT_DEVERR_BIN_OVERFLOW reports the
slow frame, and the next call re-sizes the bins (and re-captures the graph).
"""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

W, H = 192, 144


def scenes(oit):
    small = oit.make_scene(200, seed=9, radius_min=0.01, radius_max=0.02)
    big = oit.make_scene(200, seed=9, radius_min=0.2, radius_max=0.35)
    assert small[1].shape == big[1].shape and small[2] == big[2]
    return small, big


def same(alg, got, ref, L):
    np.testing.assert_array_equal(got['image'], ref['image'])
    np.testing.assert_array_equal(got['color'], ref['color'])
    assert got['fragments'] == ref['fragments']
    if alg != 6:
        pu.compare_abuffer(alg, got, ref, L, W * H, False)


@pytest.mark.parametrize('alg', [1, 3, 5, 6])
def test_grown_scene_is_complete_on_the_first_replay(engine, alg):
    import torch
    L = 8
    (vs, i, tpo), (vb, _, _) = scenes(engine)
    sd = engine.make_camera(W, H)
    kw = dict(oit_layers=L, nodes_per_pixel=64, weighted_precision=engine.OIT_WEIGHTED_FP32)
    ref_small = pu.render_gpu(alg, W, H, vs, i, tpo, sd, 70, **kw)
    ref_big = pu.render_gpu(alg, W, H, vb, i, tpo, sd, 70, **kw)
    r = engine.Renderer(engine.make_state(alg, W, H, flags=engine.OIT_FLAG_CUDA_GRAPH, **kw))
    mesh = engine.DeviceMesh(vs, i)
    r.update_scene(sd)
    for _ in range(2):  # plain frame + capture, then a replay with bins for the small scene
        r.render_frame(mesh, tpo, 70)
    got = pu.collect(r, alg, **kw)
    assert got['error'] == 0
    same(alg, got, ref_small, L)
    mesh.vertices.copy_(torch.from_numpy(vb))  # the scene grows behind the same pointer
    r.render_frame(mesh, tpo, 70)  # replay: the bins overflow
    got = pu.collect(r, alg, **kw)
    assert got['error'] == engine.OIT_DEVERR_BIN_OVERFLOW
    same(alg, got, ref_big, L)
    for _ in range(2):  # re-sized bins, a new graph, then its replay
        r.render_frame(mesh, tpo, 70)
        got = pu.collect(r, alg, **kw)
        assert got['error'] == 0
        same(alg, got, ref_big, L)


@pytest.mark.parametrize('raster_mode', [0, 1])
def test_grown_scene_in_a_batch(engine, raster_mode):
    import torch
    (vs, i, tpo), (vb, _, _) = scenes(engine)
    specs = [(1, 8), (3, 16), (0, 4)]
    views, refs = [], []
    for alg, L in specs:
        sd = engine.make_camera(W, H)
        refs.append(pu.render_gpu(alg, W, H, vb, i, tpo, sd, 100, oit_layers=L, nodes_per_pixel=64)['image'])
        r = engine.Renderer(engine.make_state(alg, W, H, oit_layers=L, nodes_per_pixel=64))
        r.update_scene(sd)
        views.append((r, engine.DeviceMesh(vs, i), tpo, 100))
    batch = engine.Batch(parallel_streams=2)
    batch.set_raster_mode(raster_mode)
    batch.set_views(views)
    for _ in range(2):
        batch.render()
    for _, m, _, _ in views:
        m.vertices.copy_(torch.from_numpy(vb))
    for k in range(2):
        batch.render()
        for (r, *_), ref in zip(views, refs):
            np.testing.assert_array_equal(r.output(), ref)
            assert r.get_error() == (engine.OIT_DEVERR_BIN_OVERFLOW if k == 0 else 0)
