"""The batched resolve (oit_batch_resolve, and oit_batch_render's resolve):
every view's image must equal the one its own composite launch gives (the
same FP32 operations in the same order), and the oracle's within 1 LSB."""
import ctypes

import numpy as np
import pytest

import parity_util as pu
import vk_order_independent_transparency_gb300 as oit

pytestmark = pytest.mark.gpu

# (algorithm, width, height, layers, objects, tail, aa, record format); sizes
# that are not multiples of the 8x4 micro-tile exercise partial micro-tiles
SPECS = [
    (oit.OIT_LINKEDLIST, 97, 61, 1, 30, True, 0, 0),
    (oit.OIT_LINKEDLIST, 128, 96, 2, 40, False, 0, 0),
    (oit.OIT_LINKEDLIST, 75, 133, 4, 60, True, 0, 0),
    (oit.OIT_LINKEDLIST, 160, 120, 8, 80, True, 0, 0),
    (oit.OIT_LINKEDLIST, 64, 64, 16, 90, False, 0, 0),
    (oit.OIT_LINKEDLIST, 150, 100, 32, 120, True, 0, 0),
    (oit.OIT_LOOP64, 99, 77, 1, 30, True, 0, 0),
    (oit.OIT_LOOP64, 128, 128, 4, 70, False, 0, 0),
    (oit.OIT_LOOP64, 141, 90, 8, 80, True, 0, 0),
    (oit.OIT_LOOP64, 200, 136, 16, 100, True, 0, 0),
    # resolved by their own composite launches inside the batch
    (oit.OIT_LINKEDLIST, 96, 80, 8, 40, True, 0, oit.OIT_RECORD_RGBA32F),
    (oit.OIT_INTERLOCK, 96, 72, 8, 40, True, oit.OIT_AA_MSAA_4X, 0),
    (oit.OIT_LOOP64, 64, 48, 8, 30, True, oit.OIT_AA_SUPER_4X, 0),
]


def _views(specs, seed0, dup=False):
    views, refs, scenes = [], [], []
    for k, (alg, W, H, L, n, tail, aa, fmt) in enumerate(specs):
        v, i, tpo, sd = pu.scene(n, W, H, seed=seed0 + k, radius_min=0.08, radius_max=0.3)
        if dup:
            # every object twice: each fragment has an equal-depth twin
            i = np.concatenate([i, i])
        kw = dict(oit_layers=L, nodes_per_pixel=12, tail_blend=tail, aa_type=aa, record_format=fmt)
        g = pu.render_gpu(alg, W, H, v, i, tpo, sd, 100, **kw)
        refs.append(g['image'])
        g['renderer'].close()
        r = oit.Renderer(oit.make_state(alg, W, H, **kw))
        r.update_scene(sd)
        views.append((r, oit.DeviceMesh(v, i), tpo, 100))
        scenes.append((v, i, tpo, sd, kw))
    return views, refs, scenes


@pytest.mark.parametrize('raster_mode', [0, 1])
def test_batch_render_and_resolve_match_single_frames(raster_mode):
    views, refs, _ = _views(SPECS, 300)
    batch = oit.Batch(parallel_streams=4)
    batch.set_raster_mode(raster_mode)
    batch.set_views(views)
    for _ in range(3):  # plain frames + autotune + capture, then replays
        batch.render()
        for (r, _, _, _), ref in zip(views, refs):
            np.testing.assert_array_equal(r.output(), ref)
            assert r.get_error() == 0
    cfg = batch.resolve_config()
    for part in ('linkedlist', 'loop64'):
        assert cfg[part]['threads_per_block'] in (64, 128, 256) and cfg[part]['blocks'] >= 1
    assert cfg['linkedlist']['shared_slots'] in (0, 8) and cfg['loop64']['shared_slots'] == 0
    assert cfg['linkedlist']['register_slots'] in (0, 4, 8) and cfg['loop64']['register_slots'] == 0
    assert cfg['loop64']['items_per_step'] in (1, 2) and cfg['loop64']['dense'] in (0, 1)
    assert cfg['loop64']['items_per_step'] == 1 or not cfg['loop64']['dense']
    # resolve alone, after clearing the outputs
    import torch
    for r, _, _, _ in views:
        ptr, nb = r.buffer(oit.OIT_BUF_OUTPUT)
        oit._cudart().cudaMemset(ctypes.c_void_p(ptr), 0, ctypes.c_size_t(nb))
    torch.cuda.synchronize()
    batch.resolve()
    for (r, _, _, _), ref in zip(views, refs):
        np.testing.assert_array_equal(r.output(), ref)


@pytest.mark.parametrize('L', [2, 4, 16])
def test_batch_resolve_equal_depths(L):
    """Equal depths make bubbleSort's order depend on its passes: the batched
    resolve must reproduce it (kept entries) and insertionSortTail's (tail)."""
    specs = [(oit.OIT_LINKEDLIST, 96, 80, L, 30, True, 0, 0), (oit.OIT_LINKEDLIST, 64, 56, L, 20, False, 0, 0),
             (oit.OIT_LOOP64, 80, 64, L, 25, True, 0, 0)]
    views, refs, scenes = _views(specs, 500 + L, dup=True)
    batch = oit.Batch(parallel_streams=2)
    batch.set_views(views)
    batch.render()
    batch.render()
    for (r, _, _, _), ref, (v, i, tpo, sd, kw), spec in zip(views, refs, scenes, specs):
        img = r.output()
        np.testing.assert_array_equal(img, ref)
        W, H = spec[1], spec[2]
        o = pu.render_oracle(spec[0], W, H, v, i, tpo, sd, 100, **kw)
        pu.compare_images({'image': img}, o)


def test_batch_resolve_before_render_is_a_state_error():
    r = oit.Renderer(oit.make_state(oit.OIT_LOOP64, 64, 64, oit_layers=4))
    v, i, tpo, sd = pu.scene(4, 64, 64)
    r.update_scene(sd)
    batch = oit.Batch()
    batch.set_views([(r, oit.DeviceMesh(v, i), tpo, 100)])
    with pytest.raises(oit.OitError) as e:
        batch.resolve()
    assert e.value.status == oit.OIT_ERR_STATE
    with pytest.raises(oit.OitError):
        batch.resolve_config()


# every kernel the autotuner chooses from, pinned: (part, shape)
PINNED = [
    ('linkedlist', dict(threads_per_block=128)),
    ('linkedlist', dict(threads_per_block=256, dense=1)),
    ('linkedlist', dict(threads_per_block=64, shared_slots=8)),
    ('linkedlist', dict(threads_per_block=128, items_per_step=2)),
    ('linkedlist', dict(threads_per_block=64, register_slots=4)),
    ('linkedlist', dict(threads_per_block=128, register_slots=8)),
    ('linkedlist', dict(threads_per_block=256, register_slots=8, dense=1)),
    ('linkedlist', dict(threads_per_block=256, dense=1, bin_edges=1)),
    ('loop64', dict(threads_per_block=256)),
    ('loop64', dict(threads_per_block=128, bin_edges=1)),
    ('loop64', dict(threads_per_block=128, items_per_step=2)),
    ('loop64', dict(threads_per_block=256, dense=1)),
]


@pytest.mark.parametrize('order', [0, 1])
@pytest.mark.parametrize('binned', [0, 1])
def test_every_pinned_resolve_shape(binned, order):
    """Each resolve kernel, in both work orders, binned or not, pinned
    through oit_batch_set_resolve_config, gives every view the image its own
    composite launch gives."""
    import torch
    views, refs, _ = _views(SPECS, 700)
    batch = oit.Batch(parallel_streams=4)
    batch.set_views(views)
    batch.render()
    for part, shape in PINNED:
        batch.set_resolve_config(part, dict(shape, binned=binned, tile_order=order, blocks=37))
        for r, _, _, _ in views:
            ptr, nb = r.buffer(oit.OIT_BUF_OUTPUT)
            oit._cudart().cudaMemset(ctypes.c_void_p(ptr), 0, ctypes.c_size_t(nb))
        torch.cuda.synchronize()
        batch.resolve()
        got = batch.resolve_config()[part]
        for f, v in shape.items():
            if f != 'bin_edges':  # reported for binned work lists only (checked below)
                assert got[f] == v, (part, shape, got)
        assert got['binned'] == bool(binned) and got['tile_order'] == bool(order)
        assert got['bin_edges'] == (shape.get('bin_edges', 0) if binned else 0)
        for k, ((r, _, _, _), ref) in enumerate(zip(views, refs)):
            np.testing.assert_array_equal(r.output(), ref, err_msg='%s %s view %d' % (part, shape, k))
        batch.set_resolve_config(part, None)
    # pinned, the graph replays it too
    batch.set_resolve_config('linkedlist', dict(threads_per_block=64, register_slots=8, blocks=0))
    for _ in range(3):
        batch.render()
    assert batch.resolve_config()['linkedlist']['register_slots'] == 8
    for (r, _, _, _), ref in zip(views, refs):
        np.testing.assert_array_equal(r.output(), ref)


def test_pinned_shape_validation():
    batch = oit.Batch()
    bad = [('loop64', dict(threads_per_block=128, shared_slots=8)), ('loop64', dict(threads_per_block=128,
                                                                                    register_slots=4)),
           ('loop64', dict(threads_per_block=128, items_per_step=2, dense=1)),
           ('linkedlist', dict(threads_per_block=128, shared_slots=8, register_slots=8)),
           ('linkedlist', dict(threads_per_block=128, register_slots=4, dense=1)),
           ('linkedlist', dict(threads_per_block=128, items_per_step=3)),
           ('linkedlist', dict(threads_per_block=48)), ('linkedlist', dict(threads_per_block=512)),
           ('linkedlist', dict(threads_per_block=128, shared_slots=4)),
           ('linkedlist', dict(threads_per_block=128, bin_edges=2))]
    for part, shape in bad:
        with pytest.raises(oit.OitError) as e:
            batch.set_resolve_config(part, shape)
        assert e.value.status == oit.OIT_ERR_INVALID_ARGUMENT
    batch.set_resolve_config('linkedlist', dict(threads_per_block=128))
    batch.set_resolve_config('linkedlist', None)



def test_raster_config_validation():
    batch = oit.Batch()
    for cfg in ({'multi_view': 2}, {'warps_per_sm': 40}, {'multi_view': 1, 'warps_per_sm': 32}, {'lane_order': 2},
                {'lane_order': -1}):
        with pytest.raises(oit.OitError) as e:
            batch.set_raster_config(cfg)
        assert e.value.status == oit.OIT_ERR_INVALID_ARGUMENT
    with pytest.raises(oit.OitError) as e:
        batch.raster_config()  # nothing captured yet
    assert e.value.status == oit.OIT_ERR_STATE
    batch.set_raster_config({'multi_view': 0, 'warps_per_sm': 32})
    batch.set_raster_config({'multi_view': 0, 'lane_order': 1})
    batch.set_raster_config(None)
