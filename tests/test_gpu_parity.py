"""GPU parity: the CUDA engine against the CPU oracle on the same seeded scenes.

Bit-exact: fragment counts, every algorithm's A-buffer state (Simple /
Spinlock / Interlock records and counters, linked lists in list order, Loop32
depth and colour layers, Loop64 keys), the opaque depth buffer.
Colour: the RGBA8 image within 1 LSB (GPU blends in FP32, the oracle in
FP64); the tail-blended colour target within 2e-5 absolute.
"""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

ALGS = [0, 1, 2, 3, 4, 5, 6]
AA = {'1x': 0, 'msaa4': 1, 'msaa8': 4, 'ssaa4': 2, 'ssaa8': 5}


def run_pair(engine, alg, W, H, n_obj, percent=100, seed=3, rmin=0.05, rmax=0.2, **kw):
    v, i, tpo, sd = pu.scene(n_obj, W, H, seed=seed, radius_min=rmin, radius_max=rmax)
    g = pu.render_gpu(alg, W, H, v, i, tpo, sd, percent, **kw)
    o = pu.render_oracle(alg, W, H, v, i, tpo, sd, percent, **kw)
    return g, o


def check(engine, alg, g, o, W, H, L, aa=0, ss=1, fp32=False):
    pu.check_pair(alg, g, o, W, H, L, aa, ss, fp32)


@pytest.mark.parametrize('tail', [True, False])
@pytest.mark.parametrize('aa', list(AA))
@pytest.mark.parametrize('alg', ALGS)
def test_algorithm(engine, alg, aa, tail):
    W, H, L = 128, 96, 4
    kw = dict(oit_layers=L, nodes_per_pixel=6, aa_type=AA[aa], tail_blend=tail,
              weighted_precision=engine.OIT_WEIGHTED_FP32)
    g, o = run_pair(engine, alg, W, H, 40, **kw)
    check(engine, alg, g, o, W, H, L, AA[aa])


@pytest.mark.parametrize('L', [1, 2, 8, 16, 32])
@pytest.mark.parametrize('alg', [0, 1, 2, 3, 4])
def test_layers(engine, alg, L):
    W, H = 96, 80
    g, o = run_pair(engine, alg, W, H, 48, seed=11, rmin=0.1, rmax=0.3, oit_layers=L, nodes_per_pixel=40)
    check(engine, alg, g, o, W, H, L)


@pytest.mark.parametrize('alg', [0, 1, 2, 3, 4])
def test_layers_sample_shading(engine, alg):
    W, H, L = 64, 48, 16
    g, o = run_pair(engine, alg, W, H, 32, seed=13, rmin=0.1, rmax=0.3, oit_layers=L, nodes_per_pixel=12, aa_type=5)
    check(engine, alg, g, o, W, H, L, aa=5)


@pytest.mark.parametrize('alg', ALGS)
def test_opaque_and_transparent(engine, alg):
    W, H, L = 160, 120, 8
    g, o = run_pair(engine, alg, W, H, 64, percent=60, seed=21, oit_layers=L, nodes_per_pixel=8,
                    weighted_precision=engine.OIT_WEIGHTED_FP32)
    np.testing.assert_array_equal(g['depth'][:W * H], o['depth'][:W * H])
    check(engine, alg, g, o, W, H, L)


@pytest.mark.parametrize('alg', [0, 1, 3, 6])
def test_supersample(engine, alg):
    W, H, L = 64, 48, 4
    g, o = run_pair(engine, alg, W, H, 32, aa_type=3, oit_layers=L, nodes_per_pixel=8,
                    weighted_precision=engine.OIT_WEIGHTED_FP32)
    check(engine, alg, g, o, W, H, L, aa=3, ss=2)


def test_linked_list_overflow(engine):
    """A pool smaller than the fragment count: each pixel keeps a primitive-order
    prefix of its fragments (the counter order decides which); the rest are tail
    blended. The oracle replays the GPU's per-pixel prefix lengths."""
    W, H, L = 128, 96, 4
    v, i, tpo, sd = pu.scene(48, W, H, seed=9, radius_min=0.1, radius_max=0.25)
    g = pu.render_gpu(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, oit_layers=L, nodes_per_pixel=1)
    full = pu.render_oracle(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, oit_layers=L, nodes_per_pixel=64)
    P = W * H
    assert g['fragments'] > P  # the pool (P nodes) overflowed
    assert g['counter'][0] == g['fragments']
    gl = pu.walk_lists(g['abuf'], g['aux'][:P])
    ol = pu.walk_lists(full['abuf'], full['aux'][:P])
    stored = 0
    for a, b in zip(gl, ol):
        # lists are in reverse arrival order: the stored ones are the oldest
        assert a == b[len(b) - len(a):]
        stored += len(a)
    assert stored == P - 1  # nodes 1..P-1 are all used
    import oracle as orc
    fr = orc.Frame(orc.LINKEDLIST, W, H, oit_layers=L, nodes_per_pixel=1)
    fr.set_ll_store_limit(np.array([len(a) for a in gl], np.uint32))
    fr.draw_transparent(sd, v, i, 0, i.shape[0])
    ref8, _ = fr.composite()
    d = np.abs(g['image'].astype(np.int32) - ref8.astype(np.int32))
    assert d.max() <= 1


@pytest.mark.parametrize('prec', [0, 1])
def test_weighted_accumulators(engine, prec):
    """WBOIT accumulation vs FP64, bounds at about twice the values measured on
    a GB300 (deterministic inputs): FP16 (RGBA16F emulation, rounding after
    every blend) accumulation 1.52e-3 relative, revealage 3.1e-3; FP32
    accumulation 4.5e-7, revealage 2.4e-7."""
    W, H = 128, 96
    v, i, tpo, sd = pu.scene(64, W, H, seed=4)
    g = pu.render_gpu(engine.OIT_WEIGHTED, W, H, v, i, tpo, sd, weighted_precision=prec)
    o = pu.render_oracle(engine.OIT_WEIGHTED, W, H, v, i, tpo, sd)
    acc_g, acc_o = g['accum'], o['accum']
    mask = np.abs(acc_o) > 1e-3
    rel = np.abs(acc_g - acc_o)[mask] / np.abs(acc_o)[mask]
    tol, rtol = (1e-6, 5e-7) if prec == 1 else (3e-3, 6.5e-3)
    assert rel.max() < tol, rel.max()
    rrel = np.abs(g['reveal'] - o['reveal']) / np.maximum(o['reveal'], 1e-3)
    assert rrel.max() < rtol, rrel.max()
    if prec == 1:
        pu.compare_images(g, o)


def test_deterministic(engine):
    """Two runs give identical images and A-buffer state (slots the reference
    leaves undefined, e.g. Simple records past each pixel's count, excluded)."""
    W, H = 160, 120
    v, i, tpo, sd = pu.scene(64, W, H, seed=2)
    for alg in ALGS:
        a = pu.render_gpu(alg, W, H, v, i, tpo, sd, oit_layers=8)
        b = pu.render_gpu(alg, W, H, v, i, tpo, sd, oit_layers=8)
        np.testing.assert_array_equal(a['image'], b['image'])
        np.testing.assert_array_equal(a['color'], b['color'])
        if alg != engine.OIT_WEIGHTED:
            pu.compare_abuffer(alg, a, b, 8, W * H, False)


def test_linked_list_640x480(engine):
    """The reference's CPU-runnable workload: Linked List, 640x480, OIT_LAYERS=8,
    8 nodes per pixel, 256 spheres (radii 0.05-0.15), fully transparent."""
    W, H = 640, 480
    v, i, tpo, sd = pu.scene(256, W, H, seed=1, radius_min=0.05, radius_max=0.15)
    g = pu.render_gpu(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, oit_layers=8, nodes_per_pixel=8)
    o = pu.render_oracle(engine.OIT_LINKEDLIST, W, H, v, i, tpo, sd, oit_layers=8, nodes_per_pixel=8)
    check(engine, engine.OIT_LINKEDLIST, g, o, W, H, 8)


@pytest.mark.parametrize('alg', [3, 4])
def test_kbuffer_1080p(engine, alg):
    """Loop64 and Spinlock at 1920x1080, OIT_LAYERS=16, 1024 spheres (radii
    0.03-0.1), 60% transparent over an opaque depth pre-pass, tail blend on."""
    W, H, L = 1920, 1080, 16
    v, i, tpo, sd = pu.scene(1024, W, H, seed=2, radius_min=0.03, radius_max=0.1)
    g = pu.render_gpu(alg, W, H, v, i, tpo, sd, 60, oit_layers=L)
    o = pu.render_oracle(alg, W, H, v, i, tpo, sd, 60, oit_layers=L)
    np.testing.assert_array_equal(g['depth'][:W * H], o['depth'][:W * H])
    check(engine, alg, g, o, W, H, L)


def big_triangle_mesh(seed=5, n=24):
    """Hand-built triangles of every size, some far larger than 64 px and some
    crossing the viewport border (the int64 edge-function path)."""
    rng = np.random.default_rng(seed)
    verts, idx = [], []
    for k in range(n):
        c = rng.uniform(-1.2, 1.2, 3) * [1, 1, 0.6]
        size = [0.05, 0.3, 1.5, 3.0][k % 4]
        col = list(rng.uniform(0, 1, 4))
        for _ in range(3):
            p = c + rng.uniform(-size, size, 3) * [1, 1, 0.2]
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            verts.append(list(p) + list(nrm) + col)
        idx.append([3 * k, 3 * k + 1, 3 * k + 2])
    return np.array(verts, np.float32), np.array(idx, np.uint32)


@pytest.mark.parametrize('aa', [0, 4, 2])
@pytest.mark.parametrize('alg', ALGS)
def test_large_triangles(engine, alg, aa):
    W, H, L = 200, 150, 4
    v, i = big_triangle_mesh()
    sd = engine.make_camera(W, H)
    kw = dict(oit_layers=L, nodes_per_pixel=8, aa_type=aa, weighted_precision=engine.OIT_WEIGHTED_FP32)
    g = pu.render_gpu(alg, W, H, v, i, 1, sd, 100, **kw)
    o = pu.render_oracle(alg, W, H, v, i, 1, sd, 100, **kw)
    check(engine, alg, g, o, W, H, L, aa)
    # opaque half: the first 12 triangles transparent, the rest opaque
    g = pu.render_gpu(alg, W, H, v, i, 1, sd, 50, **kw)
    o = pu.render_oracle(alg, W, H, v, i, 1, sd, 50, **kw)
    np.testing.assert_array_equal(g['depth'], o['depth'])
    check(engine, alg, g, o, W, H, L, aa)


@pytest.mark.parametrize('alg', [1, 3, 4])
def test_separate_draw_calls_match_frame(engine, alg):
    """The reference-style call sequence (begin, clearTransparent, opaque draw,
    drawTransparent COLOR, COMPOSITE) gives the same image as render_frame,
    which bins opaque and transparent triangles in one pass."""
    W, H = 160, 120
    v, i, tpo, sd = pu.scene(40, W, H, seed=8)
    frame = pu.render_gpu(alg, W, H, v, i, tpo, sd, 60, oit_layers=8)
    st = engine.make_state(alg, W, H, oit_layers=8)
    r = engine.Renderer(st)
    mesh = engine.DeviceMesh(v, i)
    r.update_scene(sd)
    nt = (40 * 60 // 100) * tpo
    r.begin_frame()
    r.clear_transparent()
    r.draw_opaque(mesh, nt, i.shape[0] - nt)
    r.draw_transparent_color(mesh, 0, nt)
    r.composite()
    np.testing.assert_array_equal(r.output(), frame['image'])
    assert r.fragment_count() == frame['fragments']


@pytest.mark.parametrize('alg', [0, 1, 2, 3, 6])
def test_cuda_graph_replay(engine, alg):
    """OIT_FLAG_CUDA_GRAPH: the replayed frame equals the plain frame."""
    W, H = 192, 144
    v, i, tpo, sd = pu.scene(48, W, H, seed=12)
    plain = pu.render_gpu(alg, W, H, v, i, tpo, sd, 70, oit_layers=8)
    st = engine.make_state(alg, W, H, oit_layers=8, flags=engine.OIT_FLAG_CUDA_GRAPH)
    r = engine.Renderer(st)
    mesh = engine.DeviceMesh(v, i)
    r.update_scene(sd)
    for k in range(3):
        r.render_frame(mesh, tpo, 70)
        np.testing.assert_array_equal(r.output(), plain['image'])
        assert r.fragment_count() == plain['fragments']
    assert r.get_error() == 0


RASTER_CONFIGS = [{'multi_view': 0}, {'multi_view': 0, 'warps_per_sm': 32}, {'multi_view': 0, 'lane_order': 1},
                  {'multi_view': 1}, None]


@pytest.mark.parametrize('raster_cfg', RASTER_CONFIGS)
def test_batched_views_match_single_frames(engine, raster_cfg):
    """oit_batch_render (one CUDA graph, views on forked streams) gives every
    view the image its own oit_render_frame gives, with one raster launch per
    view and pass (at either register budget, views spread over the streams
    in view order or longest first), multi-view raster launches, or the
    autotuner's pick of those."""
    specs = [(1, 96, 80, 4, 12), (3, 160, 120, 16, 40), (1, 64, 64, 8, 8), (3, 128, 128, 32, 30),
             (0, 80, 60, 8, 20), (6, 96, 96, 8, 24)]
    views, refs, keep = [], [], []
    for k, (alg, W, H, L, n) in enumerate(specs):
        v, i, tpo, sd = pu.scene(n, W, H, seed=30 + k)
        refs.append(pu.render_gpu(alg, W, H, v, i, tpo, sd, 80, oit_layers=L)['image'])
        r = engine.Renderer(engine.make_state(alg, W, H, oit_layers=L))
        r.update_scene(sd)
        mesh = engine.DeviceMesh(v, i)
        views.append((r, mesh, tpo, 80))
    batch = engine.Batch(parallel_streams=4)
    batch.set_raster_config(raster_cfg)
    batch.set_views(views)
    for _ in range(3):
        batch.render()
        for (r, _, _, _), ref in zip(views, refs):
            np.testing.assert_array_equal(r.output(), ref)
            assert r.get_error() == 0
    got = batch.raster_config()
    if raster_cfg is None:
        assert (got['multi_view'], got['warps_per_sm'], got['lane_order']) in (
            (0, 36, 0), (0, 36, 1), (0, 32, 0), (0, 32, 1), (1, 36, 0))
    else:
        assert got == dict({'warps_per_sm': 36, 'lane_order': 0}, **raster_cfg)
    assert batch.launch_count() >= len(specs) * 6


@pytest.mark.parametrize('aa', [0, 1, 5])
@pytest.mark.parametrize('L', [4, 16, 32])
@pytest.mark.parametrize('alg', [1, 3])
def test_rgba32f_records(engine, alg, L, aa):
    """Plain FP32 records: float colours stored bit-exactly (nodes / payloads),
    kept sets and order as with RGBA8 keys, image within 1 LSB of the oracle."""
    W, H = 128, 96
    kw = dict(oit_layers=L, nodes_per_pixel=10, aa_type=aa, record_format=engine.OIT_RECORD_RGBA32F)
    g, o = run_pair(engine, alg, W, H, 40, percent=70, seed=17, **kw)
    check(engine, alg, g, o, W, H, L, aa, fp32=True)


def test_rgba32f_unsupported_combinations(engine):
    import ctypes
    for alg, L in ((0, 8), (2, 8), (4, 8), (5, 8), (6, 8)):
        st = engine.make_state(alg, 64, 64, oit_layers=L, record_format=engine.OIT_RECORD_RGBA32F)
        ctx = ctypes.c_void_p()
        assert engine.library().oit_create(ctypes.byref(st), ctypes.byref(ctx)) == engine.OIT_ERR_UNSUPPORTED


@pytest.mark.parametrize('aa', [0, 1, 2])
@pytest.mark.parametrize('alg', [0, 1, 2, 3, 4])
def test_half_colour_target(engine, alg, aa):
    """OIT_FLAG_HALF_COLOR: the tail-blended colour target stored as FP16
    (rounded once per tile). A-buffer bit-exact; colour target within half
    precision (relative 2^-11, plus 1e-4 absolute for the FP32 blend); image
    within 1 LSB."""
    W, H, L = 128, 96, 4
    kw = dict(oit_layers=L, nodes_per_pixel=6, aa_type=aa, flags=engine.OIT_FLAG_HALF_COLOR)
    g, o = run_pair(engine, alg, W, H, 40, percent=70, **kw)
    pu.check_pair(alg, g, o, W, H, L, aa, color_atol=1e-4, color_rtol=2.0 ** -11)


@pytest.mark.parametrize('alg', ALGS)
def test_empty_mesh_gives_background(engine, alg):
    """No triangles at all: every pixel is the cleared background (0.2 linear,
    oitRender.cpp:90) through every algorithm's composite."""
    W, H = 40, 24
    v = np.zeros((3, 10), np.float32)
    i = np.zeros((0, 3), np.uint32)
    r = engine.Renderer(engine.make_state(alg, W, H, oit_layers=4))
    r.update_scene(engine.make_camera(W, H))
    mesh = engine.DeviceMesh(v, np.zeros((1, 3), np.uint32))
    mesh.c.num_triangles = 0
    r.render_frame(mesh, 1, 100)
    img = r.output()
    assert r.get_error() == 0
    thr, _ = engine.srgb_tables()
    code = int(np.searchsorted(thr, np.float32(0.2), side='right'))
    alpha = int(np.rint(np.float32(0.2) * np.float32(255.0)))
    np.testing.assert_array_equal(img[..., :3], np.full((H, W, 3), code, np.uint8))
    np.testing.assert_array_equal(img[..., 3], np.full((H, W), alpha, np.uint8))


@pytest.mark.parametrize('alg', ALGS)
def test_one_pixel_viewport(engine, alg):
    g, o = run_pair(engine, alg, 1, 1, 20, seed=21, rmin=0.3, rmax=0.6, oit_layers=4, nodes_per_pixel=8)
    check(engine, alg, g, o, 1, 1, 4)
