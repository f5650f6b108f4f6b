"""Scene constants changed between frames reach captured CUDA graphs.

The reference records the SceneData upload into every frame's command buffer
(Sample::updateUniformBuffer, main.cpp:625-643, called from
oitRender.cpp:38), so a moving camera is seen by every frame. Here a frame
replayed from a CUDA graph (OIT_FLAG_CUDA_GRAPH, and oit_batch_render) must
render the camera set by the latest oit_update_scene: the same image, A-buffer
and colour target as a frame rendered without a graph from that camera.
"""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

W, H = 160, 120


def cameras(oit):
    a = oit.make_camera(W, H)
    # further back and to the side: every sphere covers fewer tiles, so the
    # bins sized for camera A hold camera B's pairs
    b = oit.make_camera(W, H, eye=(0.5, 0.35, 3.6), target=(0.1, 0.0, 0.0))
    return a, b


def same_frame(alg, got, ref, L):
    np.testing.assert_array_equal(got['image'], ref['image'])
    np.testing.assert_array_equal(got['color'], ref['color'])
    assert got['fragments'] == ref['fragments']
    assert got['error'] == 0
    if alg != 6:
        pu.compare_abuffer(alg, got, ref, L, W * H, False)


@pytest.mark.parametrize('alg', [1, 3, 5, 6])
def test_graph_replay_follows_camera(engine, alg):
    v, i, tpo = engine.make_scene(48, seed=12, radius_min=0.05, radius_max=0.2)
    cam_a, cam_b = cameras(engine)
    L = 8
    ref_a = pu.render_gpu(alg, W, H, v, i, tpo, cam_a, 70, oit_layers=L)
    ref_b = pu.render_gpu(alg, W, H, v, i, tpo, cam_b, 70, oit_layers=L)
    assert not np.array_equal(ref_a['image'], ref_b['image'])
    r = engine.Renderer(engine.make_state(alg, W, H, oit_layers=L, flags=engine.OIT_FLAG_CUDA_GRAPH))
    mesh = engine.DeviceMesh(v, i)
    r.update_scene(cam_a)
    for _ in range(2):  # plain frame + capture, then a replay
        r.render_frame(mesh, tpo, 70)
    same_frame(alg, pu.collect(r, alg), ref_a, L)
    r.update_scene(cam_b)
    r.render_frame(mesh, tpo, 70)  # replay with camera B
    same_frame(alg, pu.collect(r, alg), ref_b, L)
    r.update_scene(cam_a)
    r.render_frame(mesh, tpo, 70)  # and back to camera A
    same_frame(alg, pu.collect(r, alg), ref_a, L)


class _DeviceArray:
    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {'shape': shape, 'typestr': typestr, 'data': (ptr, False), 'version': 3}


def test_queued_frames_keep_their_camera(engine):
    """Graph replays queued without waiting, each after its own
    oit_update_scene (more updates than the pinned ring has slots): every
    replay renders the camera it was called with. Each frame's image is copied
    out on the same stream right after it."""
    import torch
    alg, L = 1, 8
    v, i, tpo = engine.make_scene(48, seed=12, radius_min=0.05, radius_max=0.2)
    cams = [engine.make_camera(W, H, eye=(0.1 * k, 0.05 * k, 3.0 + 0.15 * k)) for k in range(7)]
    refs = [pu.render_gpu(alg, W, H, v, i, tpo, c, 100, oit_layers=L)['image'] for c in cams]
    r = engine.Renderer(engine.make_state(alg, W, H, oit_layers=L, flags=engine.OIT_FLAG_CUDA_GRAPH))
    mesh = engine.DeviceMesh(v, i)
    ptr, nbytes = r.buffer(engine.OIT_BUF_OUTPUT)
    out = torch.as_tensor(_DeviceArray(ptr, (H, W, 4), '|u1'), device='cuda')
    copies = [torch.zeros((H, W, 4), dtype=torch.uint8, device='cuda') for _ in cams]
    r.update_scene(cams[0])
    r.render_frame(mesh, tpo, 100)  # plain frame + capture
    torch.cuda.synchronize()
    for _ in range(2):
        for c, dst in zip(cams, copies):
            r.update_scene(c)
            r.render_frame(mesh, tpo, 100)  # replay on the legacy default stream's order
            dst.copy_(out)
        torch.cuda.synchronize()
        for dst, ref in zip(copies, refs):
            np.testing.assert_array_equal(dst.cpu().numpy(), ref)


@pytest.mark.parametrize('raster_mode', [0, 1])
def test_batch_replay_follows_camera(engine, raster_mode):
    specs = [(1, 96, 80, 4, 12), (3, 160, 120, 16, 40), (5, 128, 96, 8, 30), (6, 96, 96, 8, 24)]
    views, rigs = [], []
    for k, (alg, w, h, L, n) in enumerate(specs):
        v, i, tpo = engine.make_scene(n, seed=40 + k, radius_min=0.05, radius_max=0.2)
        ca = engine.make_camera(w, h)
        cb = engine.make_camera(w, h, eye=(-0.4, 0.2, 3.5))
        r = engine.Renderer(engine.make_state(alg, w, h, oit_layers=L))
        r.update_scene(ca)
        mesh = engine.DeviceMesh(v, i)
        views.append((r, mesh, tpo, 80))
        rigs.append((alg, w, h, L, v, i, tpo, ca, cb))
    batch = engine.Batch(parallel_streams=4)
    batch.set_raster_mode(raster_mode)
    batch.set_views(views)
    for _ in range(2):  # plain frames + capture, then a replay
        batch.render()
    for cam in (8, 7, 8):  # index of the camera in each rig: B, then A, then B
        for (r, *_), rig in zip(views, rigs):
            r.update_scene(rig[cam])
        batch.render()
        for (r, *_), (alg, w, h, L, v, i, tpo, ca, cb) in zip(views, rigs):
            ref = pu.render_gpu(alg, w, h, v, i, tpo, ca if cam == 7 else cb, 80, oit_layers=L)
            np.testing.assert_array_equal(r.output(), ref['image'])
            assert r.get_error() == 0
