"""Instanced meshes: one template sphere plus a 32-byte record per object in
place of the flattened buffer Sample::initScene builds (main.cpp:343-387).
The frame must be bit-identical to the flattened mesh's."""
import ctypes

import numpy as np
import pytest

import parity_util as pu
import vk_order_independent_transparency_gb300 as oit


def flatten(tv, ti, inst):
    """The flattened mesh of a template and instance table (float32 multiply
    then add, as oit_scene_generate computes it)."""
    n = inst.shape[0]
    r = inst[:, None, 3:4]
    pos = tv[None, :, :3] * r + inst[:, None, :3]
    v = np.concatenate([pos, np.broadcast_to(tv[None, :, 3:6], pos.shape),
                        np.broadcast_to(inst[:, None, 4:8], (n, tv.shape[0], 4))], axis=2)
    i = ti[None] + (np.arange(n, dtype=np.uint32) * tv.shape[0])[:, None, None]
    return v.reshape(-1, 10).astype(np.float32), i.reshape(-1, 3)


@pytest.mark.parametrize('stacks,slices', [(16, 32), (2, 4), (5, 7)])
def test_instanced_scene_matches_flattened(stacks, slices):
    kw = dict(seed=77, radius_min=0.03, radius_max=0.2, half_extent=1.5, stacks=stacks, slices=slices)
    v, i, tpo = oit.make_scene(37, **kw)
    tv, ti, inst = oit.make_scene_instanced(37, **kw)
    assert ti.shape[0] == tpo and inst.shape == (37, 8)
    fv, fi = flatten(tv, ti, inst)
    np.testing.assert_array_equal(fv.view(np.uint32), v.view(np.uint32))
    np.testing.assert_array_equal(fi, i)


def _frame(alg, W, H, mesh_args, instanced, percent=100, **kw):
    st = oit.make_state(alg, W, H, **kw)
    r = oit.Renderer(st)
    r.update_scene(oit.make_camera(W, H))
    if instanced:
        m = oit.DeviceInstancedMesh(*mesh_args)
        r.render_frame_instanced(m, percent)
    else:
        v, i, tpo = mesh_args
        m = oit.DeviceMesh(v, i)
        r.render_frame(m, tpo, percent)
    out = {k: r.read_buffer(b) for k, b in (('abuf', oit.OIT_BUF_ABUFFER), ('aux', oit.OIT_BUF_AUX),
                                             ('color', oit.OIT_BUF_COLOR), ('out', oit.OIT_BUF_OUTPUT),
                                             ('depth', oit.OIT_BUF_DEPTH))}
    out['fragments'] = r.fragment_count()
    out['error'] = r.get_error()
    r.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize('alg,aa,percent', [(oit.OIT_LINKEDLIST, 0, 100), (oit.OIT_LOOP64, 0, 60),
                                            (oit.OIT_INTERLOCK, oit.OIT_AA_MSAA_8X, 100),
                                            (oit.OIT_WEIGHTED, 0, 100), (oit.OIT_SPINLOCK, oit.OIT_AA_SSAA_4X, 70),
                                            (oit.OIT_LOOP, oit.OIT_AA_SUPER_4X, 100)])
def test_instanced_frame_bit_identical(alg, aa, percent):
    W, H = 160, 112
    kw = dict(seed=5, radius_min=0.05, radius_max=0.2)
    flat = oit.make_scene(200, **kw)
    tmpl = oit.make_scene_instanced(200, **kw)
    a = _frame(alg, W, H, flat, False, percent, aa_type=aa, oit_layers=8, nodes_per_pixel=12)
    b = _frame(alg, W, H, tmpl, True, percent, aa_type=aa, oit_layers=8, nodes_per_pixel=12)
    assert a['error'] == 0 and b['error'] == 0
    assert a['fragments'] == b['fragments'] > 0
    for k in ('abuf', 'aux', 'color', 'out', 'depth'):
        if k in ('abuf', 'aux') and alg == oit.OIT_LINKEDLIST:
            # node numbers follow the order in which tiles allocate them: compare the lists
            assert pu.walk_lists(a['abuf'], a['aux']) == pu.walk_lists(b['abuf'], b['aux'])
            continue
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.gpu
def test_instanced_host_path_and_oracle():
    W, H = 128, 96
    kw = dict(seed=8, radius_min=0.05, radius_max=0.2)
    tv, ti, inst = oit.make_scene_instanced(120, **kw)
    v, i, tpo = oit.make_scene(120, **kw)
    sd = oit.make_camera(W, H)
    with oit.Renderer(oit.make_state(oit.OIT_LOOP64, W, H, oit_layers=8, flags=oit.OIT_FLAG_CUDA_GRAPH)) as r:
        r.update_scene(sd)
        imgs = []
        for _ in range(3):  # plain frame + capture, then graph replays
            out = np.empty((H, W, 4), np.uint8)
            r.render_frame_instanced_host(tv, ti, inst, 100, out)
            imgs.append(out)
        assert r.get_error() == 0
    o = pu.render_oracle(oit.OIT_LOOP64, W, H, v, i, tpo, sd, oit_layers=8)
    for img in imgs:
        pu.compare_images({'image': img}, o)


@pytest.mark.gpu
def test_instanced_invalid_arguments():
    tv, ti, inst = oit.make_scene_instanced(4)
    m = oit.DeviceInstancedMesh(tv, ti, inst)
    with oit.Renderer(oit.make_state(oit.OIT_SIMPLE, 64, 64)) as r:
        lib = oit.library()
        # no scene constants yet
        assert lib.oit_render_frame_instanced(r._ctx, ctypes.byref(m.c), 100, None, None) == oit.OIT_ERR_STATE
        r.update_scene(oit.make_camera(64, 64))
        bad = oit.OitInstancedMesh(m.c.template_vertices_device, m.c.template_indices_device,
                                   m.c.instances_device + 4, m.c.template_vertices, m.c.template_triangles, 3)
        assert lib.oit_render_frame_instanced(r._ctx, ctypes.byref(bad), 100, None, None) == \
            oit.OIT_ERR_INVALID_ARGUMENT
        empty = oit.OitInstancedMesh(m.c.template_vertices_device, m.c.template_indices_device,
                                     m.c.instances_device, m.c.template_vertices, m.c.template_triangles, 0)
        assert lib.oit_render_frame_instanced(r._ctx, ctypes.byref(empty), 100, None, None) == \
            oit.OIT_ERR_INVALID_ARGUMENT
        assert lib.oit_render_frame_instanced(r._ctx, None, 100, None, None) == oit.OIT_ERR_INVALID_ARGUMENT
        r.render_frame_instanced(m)
        assert r.get_error() == 0


@pytest.mark.gpu
def test_batch_with_instanced_views():
    """Batch views may carry instanced meshes: each view's image equals its
    flattened mesh rendered alone."""
    specs = [(oit.OIT_LINKEDLIST, 120, 90, 8, 0), (oit.OIT_LOOP64, 96, 96, 4, 0),
             (oit.OIT_INTERLOCK, 80, 64, 8, oit.OIT_AA_MSAA_4X)]
    views, refs = [], []
    for k, (alg, W, H, L, aa) in enumerate(specs):
        kw = dict(seed=40 + k, radius_min=0.05, radius_max=0.2)
        flat = oit.make_scene(60, **kw)
        refs.append(_frame(alg, W, H, flat, False, 80, aa_type=aa, oit_layers=L, nodes_per_pixel=10)['out'])
        r = oit.Renderer(oit.make_state(alg, W, H, aa_type=aa, oit_layers=L, nodes_per_pixel=10))
        r.update_scene(oit.make_camera(W, H))
        views.append((r, oit.DeviceInstancedMesh(*oit.make_scene_instanced(60, **kw)), 0, 80))
    batch = oit.Batch(parallel_streams=2)
    batch.set_views(views)
    for _ in range(3):
        batch.render()
        for (r, _, _, _), ref in zip(views, refs):
            np.testing.assert_array_equal(r.read_buffer(oit.OIT_BUF_OUTPUT), ref)
            assert r.get_error() == 0


@pytest.mark.gpu
def test_batch_packed_scene_and_outputs():
    """One template shared by every view, the views' instance tables slices of
    one device buffer, and every image written into one device buffer through
    the views' output pointers: the images equal the views' flattened meshes
    rendered alone."""
    import torch
    specs = [(oit.OIT_LINKEDLIST, 72, 56, 8, 40), (oit.OIT_LOOP64, 64, 48, 4, 25), (oit.OIT_SIMPLE, 40, 40, 1, 31)]
    scenes = [oit.make_scene_instanced(n, seed=70 + k, radius_min=0.05, radius_max=0.2)
              for k, (_, _, _, _, n) in enumerate(specs)]
    tv, ti = scenes[0][0], scenes[0][1]
    tv_dev = torch.from_numpy(tv).cuda()
    ti_dev = torch.from_numpy(ti.view(np.int32)).cuda()
    # odd object counts: slices after the first start at 16-byte multiples anyway (32-byte records)
    inst_dev = torch.from_numpy(np.concatenate([s[2] for s in scenes])).cuda()
    starts = np.concatenate([[0], np.cumsum([s[2].shape[0] for s in scenes])])
    sizes = [W * H * 4 for _, W, H, _, _ in specs]
    at = np.concatenate([[0], np.cumsum(sizes)])
    out = torch.full((int(at[-1]),), 7, dtype=torch.uint8, device='cuda')
    views, refs = [], []
    for k, (alg, W, H, L, n) in enumerate(specs):
        kw = dict(seed=70 + k, radius_min=0.05, radius_max=0.2)
        refs.append(_frame(alg, W, H, oit.make_scene(n, **kw), False, 90, oit_layers=L, nodes_per_pixel=10)['out'])
        r = oit.Renderer(oit.make_state(alg, W, H, oit_layers=L, nodes_per_pixel=10))
        r.update_scene(oit.make_camera(W, H))
        m = oit.DeviceInstancedMesh.from_tensors(tv_dev, ti_dev, inst_dev[int(starts[k]):int(starts[k + 1])])
        views.append((r, m, 0, 90, out.data_ptr() + int(at[k])))
    batch = oit.Batch(parallel_streams=2)
    batch.set_views(views)
    for _ in range(3):
        out.fill_(7)
        batch.render()
        torch.cuda.synchronize()
        host = out.cpu().numpy()
        for k, ref in enumerate(refs):
            np.testing.assert_array_equal(host[at[k]:at[k + 1]], np.ascontiguousarray(ref).view(np.uint8).reshape(-1))
            assert views[k][0].get_error() == 0
