"""Triangles that cross the near plane.

The reference's pipeline clips primitives against the view volume after the
vertex shader (object.vert.glsl:34 writes gl_Position; the fixed-function
clipper does the rest), so geometry in front of and behind the near plane is
drawn in part. The engine clips each triangle against z = 0 in Vulkan clip
space (the near plane) in its setup kernel into one triangle or two (a quad
split into a fan); the oracle clips with the same float operations, so the
fragments, A-buffers and images match as for any other triangle. The camera
here sits inside the sphere cloud, so many spheres cross the near plane.
"""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

W, H = 160, 120


def inside_camera(oit):
    return oit.make_camera(W, H, eye=(0.1, 0.05, 0.35), target=(0.0, 0.0, -1.0), z_near=0.1, z_far=10.0)


def crossing_triangles(v, i, sd):
    """Triangles with vertices on both sides of the near plane (clip z = 0)."""
    m = np.array(sd.proj_view_matrix, np.float64).reshape(4, 4).T  # column-major
    pos = np.concatenate([v[:, :3].astype(np.float64), np.ones((v.shape[0], 1))], axis=1)
    z = (pos @ m.T)[:, 2]
    zt = z[i]
    return int(((zt >= 0).any(axis=1) & (zt < 0).any(axis=1)).sum())


@pytest.mark.parametrize('aa', [0, 1])
@pytest.mark.parametrize('alg', [0, 1, 2, 3, 4, 5, 6])
def test_near_plane_clip_matches_oracle(engine, alg, aa):
    L = 8
    v, i, tpo = engine.make_scene(120, seed=41, radius_min=0.05, radius_max=0.2)
    sd = inside_camera(engine)
    assert crossing_triangles(v, i, sd) > 50
    kw = dict(oit_layers=L, nodes_per_pixel=32, aa_type=aa, weighted_precision=engine.OIT_WEIGHTED_FP32)
    g = pu.render_gpu(alg, W, H, v, i, tpo, sd, 60, **kw)
    o = pu.render_oracle(alg, W, H, v, i, tpo, sd, 60, **kw)
    msaa = 4 if aa == 1 else 1
    np.testing.assert_array_equal(g['depth'][:msaa * W * H], o['depth'][:msaa * W * H])
    pu.check_pair(alg, g, o, W, H, L, aa)


def test_near_plane_clip_in_overflowed_bins(engine):
    """A replayed frame whose bins overflow walks the unbinned triangles with
    both halves of every clipped one, in primitive order."""
    import torch
    L = 8
    v, i, tpo = engine.make_scene(120, seed=41, radius_min=0.005, radius_max=0.01)
    vb, _, _ = engine.make_scene(120, seed=41, radius_min=0.05, radius_max=0.2)
    sd = inside_camera(engine)
    assert crossing_triangles(vb, i, sd) > 50
    for alg in (1, 3, 5):
        ref = pu.render_gpu(alg, W, H, vb, i, tpo, sd, 60, oit_layers=L, nodes_per_pixel=32)
        r = engine.Renderer(engine.make_state(alg, W, H, oit_layers=L, nodes_per_pixel=32,
                                              flags=engine.OIT_FLAG_CUDA_GRAPH))
        mesh = engine.DeviceMesh(v, i)
        r.update_scene(sd)
        for _ in range(2):
            r.render_frame(mesh, tpo, 60)
        mesh.vertices.copy_(torch.from_numpy(vb))
        r.render_frame(mesh, tpo, 60)
        got = pu.collect(r, alg)
        assert got['error'] == engine.OIT_DEVERR_BIN_OVERFLOW
        np.testing.assert_array_equal(got['image'], ref['image'])
        np.testing.assert_array_equal(got['depth'][:W * H], ref['depth'][:W * H])
        pu.compare_abuffer(alg, got, ref, L, W * H, False)


def test_near_plane_clip_arrival_order(engine):
    """The arrival-order pass draws the second halves too: every pixel's list
    holds the oracle's fragments."""
    v, i, tpo = engine.make_scene(120, seed=41, radius_min=0.05, radius_max=0.2)
    sd = inside_camera(engine)
    kw = dict(oit_layers=16, nodes_per_pixel=64)
    g = pu.render_gpu(1, W, H, v, i, tpo, sd, 100, flags=engine.OIT_FLAG_ARRIVAL_ORDER, **kw)
    o = pu.render_oracle(1, W, H, v, i, tpo, sd, 100, **kw)
    assert g['error'] == 0 and g['fragments'] == o['fragments']
    gl = pu.walk_lists(g['abuf'], g['aux'][:W * H])
    ol = pu.walk_lists(o['abuf'], o['aux'][:W * H])
    for a, b in zip(gl, ol):
        assert sorted(a) == sorted(b)
