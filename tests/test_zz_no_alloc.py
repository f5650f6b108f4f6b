"""The allocation-free frame entry point (oit_render_frame_noalloc).

It serves callers that cannot let a library allocate device memory: hosts
that own every allocation and budget it up front, per-frame paths that must
not risk cudaMalloc's device-wide synchronisation, processes near a memory
limit. Its scratch lives in one fixed 64 MiB device array that every call
shares, so each call must give exactly the image the context path
(oit_render_frame, whose buffers oit_create allocates) gives -- both run the
same kernels -- whatever an earlier call left in the array, and frames that do
not fit must be rejected. This file is collected last so that a failure here
leaves every other test already run; it passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu


def noalloc_frame(oit, state, scene, mesh, tpo, percent):
    import torch
    out = torch.zeros((state.height, state.width, 4), dtype=torch.uint8, device='cuda')
    st = oit.library().oit_render_frame_noalloc(ctypes.byref(state), ctypes.byref(scene), ctypes.byref(mesh.c), tpo,
                                                percent, ctypes.c_void_p(out.data_ptr()), None)
    return st, out.cpu().numpy()


CASES = [
    # algorithm, aa type, percent transparent, extra state
    (1, 0, 100, {}),                                  # linked list
    (3, 0, 60, {}),                                   # Loop64 over opaque
    (0, 4, 100, {}),                                  # Simple, MSAA 8x coverage
    (2, 0, 70, {}),                                   # Loop32 (two passes)
    (4, 0, 60, {}),                                   # Spinlock
    (5, 4, 80, {}),                                   # Interlock, MSAA 8x coverage
    (1, 1, 100, {}),                                  # linked list, MSAA 4x
    (6, 0, 80, {}),                                   # WBOIT FP16
    (6, 4, 80, {'weighted_precision': 1}),            # WBOIT FP32, MSAA 8x
    (3, 0, 100, {'flags': 0x4}),                      # Loop64, FP16 colour target
]


@pytest.mark.parametrize('alg,aa,percent,extra', CASES)
def test_noalloc_matches_context_path(engine, alg, aa, percent, extra):
    W, H = 160, 120
    v, i, tpo, sd = pu.scene(40, W, H, seed=6)
    ref = pu.render_gpu(alg, W, H, v, i, tpo, sd, percent, oit_layers=8, aa_type=aa, **extra)
    assert ref['error'] == 0
    state = engine.make_state(alg, W, H, oit_layers=8, aa_type=aa, **extra)
    mesh = engine.DeviceMesh(v, i)
    for _ in range(2):  # the second call finds the first call's data in the array
        st, img = noalloc_frame(engine, state, sd, mesh, tpo, percent)
        assert st == engine.OIT_OK, engine.status_string(st)
        np.testing.assert_array_equal(img, ref['image'])


def test_noalloc_calls_in_sequence(engine):
    """Different algorithms, sizes and scenes one after the other through the
    shared array: a value one call leaves behind (error word, pair count,
    node counter, A-buffer, colour target) must not leak into the next."""
    frames = [
        (1, 160, 120, 6, 40, 100, 8),   # linked list
        (3, 96, 64, 17, 64, 60, 16),    # Loop64 at another size, scene and OIT_LAYERS
        (2, 200, 90, 23, 30, 100, 4),   # Loop32
        (1, 160, 120, 6, 40, 100, 8),   # the first frame again
        (5, 64, 48, 31, 20, 80, 2),     # Interlock, small
        (1, 96, 64, 17, 64, 60, 16),    # linked list on the second scene
    ]
    for alg, W, H, seed, n, percent, L in frames:
        v, i, tpo, sd = pu.scene(n, W, H, seed=seed)
        ref = pu.render_gpu(alg, W, H, v, i, tpo, sd, percent, oit_layers=L)
        state = engine.make_state(alg, W, H, oit_layers=L)
        st, img = noalloc_frame(engine, state, sd, engine.DeviceMesh(v, i), tpo, percent)
        assert st == engine.OIT_OK, engine.status_string(st)
        np.testing.assert_array_equal(img, ref['image'], err_msg='alg %d %dx%d' % (alg, W, H))


def test_noalloc_rejects_unsupported_and_oversized(engine):
    v, i, tpo, _ = pu.scene(2, 64, 64, seed=1)
    mesh = engine.DeviceMesh(v, i)
    W, H = 4096, 4096  # a 16-layer Loop64 A-buffer alone needs 2 GiB
    st, _ = noalloc_frame(engine, engine.make_state(engine.OIT_LOOP64, W, H, oit_layers=16),
                          engine.make_camera(W, H), mesh, tpo, 100)
    assert st == engine.OIT_ERR_TOO_LARGE
    assert 'scratch arena' in engine.status_string(st)
    sd = engine.make_camera(64, 64)
    for kw in ({'flags': engine.OIT_FLAG_LINEAR_OUTPUT}, {'aa_type': engine.OIT_AA_SUPER_4X},
               {'record_format': engine.OIT_RECORD_RGBA32F}):
        st, _ = noalloc_frame(engine, engine.make_state(engine.OIT_LINKEDLIST, 64, 64, **kw), sd, mesh, tpo, 100)
        assert st == engine.OIT_ERR_UNSUPPORTED, kw
