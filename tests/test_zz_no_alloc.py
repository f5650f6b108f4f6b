"""The allocation-free frame entry point (oit_render_frame_noalloc).

It serves callers that cannot let a library allocate device memory (hosts
that own all allocations and budget them up front, per-frame paths that must
not risk cudaMalloc's device-wide synchronisation, processes near a memory
limit). Its scratch lives in a fixed 64 MiB device array, so it must give the
same image as the context path (oit_render_frame, which allocates its buffers
in oit_create) on consecutive calls that reuse the array, and reject frames
that do not fit. This file is collected last so that a failure here leaves
every other test already run.
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


@pytest.mark.parametrize('alg,aa,percent', [(1, 0, 100), (3, 0, 60), (0, 4, 100), (4, 0, 60), (6, 0, 80)])
def test_noalloc_matches_context_path(engine, alg, aa, percent):
    W, H = 160, 120
    v, i, tpo, sd = pu.scene(40, W, H, seed=6)
    ref = pu.render_gpu(alg, W, H, v, i, tpo, sd, percent, oit_layers=8, aa_type=aa)
    state = engine.make_state(alg, W, H, oit_layers=8, aa_type=aa)
    mesh = engine.DeviceMesh(v, i)
    for _ in range(2):  # the second call finds the first call's data in the arena
        st, img = noalloc_frame(engine, state, sd, mesh, tpo, percent)
        assert st == engine.OIT_OK, engine.status_string(st)
        d = np.abs(img.astype(np.int32) - ref['image'].astype(np.int32))
        assert d.max() <= 1


def test_noalloc_rejects_frames_beyond_the_arena(engine):
    W, H = 4096, 4096  # a 16-layer Loop64 A-buffer alone needs 2 GiB
    v, i, tpo, _ = pu.scene(2, 64, 64, seed=1)
    sd = engine.make_camera(W, H)
    state = engine.make_state(engine.OIT_LOOP64, W, H, oit_layers=16)
    mesh = engine.DeviceMesh(v, i)
    st, _ = noalloc_frame(engine, state, sd, mesh, tpo, 100)
    assert st == engine.OIT_ERR_TOO_LARGE
    assert 'scratch arena' in engine.status_string(st)
