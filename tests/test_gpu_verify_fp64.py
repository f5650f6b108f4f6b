"""The FP64 verification resolve (oit_verify_composite_fp64) against the CPU
oracle's FP64 composite.

The verification kernel recomputes the COMPOSITE pass in double from the
GPU's own A-buffer and colour target. Where the GPU's tail-blended colour
target holds exactly what the oracle's FP64 one holds (tail blending off, so
only the opaque pass or the background writes it; or a linked list whose pool
never overflows, whose raster blends nothing), the only difference left is
the order of double operations: the premultiplied linear output must agree
with the oracle's within 1e-12, and the RGBA8 image exactly. Against the
production FP32 resolve it stays within 1 LSB.
"""
import numpy as np
import pytest

import parity_util as pu

pytestmark = pytest.mark.gpu

CASES = [
    # algorithm, aa type, tail blend, percent transparent, OIT_LAYERS, nodes per pixel
    (0, 0, False, 60, 8, 8),
    (1, 0, True, 60, 4, 64),     # composite tail (insertionSortTail) in FP64, no pool overflow
    (1, 0, False, 100, 8, 64),
    (2, 0, False, 60, 8, 8),
    (3, 0, False, 60, 8, 8),
    (4, 0, False, 60, 8, 8),
    (5, 0, False, 60, 8, 8),
    (3, 2, False, 100, 4, 8),    # sample shading: per-sample A-buffers and colour targets
    (1, 3, True, 100, 4, 64),    # 2x2 supersampling
    (5, 3, False, 80, 4, 8),
]


@pytest.mark.parametrize('alg,aa,tail,percent,L,npp', CASES)
def test_fp64_resolve_matches_oracle(engine, alg, aa, tail, percent, L, npp):
    W, H = 128, 96
    v, i, tpo, sd = pu.scene(48, W, H, seed=14, radius_min=0.08, radius_max=0.25)
    kw = dict(oit_layers=L, nodes_per_pixel=npp, aa_type=aa, tail_blend=tail)
    g = pu.render_gpu(alg, W, H, v, i, tpo, sd, percent, **kw)
    o = pu.render_oracle(alg, W, H, v, i, tpo, sd, percent, **kw)
    assert g['error'] == 0 and g['fragments'] == o['fragments']
    if alg == 1:
        assert g['counter'][0] < npp * W * H * (4 if aa == 3 else 1)  # no pool overflow
    lin, img = g['renderer'].verify_composite_fp64()
    ref = o['linear'].reshape(H, W, 4)
    err = np.abs(lin - ref).max()
    assert err < 1e-12, err
    np.testing.assert_array_equal(img, o['image'])
    d = np.abs(img.astype(np.int32) - g['image'].astype(np.int32))
    assert d.max() <= 1


@pytest.mark.parametrize('alg', [1, 3])
def test_fp64_resolve_of_batched_views(engine, alg):
    """The verification resolve reads a batch view's frame (RGBA8 records,
    FP16 colour target): the production image is within 1 LSB of it."""
    W, H = 160, 120
    v, i, tpo, sd = pu.scene(40, W, H, seed=5)
    r = engine.Renderer(engine.make_state(alg, W, H, oit_layers=8, flags=engine.OIT_FLAG_HALF_COLOR))
    r.update_scene(sd)
    mesh = engine.DeviceMesh(v, i)
    batch = engine.Batch(parallel_streams=2)
    batch.set_views([(r, mesh, tpo, 100)])
    for _ in range(2):
        batch.render()
    _, img = r.verify_composite_fp64()
    d = np.abs(img.astype(np.int32) - r.output().astype(np.int32))
    assert d.max() <= 1
