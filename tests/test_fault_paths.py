"""Error paths without a GPU fault: a device allocation made to fail (as an
exhausted device would) is reported as OIT_ERR_OUT_OF_MEMORY by the call that
meets it, and the same context or batch then renders the frame correctly."""
import numpy as np
import pytest

import parity_util as pu
import vk_order_independent_transparency_gb300 as oit

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _disarm():
    """However a test ends, no armed failure reaches the next test."""
    yield
    oit.debug_fail_allocations(-1)


@pytest.mark.parametrize('alg', [oit.OIT_LINKEDLIST, oit.OIT_LOOP64, oit.OIT_WEIGHTED])
@pytest.mark.parametrize('after', [0, 1, 3])
def test_allocation_failure_recovers(alg, after):
    W, H = 96, 64
    v, i, tpo, sd = pu.scene(40, W, H, seed=9)
    ref = pu.render_gpu(alg, W, H, v, i, tpo, sd, 100, oit_layers=8)['image']
    st = oit.make_state(alg, W, H, oit_layers=8)
    mesh = oit.DeviceMesh(v, i)
    oit.debug_fail_allocations(after)
    failed = 0
    try:
        r = oit.Renderer(st)
    except oit.OitError as e:
        assert e.status == oit.OIT_ERR_OUT_OF_MEMORY
        failed += 1
        r = oit.Renderer(st)
    r.update_scene(sd)
    for _ in range(3):  # the failure fires once, at creation or in a frame
        try:
            r.render_frame(mesh, tpo, 100)
            break
        except oit.OitError as e:
            assert e.status == oit.OIT_ERR_OUT_OF_MEMORY
            failed += 1
    oit.debug_fail_allocations(-1)
    assert failed == 1
    np.testing.assert_array_equal(r.output(), ref)
    assert r.get_error() == 0
    r.render_frame(mesh, tpo, 100)
    np.testing.assert_array_equal(r.output(), ref)
    r.close()


def test_batch_allocation_failure_recovers():
    specs = [(oit.OIT_LINKEDLIST, 80, 64, 8), (oit.OIT_LOOP64, 64, 48, 4)]
    views, refs = [], []
    for k, (alg, W, H, L) in enumerate(specs):
        v, i, tpo, sd = pu.scene(30, W, H, seed=20 + k)
        refs.append(pu.render_gpu(alg, W, H, v, i, tpo, sd, 100, oit_layers=L)['image'])
        r = oit.Renderer(oit.make_state(alg, W, H, oit_layers=L))
        r.update_scene(sd)
        r.render_frame(oit.DeviceMesh(v, i), tpo, 100)  # the context's own buffers exist
        views.append((r, oit.DeviceMesh(v, i), tpo, 100))
    batch = oit.Batch(parallel_streams=2)
    batch.set_views(views)
    oit.debug_fail_allocations(0)  # the batched resolve's first allocation
    with pytest.raises(oit.OitError) as e:
        batch.render()
    oit.debug_fail_allocations(-1)
    assert e.value.status == oit.OIT_ERR_OUT_OF_MEMORY
    for _ in range(3):
        batch.render()
    for (r, _, _, _), ref in zip(views, refs):
        np.testing.assert_array_equal(r.output(), ref)
        assert r.get_error() == 0


def test_invalid_hook_argument():
    with pytest.raises(oit.OitError) as e:
        oit.debug_fail_allocations(-2)
    assert e.value.status == oit.OIT_ERR_INVALID_ARGUMENT
