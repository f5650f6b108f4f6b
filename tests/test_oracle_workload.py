"""The CPU legs' workload generator in the oracle library against the
engine's: seeded sphere scenes and cameras, bit for bit, so a process that
times the oracle needs no product code to build its inputs."""
import numpy as np
import pytest

import vk_order_independent_transparency_gb300 as oit

orc = pytest.importorskip('oracle')


@pytest.mark.parametrize('n,seed,rmin,rmax', [(1, 1, 0.05, 0.15), (64, 7, 0.01, 0.05), (300, 2000, 0.2, 0.35),
                                              (1024, 3625, 0.03, 0.1)])
def test_scene_matches_engine(n, seed, rmin, rmax):
    a = oit.make_scene(n, seed=seed, radius_min=rmin, radius_max=rmax)
    b = orc.make_scene(n, seed=seed, radius_min=rmin, radius_max=rmax)
    assert a[2] == b[2]
    np.testing.assert_array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    np.testing.assert_array_equal(a[1], b[1])


def test_scene_shapes_match_engine():
    for stacks, slices in ((2, 3), (8, 12), (16, 32)):
        a = oit.make_scene(5, seed=3, stacks=stacks, slices=slices)
        b = orc.make_scene(5, seed=3, stacks=stacks, slices=slices)
        np.testing.assert_array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
        np.testing.assert_array_equal(a[1], b[1])
    with pytest.raises(ValueError):
        orc.make_scene(0)


@pytest.mark.parametrize('w,h,eye,target,fov,zn,zf', [
    (640, 480, (0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 45.0, 0.1, 10.0),
    (1920, 1080, (0.3, -0.2, 2.5), (0.1, 0.0, -0.5), 60.0, 0.05, 20.0),
    (160, 120, (0.1, 0.05, 0.35), (0.0, 0.0, -1.0), 45.0, 0.1, 10.0)])
def test_camera_matches_engine(w, h, eye, target, fov, zn, zf):
    a = oit.make_camera(w, h, eye=eye, target=target, fov_y=fov, z_near=zn, z_far=zf)
    b = orc.make_camera(w, h, eye=eye, target=target, fov_y=fov, z_near=zn, z_far=zf)
    for name in ('proj_view_matrix', 'view_matrix'):
        x = np.ctypeslib.as_array(getattr(a, name)).view(np.uint32)
        y = np.ctypeslib.as_array(getattr(b, name)).view(np.uint32)
        np.testing.assert_array_equal(x, y)
