"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, and its host-only entry points (sizing, scene, camera, sRGB tables,
argument validation) behave without touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import vk_order_independent_transparency_gb300 as oit
from vk_order_independent_transparency_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def lib():
    _build.build()
    return oit.library()


def header_functions():
    with open(os.path.join(ROOT, 'include', 'oit_gb300.h')) as f:
        text = f.read()
    return sorted(set(re.findall(r'^(?:int|const char\*)\s+(oit_\w+)\(', text, re.M)))


def test_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 20
    raw = ctypes.CDLL(oit.LIB_PATH)
    for n in names:
        assert hasattr(raw, n), n
    assert sorted(oit.EXPORTS) == names


def test_version_and_status(lib):
    assert lib.oit_version() == 100
    assert oit.status_string(oit.OIT_ERR_INVALID_ARGUMENT) == 'invalid argument'


@pytest.mark.parametrize('alg', range(7))
@pytest.mark.parametrize('aa', range(6))
def test_abuffer_sizing_matches_reference(lib, alg, aa):
    """oit.cpp:100-163: bytes = w*h*elementsPerSample*stride (x msaa with sample shading)."""
    st = oit.make_state(alg, 800, 512, oit_layers=8, nodes_per_pixel=10, aa_type=aa)
    ab, aux = oit.abuffer_bytes(st)
    msaa, ss, sup = oit.aa_settings(aa)
    w, h = 800 * sup, 512 * sup
    cov = msaa > 1 and not ss
    per, stride = {0: (8, 16 if cov else 8), 1: (10, 16), 2: (16, 4), 3: (8, 8), 4: (8, 16 if cov else 8),
                   5: (8, 16 if cov else 8), 6: (0, 0)}[alg]
    if ss:
        per *= msaa
    assert ab == w * h * per * stride


def test_scene_is_deterministic_and_closed(lib):
    v, i, tpo = oit.make_scene(4, seed=9)
    v2, i2, _ = oit.make_scene(4, seed=9)
    assert tpo == 960 and i.shape == (4 * 960, 3) and v.shape == (4 * 561, 10)
    np.testing.assert_array_equal(v, v2)
    np.testing.assert_array_equal(i, i2)
    # every sphere's triangles are wound outward (counter-clockwise seen from outside)
    p = v[:, :3].astype(np.float64)
    a, b, c = p[i[:, 0]], p[i[:, 1]], p[i[:, 2]]
    n = np.cross(b - a, c - a)
    centre = np.repeat(v[:, :3].reshape(4, 561, 3).mean(axis=1), 960, axis=0)
    out = ((a + b + c) / 3 - centre)
    scale = np.linalg.norm(n, axis=1) * np.linalg.norm(out, axis=1)
    cosang = np.einsum('ij,ij->i', n, out) / np.maximum(scale, 1e-30)
    assert (cosang > -1e-6).all()
    assert (cosang > 0.5).mean() > 0.95
    # colours are constant per object, in [0, 1)
    assert (v[:, 6:] >= 0).all() and (v[:, 6:] < 1).all()
    assert np.all(v[:561, 6:] == v[0, 6:])


def test_camera_matrices(lib):
    sd = oit.make_camera(640, 480)
    pv = np.array(sd.proj_view_matrix, np.float64).reshape(4, 4).T  # column-major
    vw = np.array(sd.view_matrix, np.float64).reshape(4, 4).T
    def project(x):
        c = pv @ np.array([*x, 1.0])
        return c[:3] / c[3]
    assert np.allclose(project([0, 0, 0]), [0, 0, (10 * (3 - 0.1)) / (3 * 9.9)], atol=1e-6)
    assert project([0, 1, 0])[1] < 0  # +y world is up on screen (Vulkan y down)
    assert project([1, 0, 0])[0] > 0
    assert np.isclose((vw @ np.array([0, 0, 0, 1.0]))[2], -3.0)


def test_srgb_tables_match_oracle(lib, oracle_lib):
    thr, dec = oit.srgb_tables()
    L = oracle_lib.lib()
    for k in range(255):
        assert np.float32(L.or_srgb_threshold(k)) == thr[k]
    for k in range(256):
        assert np.float32(L.or_srgb_decode(k)) == dec[k]
    assert thr[255] > 1e30


def test_srgb_table_file_is_current():
    import importlib.util
    import io
    path = os.path.join(ROOT, 'vk_order_independent_transparency_gb300', 'csrc', 'gen_srgb_tables.py')
    spec = importlib.util.spec_from_file_location('gen', path)
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    buf = io.StringIO()
    gen.main(buf)
    with open(os.path.join(ROOT, 'vk_order_independent_transparency_gb300', 'csrc', 'srgb_tables.inc')) as f:
        assert f.read() == buf.getvalue()


@pytest.mark.parametrize('field,value', [('algorithm', 7), ('oit_layers', 3), ('oit_layers', 64), ('aa_type', 6),
                                         ('width', 0), ('linked_list_allocated_per_element', 0),
                                         ('record_format', 5), ('width', 20000), ('width', 16385),
                                         ('height', 16385)])
def test_create_rejects_invalid_state(lib, field, value):
    st = oit.make_state(oit.OIT_LINKEDLIST, 64, 64)
    setattr(st, field, value)
    ctx = ctypes.c_void_p()
    assert lib.oit_create(ctypes.byref(st), ctypes.byref(ctx)) == oit.OIT_ERR_INVALID_ARGUMENT
    assert not ctx.value


def test_create_rejects_supersampled_size_past_the_limit(lib):
    # 2x2 supersampling renders at twice the size: 8193 px wide is 16386 rendered
    st = oit.make_state(oit.OIT_LOOP64, 8193, 64, aa_type=oit.OIT_AA_SUPER_4X)
    ctx = ctypes.c_void_p()
    assert lib.oit_create(ctypes.byref(st), ctypes.byref(ctx)) == oit.OIT_ERR_INVALID_ARGUMENT


def test_null_arguments(lib):
    assert lib.oit_create(None, None) == oit.OIT_ERR_INVALID_ARGUMENT
    assert lib.oit_destroy(None) == oit.OIT_ERR_INVALID_ARGUMENT
    assert lib.oit_composite(None, None, None) == oit.OIT_ERR_INVALID_ARGUMENT
    assert lib.oit_render_frame(None, None, 1, 100, None, None) == oit.OIT_ERR_INVALID_ARGUMENT
    sd = oit.OitSceneData()
    assert lib.oit_update_scene(None, ctypes.byref(sd)) == oit.OIT_ERR_INVALID_ARGUMENT
    d = oit.OitSceneDesc(1, 0, 16, 32, 1.0, 0.1, 0.2)
    assert lib.oit_scene_generate(ctypes.byref(d), None, None) == oit.OIT_ERR_INVALID_ARGUMENT
    assert lib.oit_debug_hold_arrival_lock(None, 0) == oit.OIT_ERR_INVALID_ARGUMENT
    assert lib.oit_verify_composite_fp64(None, None, None, None) == oit.OIT_ERR_INVALID_ARGUMENT
    assert lib.oit_batch_set_raster_config(None, None) == oit.OIT_ERR_INVALID_ARGUMENT
    rc = oit.OitRasterConfig()
    assert lib.oit_batch_raster_config(None, ctypes.byref(rc)) == oit.OIT_ERR_INVALID_ARGUMENT
