"""ctypes wrapper of the CPU oracle (liboit_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg as the parity oracle; the engine never uses it.
variant='fp32_omp' loads the same source built with FP32 blending and
OpenMP tile-parallel draws (liboit_oracle_fp32_omp.so): a CPU baseline, never
used for parity.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'liboit_oracle.so')
LIB_PATHS = {'fp64': LIB_PATH, 'fp32_omp': os.path.join(HERE, 'liboit_oracle_fp32_omp.so')}

SIMPLE, LINKEDLIST, LOOP, LOOP64, SPINLOCK, INTERLOCK, WEIGHTED = range(7)
BUF_ABUFFER, BUF_AUX, BUF_AUXDEPTH, BUF_COUNTER, BUF_DEPTH, BUF_ACCUM, BUF_REVEAL, BUF_COLOR = range(8)


class OrParams(ctypes.Structure):
    _fields_ = [('algorithm', ctypes.c_int32), ('oit_layers', ctypes.c_int32), ('nodes_per_pixel', ctypes.c_int32),
                ('msaa', ctypes.c_int32), ('sample_shading', ctypes.c_int32), ('supersample', ctypes.c_int32),
                ('tail_blend', ctypes.c_int32), ('width', ctypes.c_int32), ('height', ctypes.c_int32),
                ('alpha_min', ctypes.c_float), ('alpha_width', ctypes.c_float), ('record_fp32', ctypes.c_int32),
                ('background', ctypes.c_float * 4)]


def build():
    """Compiles the oracle with its Makefile (gcc, -ffp-contract=off): the
    FP64 oracle, then the FP32 + OpenMP baseline build, which is skipped (and its
    bench leg reported unavailable) where the compiler has no OpenMP."""
    subprocess.run(['make', '-s', '-C', HERE, 'liboit_oracle.so'], check=True)
    subprocess.run(['make', '-s', '-C', HERE, 'liboit_oracle_fp32_omp.so'], check=False)
    return LIB_PATH


_libs = {}


def lib(variant='fp64'):
    if variant not in _libs:
        if not os.path.exists(LIB_PATHS[variant]):
            build()
        if not os.path.exists(LIB_PATHS[variant]):
            raise RuntimeError('oracle build %s unavailable (no OpenMP in this compiler?)' % variant)
        L = ctypes.CDLL(LIB_PATHS[variant])
        P = ctypes.c_void_p
        L.or_frame_create.restype = P
        L.or_frame_create.argtypes = [ctypes.POINTER(OrParams)]
        L.or_frame_destroy.argtypes = [P]
        L.or_begin.argtypes = [P]
        L.or_clear_transparent.argtypes = [P]
        for fn in (L.or_draw_opaque, L.or_draw_transparent):
            fn.argtypes = [P, P, P, P, P, ctypes.c_uint32, ctypes.c_uint32]
        L.or_inject_fragments.argtypes = [P, ctypes.c_int, P, P, P, P, P, P]
        L.or_composite.argtypes = [P, P, P]
        L.or_load_state.argtypes = [P, P, P, P]
        L.or_load_color.argtypes = [P, P]
        L.or_set_ll_store_limit.argtypes = [P, P]
        L.or_buffer.restype = P
        L.or_buffer.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
        L.or_fragment_count.restype = ctypes.c_uint64
        L.or_fragment_count.argtypes = [P]
        L.or_srgb_threshold.restype = ctypes.c_float
        L.or_srgb_threshold.argtypes = [ctypes.c_int]
        L.or_srgb_decode.restype = ctypes.c_double
        L.or_srgb_decode.argtypes = [ctypes.c_int]
        U32P = ctypes.POINTER(ctypes.c_uint32)
        L.or_scene_size.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, U32P, U32P, U32P]
        L.or_scene_generate.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_float, ctypes.c_float, ctypes.c_float, P, P]
        L.or_camera.argtypes = [ctypes.c_uint32, ctypes.c_uint32, P, P, ctypes.c_float, ctypes.c_float,
                                ctypes.c_float, P, P]
        L.or_srgb_encode.restype = ctypes.c_uint32
        L.or_srgb_encode.argtypes = [ctypes.c_float]
        _libs[variant] = L
    return _libs[variant]


def aa_settings(aa_type):
    return {0: (1, 0, 1), 1: (4, 0, 1), 2: (4, 1, 1), 3: (1, 0, 2), 4: (8, 0, 1), 5: (8, 1, 1)}[aa_type]


class Frame:
    """One oracle frame: the reference's per-frame images plus the FP64 colour target."""

    def __init__(self, algorithm, width, height, oit_layers=8, nodes_per_pixel=8, aa_type=0, tail_blend=True,
                 alpha_min=0.2, alpha_width=0.6, background=(0.2, 0.2, 0.2, 0.2), record_fp32=False,
                 variant='fp64'):
        msaa, ss, sup = aa_settings(aa_type)
        p = OrParams()
        p.algorithm = algorithm
        p.oit_layers = oit_layers
        p.nodes_per_pixel = nodes_per_pixel
        p.msaa = msaa
        p.sample_shading = ss
        p.supersample = sup
        p.tail_blend = 1 if tail_blend else 0
        p.width = width
        p.height = height
        p.alpha_min = alpha_min
        p.alpha_width = alpha_width
        p.record_fp32 = 1 if record_fp32 else 0
        p.background = (ctypes.c_float * 4)(*background)
        self.p = p
        self.msaa = msaa
        self.supersample = sup
        self.width, self.height = width, height
        self.lib = lib(variant)
        self.f = self.lib.or_frame_create(ctypes.byref(p))
        self._keep = []

    def __del__(self):
        try:
            if self.f:
                self.lib.or_frame_destroy(self.f)
                self.f = None
        except Exception:
            pass

    def begin(self):
        self.lib.or_begin(self.f)

    def clear_transparent(self):
        self.lib.or_clear_transparent(self.f)

    def _mats(self, scene):
        pv = np.ctypeslib.as_array(scene.proj_view_matrix).astype(np.float32).copy()
        vw = np.ctypeslib.as_array(scene.view_matrix).astype(np.float32).copy()
        self._keep += [pv, vw]
        return pv, vw

    def draw_opaque(self, scene, vertices, indices, first, count):
        pv, vw = self._mats(scene)
        v = np.ascontiguousarray(vertices, np.float32)
        i = np.ascontiguousarray(indices, np.uint32)
        self.lib.or_draw_opaque(self.f, pv.ctypes.data, vw.ctypes.data, v.ctypes.data, i.ctypes.data, first, count)

    def draw_transparent(self, scene, vertices, indices, first, count):
        pv, vw = self._mats(scene)
        v = np.ascontiguousarray(vertices, np.float32)
        i = np.ascontiguousarray(indices, np.uint32)
        self.lib.or_draw_transparent(self.f, pv.ctypes.data, vw.ctypes.data, v.ctypes.data, i.ctypes.data, first,
                                     count)

    def inject(self, xy, rgba, depth, sample=None, mask=None, view_z=None):
        xy = np.ascontiguousarray(xy, np.int32)
        rgba = np.ascontiguousarray(rgba, np.float32)
        depth = np.ascontiguousarray(depth, np.float32)
        n = len(depth)
        s = None if sample is None else np.ascontiguousarray(sample, np.int32)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint32)
        vz = None if view_z is None else np.ascontiguousarray(view_z, np.float32)
        self.lib.or_inject_fragments(self.f, n, xy.ctypes.data, None if s is None else s.ctypes.data,
                                     rgba.ctypes.data, depth.ctypes.data, None if m is None else m.ctypes.data,
                                     None if vz is None else vz.ctypes.data)

    def composite(self):
        """Returns (rgba8 (H,W,4) uint8, linear (H,W,4) float64)."""
        out8 = np.zeros((self.height, self.width, 4), np.uint8)
        lin = np.zeros((self.height, self.width, 4), np.float64)
        self.lib.or_composite(self.f, out8.ctypes.data, lin.ctypes.data)
        return out8, lin

    def load_state(self, abuffer=None, aux=None, counter=None):
        a = None if abuffer is None else np.ascontiguousarray(abuffer, np.uint32)
        x = None if aux is None else np.ascontiguousarray(aux, np.uint32)
        c = None if counter is None else np.ascontiguousarray(counter, np.uint32)
        self._keep += [a, x, c]
        self.lib.or_load_state(self.f, None if a is None else a.ctypes.data, None if x is None else x.ctypes.data,
                               None if c is None else c.ctypes.data)

    def load_color(self, color):
        """The colour target after tail blending ((S*P, 4) premultiplied linear)."""
        c = np.ascontiguousarray(color, np.float64)
        self._keep.append(c)
        self.lib.or_load_color(self.f, c.ctypes.data)

    def set_ll_store_limit(self, limit):
        lim = None if limit is None else np.ascontiguousarray(limit, np.uint32)
        self._keep.append(lim)
        self.lib.or_set_ll_store_limit(self.f, None if lim is None else lim.ctypes.data)

    def buffer(self, which, dtype=np.uint32):
        n = ctypes.c_size_t()
        ptr = self.lib.or_buffer(self.f, which, ctypes.byref(n))
        if not ptr or not n.value:
            return np.zeros(0, dtype)
        raw = (ctypes.c_char * n.value).from_address(ptr)
        return np.frombuffer(bytes(raw), dtype=dtype).copy()

    def fragment_count(self):
        return int(self.lib.or_fragment_count(self.f))


def render(algorithm, width, height, scene, vertices, indices, triangles_per_object, percent_transparent=100,
           **kw):
    """Whole frame as Sample::onRender: opaque draw of the last objects, transparent draw of the first."""
    fr = Frame(algorithm, width, height, **kw)
    num_objects = indices.shape[0] // triangles_per_object
    num_transparent = min(num_objects, num_objects * percent_transparent // 100)
    fr.begin()
    fr.clear_transparent()
    if num_objects - num_transparent > 0:
        fr.draw_opaque(scene, vertices, indices, num_transparent * triangles_per_object,
                       (num_objects - num_transparent) * triangles_per_object)
    fr.draw_transparent(scene, vertices, indices, 0, num_transparent * triangles_per_object)
    return fr


class Camera:
    """SceneData matrices of the oracle's camera, with the attribute names of
    the engine's scene-data structure (column-major 4x4 float32 each)."""

    def __init__(self, proj_view, view):
        self.proj_view_matrix = (ctypes.c_float * 16)(*proj_view)
        self.view_matrix = (ctypes.c_float * 16)(*view)


def make_scene(num_objects, seed=1, radius_min=0.05, radius_max=0.15, half_extent=1.0, stacks=16, slices=32):
    """The engine's seeded sphere scene (vertices float32 [nv,10], indices
    uint32 [nt,3], triangles_per_object), generated by the oracle library."""
    L = lib()
    nv, nt, tpo = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    if L.or_scene_size(num_objects, stacks, slices, ctypes.byref(nv), ctypes.byref(nt), ctypes.byref(tpo)) != 0:
        raise ValueError('invalid scene description')
    v = np.empty((nv.value, 10), np.float32)
    i = np.empty((nt.value, 3), np.uint32)
    if L.or_scene_generate(seed, num_objects, stacks, slices, half_extent, radius_min, radius_max, v.ctypes.data,
                           i.ctypes.data) != 0:
        raise ValueError('invalid scene description')
    return v, i, tpo.value


def make_camera(width, height, eye=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0), fov_y=45.0, z_near=0.1, z_far=10.0):
    """The engine's camera (lookAt + Vulkan perspective), from the oracle library."""
    e = np.asarray(eye, np.float32)
    t = np.asarray(target, np.float32)
    pv = np.empty(16, np.float32)
    vw = np.empty(16, np.float32)
    if lib().or_camera(width, height, e.ctypes.data, t.ctypes.data, fov_y, z_near, z_far, pv.ctypes.data,
                       vw.ctypes.data) != 0:
        raise ValueError('invalid camera')
    return Camera(pv, vw)
