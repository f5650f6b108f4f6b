"""GB300-native order-independent transparency engine (Python host mirror).

A thin ctypes layer over the engine's C ABI (include/oit_gb300.h), named after
the reference sample's transparent-pass interface (oit.h:379-425):
``Renderer.clear_transparent`` / ``draw_transparent`` / ``composite`` /
``render_frame`` (Sample::onRender). The compute path is the CUDA library
``liboit_gb300.so`` built in-tree for sm_103a; there is no fallback, and
importing the module fails loudly when the library is missing.

PyTorch is only used as a device allocator for meshes and outputs.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, 'liboit_gb300.so')

# Algorithms (shaders/common.h:44-50)
OIT_SIMPLE, OIT_LINKEDLIST, OIT_LOOP, OIT_LOOP64, OIT_SPINLOCK, OIT_INTERLOCK, OIT_WEIGHTED = range(7)
ALGORITHM_NAMES = ['simple', 'linkedlist', 'loop', 'loop64', 'spinlock', 'interlock', 'weighted']
# Antialiasing modes (shaders/common.h:58-64)
OIT_AA_NONE, OIT_AA_MSAA_4X, OIT_AA_SSAA_4X, OIT_AA_SUPER_4X, OIT_AA_MSAA_8X, OIT_AA_SSAA_8X = range(6)
OIT_RECORD_RGBA8, OIT_RECORD_RGBA32F = 0, 1
OIT_WEIGHTED_FP16, OIT_WEIGHTED_FP32 = 0, 1
OIT_FLAG_LINEAR_OUTPUT = 0x1
OIT_FLAG_CUDA_GRAPH = 0x2
OIT_FLAG_HALF_COLOR = 0x4
OIT_FLAG_ARRIVAL_ORDER = 0x8

OIT_OK = 0
OIT_ERR_INVALID_ARGUMENT = -1
OIT_ERR_UNSUPPORTED = -2
OIT_ERR_OUT_OF_MEMORY = -3
OIT_ERR_CUDA = -4
OIT_ERR_DEVICE = -5
OIT_ERR_STATE = -6
OIT_ERR_TOO_LARGE = -7

OIT_DEVERR_BIN_OVERFLOW = 0x1
OIT_DEVERR_TIMEOUT = 0x2

OIT_BUF_ABUFFER, OIT_BUF_AUX, OIT_BUF_AUXDEPTH, OIT_BUF_COUNTER, OIT_BUF_DEPTH, OIT_BUF_OPAQUE_COLOR, \
    OIT_BUF_COLOR, OIT_BUF_ACCUM, OIT_BUF_REVEAL, OIT_BUF_OUTPUT, OIT_BUF_OUTPUT_LINEAR, \
    OIT_BUF_MICROTILE_LENGTHS = range(12)

# The C ABI's exported symbols (include/oit_gb300.h).
EXPORTS = [
    'oit_create', 'oit_destroy', 'oit_update_scene', 'oit_begin_frame', 'oit_clear_transparent',
    'oit_draw_opaque', 'oit_draw_transparent_color', 'oit_composite', 'oit_draw_transparent',
    'oit_render_frame', 'oit_render_frame_host', 'oit_get_error', 'oit_get_buffer',
    'oit_get_fragment_count', 'oit_get_launch_count', 'oit_status_string', 'oit_abuffer_bytes',
    'oit_scene_size', 'oit_scene_generate', 'oit_camera', 'oit_srgb_tables', 'oit_version',
    'oit_profile_enable', 'oit_profile_read', 'oit_render_frame_noalloc',
    'oit_batch_create', 'oit_batch_destroy', 'oit_batch_render', 'oit_batch_launch_count',
    'oit_render_frame_instanced', 'oit_render_frame_instanced_host', 'oit_scene_generate_instanced',
    'oit_batch_resolve', 'oit_batch_resolve_config', 'oit_batch_set_resolve_config', 'oit_debug_fail_allocations', 'oit_debug_hold_arrival_lock',
    'oit_verify_composite_fp64', 'oit_batch_set_raster_config', 'oit_batch_raster_config',
]
PROF_SECTIONS = ['opaque_bin', 'opaque_raster', 'transparent_bin', 'transparent_raster', 'composite']


class OitState(ctypes.Structure):
    _fields_ = [
        ('algorithm', ctypes.c_uint32), ('oit_layers', ctypes.c_uint32),
        ('linked_list_allocated_per_element', ctypes.c_int32), ('tail_blend', ctypes.c_int32),
        ('interlock_is_ordered', ctypes.c_int32), ('aa_type', ctypes.c_uint32),
        ('width', ctypes.c_uint32), ('height', ctypes.c_uint32),
        ('alpha_min', ctypes.c_float), ('alpha_width', ctypes.c_float),
        ('record_format', ctypes.c_uint32), ('weighted_precision', ctypes.c_uint32),
        ('bin_capacity_scale', ctypes.c_float), ('flags', ctypes.c_uint32),
    ]


class OitSceneData(ctypes.Structure):
    _fields_ = [('proj_view_matrix', ctypes.c_float * 16), ('view_matrix', ctypes.c_float * 16)]


class OitMesh(ctypes.Structure):
    _fields_ = [('vertices_device', ctypes.c_void_p), ('indices_device', ctypes.c_void_p),
                ('num_vertices', ctypes.c_uint32), ('num_triangles', ctypes.c_uint32)]


class OitInstancedMesh(ctypes.Structure):
    _fields_ = [('template_vertices_device', ctypes.c_void_p), ('template_indices_device', ctypes.c_void_p),
                ('instances_device', ctypes.c_void_p), ('template_vertices', ctypes.c_uint32),
                ('template_triangles', ctypes.c_uint32), ('num_instances', ctypes.c_uint32)]


class OitResolveShape(ctypes.Structure):
    _fields_ = [('threads_per_block', ctypes.c_uint32), ('blocks', ctypes.c_uint32), ('binned', ctypes.c_int32),
                ('tile_order', ctypes.c_int32), ('shared_slots', ctypes.c_int32), ('items_per_step', ctypes.c_int32),
                ('register_slots', ctypes.c_int32), ('dense', ctypes.c_int32), ('bin_edges', ctypes.c_int32)]


class OitRasterConfig(ctypes.Structure):
    _fields_ = [('multi_view', ctypes.c_int32), ('warps_per_sm', ctypes.c_uint32), ('lane_order', ctypes.c_int32)]


class OitSceneDesc(ctypes.Structure):
    _fields_ = [('seed', ctypes.c_uint64), ('num_objects', ctypes.c_uint32), ('stacks', ctypes.c_uint32),
                ('slices', ctypes.c_uint32), ('half_extent', ctypes.c_float), ('radius_min', ctypes.c_float),
                ('radius_max', ctypes.c_float)]


class OitViewFrame(ctypes.Structure):
    _fields_ = [('ctx', ctypes.c_void_p), ('mesh', ctypes.POINTER(OitMesh)), ('triangles_per_object', ctypes.c_uint32),
                ('percent_transparent', ctypes.c_int32), ('out_rgba8_device', ctypes.c_void_p),
                ('instanced_mesh', ctypes.POINTER(OitInstancedMesh))]


class OitError(RuntimeError):
    def __init__(self, status, what=''):
        self.status = status
        super().__init__('%s: %s (%d)' % (what, status_string(status), status))


_lib = None


def library():
    """Loads liboit_gb300.so (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OitError(OIT_ERR_UNSUPPORTED,
                       'CUDA library %s is missing; build it with __graft_entry__.build()' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    I = ctypes.c_int
    U = ctypes.c_uint32
    sig = {
        'oit_create': (I, [ctypes.POINTER(OitState), ctypes.POINTER(P)]),
        'oit_destroy': (I, [P]),
        'oit_update_scene': (I, [P, ctypes.POINTER(OitSceneData)]),
        'oit_begin_frame': (I, [P, P]),
        'oit_clear_transparent': (I, [P, P]),
        'oit_draw_opaque': (I, [P, ctypes.POINTER(OitMesh), U, U, P]),
        'oit_draw_transparent_color': (I, [P, ctypes.POINTER(OitMesh), U, U, P]),
        'oit_composite': (I, [P, P, P]),
        'oit_draw_transparent': (I, [P, ctypes.POINTER(OitMesh), U, P, P]),
        'oit_render_frame': (I, [P, ctypes.POINTER(OitMesh), U, ctypes.c_int32, P, P]),
        'oit_render_frame_host': (I, [P, P, U, P, U, U, ctypes.c_int32, P, P]),
        'oit_get_error': (I, [P, ctypes.POINTER(U)]),
        'oit_get_buffer': (I, [P, I, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_size_t)]),
        'oit_get_fragment_count': (I, [P, ctypes.POINTER(ctypes.c_uint64)]),
        'oit_get_launch_count': (I, [P, ctypes.POINTER(ctypes.c_uint64)]),
        'oit_status_string': (ctypes.c_char_p, [I]),
        'oit_abuffer_bytes': (I, [ctypes.POINTER(OitState), ctypes.POINTER(ctypes.c_uint64),
                                  ctypes.POINTER(ctypes.c_uint64)]),
        'oit_scene_size': (I, [ctypes.POINTER(OitSceneDesc), ctypes.POINTER(U), ctypes.POINTER(U),
                               ctypes.POINTER(U)]),
        'oit_scene_generate': (I, [ctypes.POINTER(OitSceneDesc), P, P]),
        'oit_camera': (I, [U, U, ctypes.POINTER(ctypes.c_float * 3), ctypes.POINTER(ctypes.c_float * 3),
                           ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.POINTER(OitSceneData)]),
        'oit_srgb_tables': (I, [P, P]),
        'oit_version': (I, []),
        'oit_profile_enable': (I, [P, I]),
        'oit_batch_create': (I, [U, ctypes.POINTER(P)]),
        'oit_batch_destroy': (I, [P]),
        'oit_batch_render': (I, [P, ctypes.POINTER(OitViewFrame), U, P]),
        'oit_batch_launch_count': (I, [P, ctypes.POINTER(ctypes.c_uint64)]),
        'oit_render_frame_noalloc': (I, [ctypes.POINTER(OitState), ctypes.POINTER(OitSceneData),
                                         ctypes.POINTER(OitMesh), U, ctypes.c_int32, P, P]),
        'oit_profile_read': (I, [P, ctypes.POINTER(ctypes.c_double * 5), ctypes.POINTER(ctypes.c_uint64 * 5)]),
        'oit_render_frame_instanced': (I, [P, ctypes.POINTER(OitInstancedMesh), ctypes.c_int32, P, P]),
        'oit_render_frame_instanced_host': (I, [P, P, U, P, U, P, U, ctypes.c_int32, P, P]),
        'oit_scene_generate_instanced': (I, [ctypes.POINTER(OitSceneDesc), P, P, P]),
        'oit_batch_resolve': (I, [P, ctypes.POINTER(OitViewFrame), U, P]),
        'oit_batch_resolve_config': (I, [P, U, ctypes.POINTER(OitResolveShape)]),
        'oit_batch_set_resolve_config': (I, [P, U, ctypes.POINTER(OitResolveShape)]),
        'oit_debug_fail_allocations': (I, [ctypes.c_int32]),
        'oit_debug_hold_arrival_lock': (I, [P, ctypes.c_int32]),
        'oit_verify_composite_fp64': (I, [P, P, P, P]),
        'oit_batch_set_raster_config': (I, [P, ctypes.POINTER(OitRasterConfig)]),
        'oit_batch_raster_config': (I, [P, ctypes.POINTER(OitRasterConfig)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(status):
    try:
        return library().oit_status_string(status).decode()
    except OitError:
        return 'status %d' % status


def _check(status, what):
    if status != OIT_OK:
        raise OitError(status, what)


def make_state(algorithm=OIT_LINKEDLIST, width=640, height=480, oit_layers=8, nodes_per_pixel=8, tail_blend=True,
               aa_type=OIT_AA_NONE, alpha_min=0.2, alpha_width=0.6, record_format=OIT_RECORD_RGBA8,
               weighted_precision=OIT_WEIGHTED_FP16, interlock_is_ordered=True, flags=0):
    """oit_state with the reference's State fields (oit.h:64-116)."""
    s = OitState()
    s.algorithm = algorithm
    s.oit_layers = oit_layers
    s.linked_list_allocated_per_element = nodes_per_pixel
    s.tail_blend = 1 if tail_blend else 0
    s.interlock_is_ordered = 1 if interlock_is_ordered else 0
    s.aa_type = aa_type
    s.width = width
    s.height = height
    s.alpha_min = alpha_min
    s.alpha_width = alpha_width
    s.record_format = record_format
    s.weighted_precision = weighted_precision
    s.bin_capacity_scale = 0.0
    s.flags = flags
    return s


def aa_settings(aa_type):
    """(msaa, sample_shading, supersample): State::recomputeAntialiasingSettings (oit.h:84-115)."""
    return {OIT_AA_NONE: (1, 0, 1), OIT_AA_MSAA_4X: (4, 0, 1), OIT_AA_SSAA_4X: (4, 1, 1),
            OIT_AA_SUPER_4X: (1, 0, 2), OIT_AA_MSAA_8X: (8, 0, 1), OIT_AA_SSAA_8X: (8, 1, 1)}[aa_type]


def abuffer_bytes(state):
    a = ctypes.c_uint64()
    x = ctypes.c_uint64()
    _check(library().oit_abuffer_bytes(ctypes.byref(state), ctypes.byref(a), ctypes.byref(x)), 'oit_abuffer_bytes')
    return a.value, x.value


def make_scene(num_objects, seed=1, radius_min=0.05, radius_max=0.15, half_extent=1.0, stacks=16, slices=32):
    """Seeded sphere scene: (vertices float32 [nv,10], indices uint32 [nt,3], triangles_per_object)."""
    d = OitSceneDesc(seed, num_objects, stacks, slices, half_extent, radius_min, radius_max)
    nv = ctypes.c_uint32()
    nt = ctypes.c_uint32()
    tpo = ctypes.c_uint32()
    lib = library()
    _check(lib.oit_scene_size(ctypes.byref(d), ctypes.byref(nv), ctypes.byref(nt), ctypes.byref(tpo)),
           'oit_scene_size')
    v = np.empty((nv.value, 10), np.float32)
    i = np.empty((nt.value, 3), np.uint32)
    _check(lib.oit_scene_generate(ctypes.byref(d), v.ctypes.data, i.ctypes.data), 'oit_scene_generate')
    return v, i, tpo.value


def make_scene_instanced(num_objects, seed=1, radius_min=0.05, radius_max=0.15, half_extent=1.0, stacks=16,
                         slices=32):
    """The scene of make_scene as a template sphere and an instance table:
    (template vertices float32 [vpo,6], template indices uint32 [tpo,3],
    instances float32 [num_objects,8] = centre.xyz, radius, color.rgba)."""
    d = OitSceneDesc(seed, num_objects, stacks, slices, half_extent, radius_min, radius_max)
    tpo = ctypes.c_uint32()
    lib = library()
    _check(lib.oit_scene_size(ctypes.byref(d), None, None, ctypes.byref(tpo)), 'oit_scene_size')
    tv = np.empty(((stacks + 1) * (slices + 1), 6), np.float32)
    ti = np.empty((tpo.value, 3), np.uint32)
    inst = np.empty((num_objects, 8), np.float32)
    _check(lib.oit_scene_generate_instanced(ctypes.byref(d), tv.ctypes.data, ti.ctypes.data, inst.ctypes.data),
           'oit_scene_generate_instanced')
    return tv, ti, inst


def make_camera(width, height, eye=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0), fov_y=45.0, z_near=0.1, z_far=10.0):
    """SceneData matrices (column-major) for a camera looking at `target`."""
    sd = OitSceneData()
    e = (ctypes.c_float * 3)(*eye)
    t = (ctypes.c_float * 3)(*target)
    _check(library().oit_camera(width, height, ctypes.byref(e), ctypes.byref(t), fov_y, z_near, z_far,
                                ctypes.byref(sd)), 'oit_camera')
    return sd


def debug_fail_allocations(after):
    """Testing aid: the device allocation `after` allocations from now fails
    once with OIT_ERR_OUT_OF_MEMORY (-1 disarms)."""
    _check(library().oit_debug_fail_allocations(int(after)), 'oit_debug_fail_allocations')


def srgb_tables():
    thr = np.empty(256, np.float32)
    dec = np.empty(256, np.float32)
    _check(library().oit_srgb_tables(thr.ctypes.data, dec.ctypes.data), 'oit_srgb_tables')
    return thr, dec


class DeviceMesh:
    """A mesh resident in device memory (torch tensors keep the allocation alive)."""

    def __init__(self, vertices, indices, device='cuda'):
        import torch
        self.vertices = torch.as_tensor(np.ascontiguousarray(vertices, np.float32)).to(device)
        self.indices = torch.as_tensor(np.ascontiguousarray(indices, np.uint32).view(np.int32)).to(device)
        self.num_vertices = int(vertices.shape[0])
        self.num_triangles = int(indices.shape[0])
        self.c = OitMesh(self.vertices.data_ptr(), self.indices.data_ptr(), self.num_vertices, self.num_triangles)


class DeviceInstancedMesh:
    """A template mesh and its instance table resident in device memory."""

    def __init__(self, template_vertices, template_indices, instances, device='cuda'):
        import torch
        self._set(torch.as_tensor(np.ascontiguousarray(template_vertices, np.float32)).to(device),
                  torch.as_tensor(np.ascontiguousarray(template_indices, np.uint32).view(np.int32)).to(device),
                  torch.as_tensor(np.ascontiguousarray(instances, np.float32)).to(device))

    @classmethod
    def from_tensors(cls, template_vertices, template_indices, instances):
        """Views of existing device tensors (float32 [nv, 6], int32 [nt, 3],
        float32 [n, 8]): meshes can share one template and slice one instance
        buffer, so a batch's scenes upload in one copy."""
        m = cls.__new__(cls)
        m._set(template_vertices, template_indices, instances)
        return m

    def _set(self, tv, ti, inst):
        self.template_vertices, self.template_indices, self.instances = tv, ti, inst
        self.c = OitInstancedMesh(tv.data_ptr(), ti.data_ptr(), inst.data_ptr(), int(tv.shape[0]), int(ti.shape[0]),
                                  int(inst.shape[0]))


class Renderer:
    """One engine context: the role of the reference's Sample (oit.h:165-426)."""

    def __init__(self, state):
        self.state = state
        self.lib = library()
        self._ctx = ctypes.c_void_p()
        _check(self.lib.oit_create(ctypes.byref(state), ctypes.byref(self._ctx)), 'oit_create')
        self.msaa, self.sample_shading, self.supersample = aa_settings(state.aa_type)
        self.render_width = state.width * self.supersample
        self.render_height = state.height * self.supersample

    def close(self):
        if self._ctx:
            self.lib.oit_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- Sample interface ----
    def update_scene(self, scene):
        """updateUniformBuffer (main.cpp:625-643)."""
        _check(self.lib.oit_update_scene(self._ctx, ctypes.byref(scene)), 'oit_update_scene')

    def begin_frame(self, stream=None):
        _check(self.lib.oit_begin_frame(self._ctx, stream), 'oit_begin_frame')

    def clear_transparent(self, stream=None):
        """clearTransparent* (oitRender.cpp:156-356)."""
        _check(self.lib.oit_clear_transparent(self._ctx, stream), 'oit_clear_transparent')

    def draw_opaque(self, mesh, first, count, stream=None):
        _check(self.lib.oit_draw_opaque(self._ctx, ctypes.byref(mesh.c), first, count, stream), 'oit_draw_opaque')

    def draw_transparent_color(self, mesh, first, count, stream=None):
        _check(self.lib.oit_draw_transparent_color(self._ctx, ctypes.byref(mesh.c), first, count, stream),
               'oit_draw_transparent_color')

    def composite(self, out_ptr=None, stream=None):
        _check(self.lib.oit_composite(self._ctx, out_ptr, stream), 'oit_composite')

    def draw_transparent(self, mesh, num_triangles, out_ptr=None, stream=None):
        """drawTransparent*(cmd, numObjects) (oit.h:379-425): COLOR + COMPOSITE."""
        _check(self.lib.oit_draw_transparent(self._ctx, ctypes.byref(mesh.c), num_triangles, out_ptr, stream),
               'oit_draw_transparent')

    def render_frame(self, mesh, triangles_per_object, percent_transparent=100, out_ptr=None, stream=None):
        """Sample::onRender (oitRender.cpp:28-154)."""
        _check(self.lib.oit_render_frame(self._ctx, ctypes.byref(mesh.c), triangles_per_object,
                                         percent_transparent, out_ptr, stream), 'oit_render_frame')

    def render_frame_host(self, vertices, indices, triangles_per_object, percent_transparent, out, stream=None):
        """Whole frame from host arrays; `out` is a (height, width, 4) uint8 array."""
        v = np.ascontiguousarray(vertices, np.float32)
        i = np.ascontiguousarray(indices, np.uint32)
        _check(self.lib.oit_render_frame_host(self._ctx, v.ctypes.data, v.shape[0], i.ctypes.data, i.shape[0],
                                              triangles_per_object, percent_transparent, out.ctypes.data,
                                              stream), 'oit_render_frame_host')

    def render_frame_instanced(self, mesh, percent_transparent=100, out_ptr=None, stream=None):
        """render_frame over a DeviceInstancedMesh (one object per instance)."""
        _check(self.lib.oit_render_frame_instanced(self._ctx, ctypes.byref(mesh.c), percent_transparent, out_ptr,
                                                   stream), 'oit_render_frame_instanced')

    def render_frame_instanced_host(self, template_vertices, template_indices, instances, percent_transparent, out,
                                    stream=None):
        """Whole frame from a host template and instance table; `out` is (height, width, 4) uint8."""
        tv = np.ascontiguousarray(template_vertices, np.float32)
        ti = np.ascontiguousarray(template_indices, np.uint32)
        inst = np.ascontiguousarray(instances, np.float32)
        _check(self.lib.oit_render_frame_instanced_host(self._ctx, tv.ctypes.data, tv.shape[0], ti.ctypes.data,
                                                        ti.shape[0], inst.ctypes.data, inst.shape[0],
                                                        percent_transparent, out.ctypes.data, stream),
               'oit_render_frame_instanced_host')

    # ---- inspection ----

    def buffer(self, which):
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        _check(self.lib.oit_get_buffer(self._ctx, which, ctypes.byref(p), ctypes.byref(n)), 'oit_get_buffer')
        return p.value, n.value

    def read_buffer(self, which, dtype=np.uint32):
        """Copies a context buffer to a host numpy array (synchronous)."""
        import torch
        ptr, nbytes = self.buffer(which)
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype)
        if nbytes:
            torch.cuda.synchronize()
            _cudart().cudaMemcpy(ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(ptr), ctypes.c_size_t(nbytes), 2)
        return out

    def output(self):
        """Resolved RGBA8 image as (height, width, 4) uint8."""
        return self.read_buffer(OIT_BUF_OUTPUT, np.uint8).reshape(self.state.height, self.state.width, 4)

    def verify_composite_fp64(self, stream=None):
        """FP64 verification resolve of the current frame: (linear float64
        (height, width, 4) premultiplied, RGBA8 (height, width, 4))."""
        import torch
        H, W = self.state.height, self.state.width
        lin = torch.empty((H, W, 4), dtype=torch.float64, device='cuda')
        img = torch.empty((H, W, 4), dtype=torch.uint8, device='cuda')
        _check(self.lib.oit_verify_composite_fp64(self._ctx, ctypes.c_void_p(lin.data_ptr()),
                                                  ctypes.c_void_p(img.data_ptr()), stream),
               'oit_verify_composite_fp64')
        torch.cuda.synchronize()
        return lin.cpu().numpy(), img.cpu().numpy()

    def get_error(self):
        bits = ctypes.c_uint32()
        _check(self.lib.oit_get_error(self._ctx, ctypes.byref(bits)), 'oit_get_error')
        return bits.value

    def debug_hold_arrival_lock(self, element):
        """Testing aid: the next arrival-order frames start with this colour
        element's tail-blend lock held (-1 releases it)."""
        _check(self.lib.oit_debug_hold_arrival_lock(self._ctx, int(element)), 'oit_debug_hold_arrival_lock')

    def fragment_count(self):
        v = ctypes.c_uint64()
        _check(self.lib.oit_get_fragment_count(self._ctx, ctypes.byref(v)), 'oit_get_fragment_count')
        return v.value

    def profile_enable(self, enable=True):
        _check(self.lib.oit_profile_enable(self._ctx, 1 if enable else 0), 'oit_profile_enable')

    def profile_read(self):
        """{section: (total_ms, count)} since profiling was enabled."""
        ms = (ctypes.c_double * 5)()
        n = (ctypes.c_uint64 * 5)()
        _check(self.lib.oit_profile_read(self._ctx, ctypes.byref(ms), ctypes.byref(n)), 'oit_profile_read')
        return {PROF_SECTIONS[k]: (ms[k], n[k]) for k in range(5)}

    def launch_count(self):
        v = ctypes.c_uint64()
        _check(self.lib.oit_get_launch_count(self._ctx, ctypes.byref(v)), 'oit_get_launch_count')
        return v.value


class Batch:
    """Many views (Renderer, DeviceMesh, triangles per object, percent
    transparent) rendered as one CUDA graph with the views running concurrently."""

    def __init__(self, parallel_streams=8):
        self.lib = library()
        self._b = ctypes.c_void_p()
        _check(self.lib.oit_batch_create(parallel_streams, ctypes.byref(self._b)), 'oit_batch_create')
        self._frames = None
        self._keep = None

    def close(self):
        if self._b:
            self.lib.oit_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_views(self, views):
        """views: list of (Renderer, DeviceMesh or DeviceInstancedMesh,
        triangles_per_object, percent_transparent[, output device pointer]);
        without an output pointer a view writes its context's OIT_BUF_OUTPUT."""
        arr = (OitViewFrame * len(views))()
        for k, view in enumerate(views):
            r, mesh, tpo, pct = view[:4]
            arr[k].ctx = r._ctx.value
            if isinstance(mesh, DeviceInstancedMesh):
                arr[k].instanced_mesh = ctypes.pointer(mesh.c)
            else:
                arr[k].mesh = ctypes.pointer(mesh.c)
            arr[k].triangles_per_object = tpo
            arr[k].percent_transparent = pct
            arr[k].out_rgba8_device = view[4] if len(view) > 4 else None
        self._frames = arr
        self._keep = views

    def render(self, stream=None):
        _check(self.lib.oit_batch_render(self._b, self._frames, len(self._frames), stream), 'oit_batch_render')

    def launch_count(self):
        v = ctypes.c_uint64()
        _check(self.lib.oit_batch_launch_count(self._b, ctypes.byref(v)), 'oit_batch_launch_count')
        return v.value

    def resolve(self, stream=None):
        """COMPOSITE of every view's current frame: one persistent launch for the
        linked-list and Loop64 views, a composite launch per other view."""
        _check(self.lib.oit_batch_resolve(self._b, self._frames, len(self._frames), stream), 'oit_batch_resolve')

    def set_raster_config(self, config):
        """Pins the tile-raster configuration ({'multi_view': 0|1,
        'warps_per_sm': 36|32, 'lane_order': 0|1}) or, with None, lets the
        autotuner pick it."""
        if config is None:
            _check(self.lib.oit_batch_set_raster_config(self._b, None), 'oit_batch_set_raster_config')
            return
        c = OitRasterConfig(int(config.get('multi_view', 0)), int(config.get('warps_per_sm', 36)),
                            int(config.get('lane_order', 0)))
        _check(self.lib.oit_batch_set_raster_config(self._b, ctypes.byref(c)), 'oit_batch_set_raster_config')

    def raster_config(self):
        """The current graph's tile-raster configuration as a dict."""
        c = OitRasterConfig()
        _check(self.lib.oit_batch_raster_config(self._b, ctypes.byref(c)), 'oit_batch_raster_config')
        return {'multi_view': c.multi_view, 'warps_per_sm': c.warps_per_sm, 'lane_order': c.lane_order}

    def set_raster_mode(self, mode):
        """0 one raster launch per view and pass, 1 multi-view launches (both at
        the default register budget), -1 autotuned."""
        self.set_raster_config(None if mode < 0 else {'multi_view': int(mode)})

    def raster_mode(self):
        """The current graph's raster launches: 0 per view, 1 multi-view."""
        return self.raster_config()['multi_view']

    def resolve_config(self):
        """{'linkedlist': {...}, 'loop64': {...}}: per part of the batched
        resolve, the shape the autotuner picked (oit_resolve_shape's fields)."""
        out = {}
        for part, name in ((0, 'linkedlist'), (1, 'loop64')):
            sh = OitResolveShape()
            _check(self.lib.oit_batch_resolve_config(self._b, part, ctypes.byref(sh)), 'oit_batch_resolve_config')
            out[name] = {f: (bool(getattr(sh, f)) if f in ('binned', 'tile_order', 'dense') else getattr(sh, f))
                         for f, _ in OitResolveShape._fields_}
        return out

    def set_resolve_config(self, part, shape):
        """Pins one part's shape ('linkedlist' or 'loop64'; a dict with the
        fields resolve_config reports, missing ones 0), or unpins it (None)."""
        idx = {'linkedlist': 0, 'loop64': 1}[part] if isinstance(part, str) else int(part)
        if shape is None:
            _check(self.lib.oit_batch_set_resolve_config(self._b, idx, None), 'oit_batch_set_resolve_config')
            return
        sh = OitResolveShape(**{f: int(shape.get(f, 0)) for f, _ in OitResolveShape._fields_})
        _check(self.lib.oit_batch_set_resolve_config(self._b, idx, ctypes.byref(sh)), 'oit_batch_set_resolve_config')


_cudart_lib = None


def _cudart():
    """The CUDA runtime the engine library links (for plain device-to-host copies)."""
    global _cudart_lib
    if _cudart_lib is None:
        library()
        import ctypes.util
        for name in ('libcudart.so.13', 'libcudart.so', ctypes.util.find_library('cudart') or ''):
            if not name:
                continue
            try:
                _cudart_lib = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if _cudart_lib is None:
            raise OitError(OIT_ERR_CUDA, 'libcudart not found')
        _cudart_lib.cudaMemcpy.restype = ctypes.c_int
    return _cudart_lib
