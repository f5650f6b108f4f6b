"""The reference's test sequence, rendered headless with this engine.

The reference's only test (test.py:13-51) runs its executable with a sequence
of 93 cases -- the default state, 8 special cases and every algorithm with and
without tail blending in each antialiasing mode -- rendering one frame per
case and saving it as an image (main.cpp:884-896). This module holds the same
case list and the reference's default State (oit.h:64-76) and scene
(main.cpp:334-417: objects in [-4, 4)^3, radius 0.45*(u*scaleWidth+scaleMin),
squared RGB, alpha range 0.2..0.5, camera at (0, 0, 12)), renders every case
through the engine and writes PNGs.

  python -m vk_order_independent_transparency_gb300.sequence --out DIR [--width 800 --height 512]
"""
import argparse
import dataclasses
import os
import struct
import zlib

import numpy as np

from . import (OIT_INTERLOCK, OIT_LINKEDLIST, DeviceMesh, Renderer, aa_settings, make_camera, make_scene,
                make_state)

ALGORITHM_NAMES = ['simple', 'linkedlist', 'loop', 'loop64', 'spinlock', 'interlock', 'weighted']
TAIL_NAMES = ['notail', 'tail']
AA_NAMES = ['noaa', 'msaa4', 'ssaa4', 'super4', 'msaa8', 'ssaa8']


@dataclasses.dataclass
class State:
    """State (oit.h:64-76) with the reference's defaults."""
    algorithm: int = 4
    oitLayers: int = 8
    linkedListAllocatedPerElement: int = 10
    percentTransparent: int = 100
    tailBlend: int = 1
    interlockIsOrdered: int = 1
    numObjects: int = 1024
    subdiv: int = 16
    scaleMin: float = 0.1
    scaleWidth: float = 0.9
    aaType: int = 0


def cases():
    """(name, State) for every case of test.py:13-51, in order."""
    out = [('init', State()),
           ('interlock_unordered', State(algorithm=OIT_INTERLOCK, interlockIsOrdered=0)),
           ('opaque', State(percentTransparent=0)),
           ('opaque_msaa4', State(percentTransparent=0, aaType=1)),
           ('opaque_ssaa4', State(percentTransparent=0, aaType=2)),
           ('3objects', State(numObjects=3)),
           ('lowsubdiv', State(subdiv=2)),
           ('scaleMin', State(scaleMin=1.0)),
           ('scaleWidth', State(scaleWidth=10.0))]
    for a in range(len(ALGORITHM_NAMES)):
        for t in range(len(TAIL_NAMES)):
            for aa in range(len(AA_NAMES)):
                out.append(('%s_%s_%s' % (ALGORITHM_NAMES[a], TAIL_NAMES[t], AA_NAMES[aa]),
                            State(algorithm=a, tailBlend=t, aaType=aa)))
    return out


def scene(st, seed=3625):
    """Mesh of a State's scene: radius = 8*0.9/16 * (u*scaleWidth + scaleMin)
    (main.cpp:360-361), centres in [-4, 4)^3, RGB squared (main.cpp:366-369)."""
    base = 8.0 * 0.9 / 16.0
    v, i, tpo = make_scene(st.numObjects, seed=seed, radius_min=base * st.scaleMin,
                           radius_max=base * (st.scaleMin + st.scaleWidth), half_extent=4.0,
                           stacks=st.subdiv, slices=2 * st.subdiv)
    v = v.copy()
    v[:, 6:9] *= v[:, 6:9]
    return v, i, tpo


def camera(width, height):
    """Camera at (0, 0, 0.75 * GRID_SIZE) looking at the origin (main.cpp:121-123). The
    projection's field of view and clip planes belong to the reference's camera library,
    which it does not vendor: 45 degrees and 0.1..100 here."""
    return make_camera(width, height, eye=(0.0, 0.0, 12.0), target=(0.0, 0.0, 0.0), fov_y=45.0, z_near=0.1,
                       z_far=100.0)


def state_kwargs(st):
    """make_state keyword arguments of a State; alphaMin 0.2 and alphaWidth
    0.3 are the reference's scene constants (main.cpp:126-127)."""
    return dict(oit_layers=st.oitLayers, nodes_per_pixel=st.linkedListAllocatedPerElement,
                tail_blend=bool(st.tailBlend), aa_type=st.aaType, alpha_min=0.2, alpha_width=0.3,
                interlock_is_ordered=bool(st.interlockIsOrdered))


def engine_state(st, width, height):
    return make_state(st.algorithm, width, height, **state_kwargs(st))


def render_case(st, width, height, mesh_cache=None):
    key = (st.numObjects, st.subdiv, st.scaleMin, st.scaleWidth)
    if mesh_cache is not None and key in mesh_cache:
        v, i, tpo, mesh = mesh_cache[key]
    else:
        v, i, tpo = scene(st)
        mesh = DeviceMesh(v, i)
        if mesh_cache is not None:
            mesh_cache[key] = (v, i, tpo, mesh)
    with Renderer(engine_state(st, width, height)) as r:
        r.update_scene(camera(width, height))
        r.render_frame(mesh, tpo, st.percentTransparent)
        img = r.output()
        if r.get_error():
            raise RuntimeError('device error bits set')
    return img


def write_png(path, rgba):
    """Minimal PNG writer (8-bit RGBA, no filtering)."""
    h, w, _ = rgba.shape
    raw = b''.join(b'\x00' + rgba[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack('>I', len(data)) + tag + data + struct.pack('>I', zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, 'wb') as f:
        f.write(b'\x89PNG\r\n\x1a\n')
        f.write(chunk(b'IHDR', struct.pack('>IIBBBBB', w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b'IDAT', zlib.compress(raw, 6)))
        f.write(chunk(b'IEND', b''))


def read_png(path):
    """Reads PNGs written by write_png."""
    with open(path, 'rb') as f:
        data = f.read()
    assert data[:8] == b'\x89PNG\r\n\x1a\n'
    pos, idat, w, h = 8, b'', 0, 0
    while pos < len(data):
        n = struct.unpack('>I', data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if tag == b'IHDR':
            w, h = struct.unpack('>II', body[:8])
        elif tag == b'IDAT':
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[y * (4 * w + 1) + 1:(y + 1) * (4 * w + 1)] for y in range(h)]
    return np.frombuffer(b''.join(rows), np.uint8).reshape(h, w, 4)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split('\n\n')[0])
    ap.add_argument('--out', required=True)
    ap.add_argument('--width', type=int, default=800)
    ap.add_argument('--height', type=int, default=512)
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    cache = {}
    for name, st in cases():
        write_png(os.path.join(a.out, name + '.png'), render_case(st, a.width, a.height, cache))
        print(name)


if __name__ == '__main__':
    main()
