"""The Python mirrors of the C ABI's structures against the header itself:
a C program compiled against include/oit_gb300.h prints every structure's
size and every field's offset, which must equal the ctypes layouts the
Python binding (and the tests through it) pass to the library."""
import ctypes
import os
import shutil
import subprocess

import pytest

import vk_order_independent_transparency_gb300 as oit

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    'oit_state': oit.OitState,
    'oit_scene_data': oit.OitSceneData,
    'oit_mesh': oit.OitMesh,
    'oit_instanced_mesh': oit.OitInstancedMesh,
    'oit_view_frame': oit.OitViewFrame,
    'oit_raster_config': oit.OitRasterConfig,
    'oit_resolve_shape': oit.OitResolveShape,
    'oit_scene_desc': oit.OitSceneDesc,
}


def _c_layouts(tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "oit_gb300.h"', 'int main(void) {']
    for name, cls in STRUCTS.items():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for field in cls._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, field[0], name, field[0]))
    lines += ['  return 0;', '}']
    src = tmp_path / 'layout.c'
    src.write_text('\n'.join(lines) + '\n')
    exe = tmp_path / 'layout'
    subprocess.run(['gcc', '-std=c11', '-I', os.path.join(ROOT, 'include'), str(src), '-o', str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict((k, int(v)) for k, v in (line.split() for line in out.splitlines()))


@pytest.mark.skipif(shutil.which('gcc') is None, reason='needs a C compiler')
def test_struct_layouts_match_header(tmp_path):
    c = _c_layouts(tmp_path)
    for name, cls in STRUCTS.items():
        assert c[name] == ctypes.sizeof(cls), name
        for field in cls._fields_:
            assert c['%s.%s' % (name, field[0])] == getattr(cls, field[0]).offset, (name, field[0])
