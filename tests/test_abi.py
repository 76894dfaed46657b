"""C ABI boundary: the library loads and exports every entry point the public
headers declare, and argument errors come back as status codes (no GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def header_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(yv_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_library_exports_every_declared_symbol(yoxel_mod):
    declared = header_symbols()
    assert len(declared) > 20
    exported = exported_symbols(yoxel_mod.LIB_PATH)
    missing = sorted(declared - exported)
    assert not missing, f"declared but not exported: {missing}"


def test_binding_covers_header(yoxel_mod):
    from yoxel import _lib
    assert set(_lib.declared_symbols()) == header_symbols()


def test_status_strings(yoxel_mod):
    from yoxel import _lib as L
    assert L.status_string(L.YV_OK) == "ok"
    assert "scene" in L.status_string(L.YV_ERR_NO_SCENE)
    assert L.status_string(12345) == "unknown status"


def test_argument_errors_are_status_codes(yoxel_mod):
    from yoxel import _lib as L
    lib = L.lib
    h = C.c_void_p()
    assert lib.yv_svo_gen_spheres(C.byref(h), 0, 10, 4.0, 8.0, 1) == L.YV_ERR_INVALID_ARG
    assert lib.yv_svo_gen_spheres(C.byref(h), 5, 10, 8.0, 4.0, 1) == L.YV_ERR_INVALID_ARG
    assert lib.yv_svo_gen_terrain(C.byref(h), 5, 10, 0, 4, 1) == L.YV_ERR_INVALID_ARG
    assert lib.yv_svo_gen_spheres(None, 5, 10, 4.0, 8.0, 1) == L.YV_ERR_INVALID_ARG
    assert lib.yv_svo_load_vox(C.byref(h), b"/nonexistent/file.vox") == L.YV_ERR_IO
    assert lib.yv_renderer_create(None) == L.YV_ERR_INVALID_ARG
    assert lib.yv_set_resolution(None, 4, 4) == L.YV_ERR_INVALID_ARG
    assert lib.yv_render_frame(None, None, None, None) == L.YV_ERR_INVALID_ARG


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_renderer_create_without_gpu_reports_cuda_error(yoxel_mod):
    from yoxel import _lib as L
    h = C.c_void_p()
    st = L.lib.yv_renderer_create(C.byref(h))
    assert st == L.YV_ERR_CUDA
    assert not h.value


def test_product_package_does_not_import_oracle():
    """The product path (yoxel package, C++/CUDA sources) never touches the
    oracle: no import, no link, no path."""
    pkg = os.path.join(ROOT, "yoxel-voxel_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h", ".cuh")):
                text = open(os.path.join(dirpath, f)).read()
                for bad in ("pyoracle", "liboracle", "orc_", "import oracle",
                            "from oracle", "yv_oracle"):
                    assert bad not in text, f"{f} references the oracle ({bad})"


STRUCTS = {"VoxNode": "yv_vox_node", "LeafAttr": "yv_leaf_attr", "Light": "yv_light",
           "FrameOutputs": "yv_frame_outputs", "PointLight": "yv_point_light",
           "SsnaParams": "yv_ssna_params", "FrameStats": "yv_frame_stats",
           "LaunchConfig": "yv_launch_config", "VolumeDevice": "yv_volume_device",
           "Camera": "yv_camera", "MarchParams": "yv_march_params"}


def test_struct_layouts_match_bindings(yoxel_mod, tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler
    gives the header's struct."""
    from yoxel import _lib as L
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "yv_c_api.h"',
             'int main(void) {']
    expect = []
    for py, cname in STRUCTS.items():
        cls = getattr(L, py)
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        expect.append(C.sizeof(cls))
        for f in cls._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f[0]))
            expect.append(getattr(cls, f[0]).offset)
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == expect
