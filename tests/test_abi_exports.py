"""C ABI checks that need no GPU: the library loads, exports every entry point the public header
declares, and the ctypes mirror has the header's struct layout."""
import ctypes as C
import pathlib
import re
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "lambda_gpu.h"


def _declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"LGPU_API\s+[\w\s\*]+?\b(lgpu_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import lambda_gb300 as lg
    lg.build()
    return lg.lib()


def test_header_declares_entry_points():
    names = _declared()
    assert "lgpu_render" in names and "lgpu_scene_commit" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, "declared in the header but not exported: %s" % missing


def test_python_export_list_matches_header():
    import lambda_gb300 as lg
    assert sorted(lg.EXPORTS) == _declared()


def test_version_string(lib):
    v = lib.lgpu_version().decode()
    assert v and "sm_103a" in v


def test_ctypes_layout_matches_header(tmp_path):
    """Compile a C program against the header and compare sizeof/offsetof with the ctypes mirror."""
    from lambda_gb300 import abi
    structs = {"lgpu_mesh_desc": abi.MeshDesc, "lgpu_object_desc": abi.ObjectDesc,
               "lgpu_material_desc": abi.MaterialDesc, "lgpu_node_desc": abi.NodeDesc,
               "lgpu_light_desc": abi.LightDesc, "lgpu_medium_desc": abi.MediumDesc,
               "lgpu_scene_desc": abi.SceneDesc, "lgpu_camera_desc": abi.CameraDesc,
               "lgpu_render_opts": abi.RenderOpts, "lgpu_stats": abi.Stats}
    if hasattr(abi, "ViewDesc"):
        structs["lgpu_view_desc"] = abi.ViewDesc
    if hasattr(abi, "AdjointDesc"):
        structs["lgpu_adjoint_desc"] = abi.AdjointDesc
        structs["lgpu_texture_desc"] = abi.TextureDesc
    if hasattr(abi, "Tuning"):
        structs["lgpu_tuning"] = abi.Tuning
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "lambda_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.split("\n") if l)
    for cname, py in structs.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out["%s.%s" % (cname, f)]) == getattr(py, f).offset, "%s.%s" % (cname, f)
