"""The C ABI library without a GPU: it loads, exports every symbol the header
declares, keeps the reference's struct layouts, and its host-side scene build (SAH
BVH, lights, radius) is bit-identical to the reference's."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from realcausticsengine_gb300 import _native, abi, scenes
from realcausticsengine_gb300.scene import InitArgs
from realcausticsengine_gb300.session import Renderer

HEADER = Path(__file__).resolve().parents[1] / "include" / "realcaustics.h"


def header_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "sizeof")))


def test_library_loads_and_exports_header_symbols():
    lib = _native.lib()
    names = header_functions()
    assert "init" in names and "main" in names and "rc_trace_rays" in names
    for n in names:
        assert hasattr(lib, n), f"missing export {n}"
    assert set(names) <= set(_native.EXPORTS) | {"init", "main"}


def test_struct_layouts_match_reference():
    assert C.sizeof(abi.PythonLight) == 64 and C.sizeof(abi.PythonMaterial) == 28
    assert abi.PythonLight.power.offset == 52 and abi.PythonLight.rotation.offset == 40
    assert abi.PythonMaterial.color.offset == 16
    assert C.sizeof(abi.DebugStuff) == 24 and C.sizeof(abi.Matrix4x4) == 64


def test_layout_against_reference(ref):
    out = (C.c_longlong * 40)()
    size = ref.ref_layout(out)
    assert size == abi.MESH_BLENDER_SIZE
    assert list(out)[:3] == [abi.OFF_MPOLY, abi.OFF_MLOOP, abi.OFF_MVERT]
    assert list(out)[3:10] == [20, 12, 8, 64, 28, 64, 24]


def test_host_scene_matches_golden(golden):
    sc = scenes.test_scene(48, 36, subdiv=2, samples=2)
    r = Renderer(sc)
    info = r.prepare_host()
    assert (info.view(np.uint32) == golden["prep_info"].view(np.uint32)).all()
    for m in range(len(sc.meshes)):
        nodes, cost = r.host_mesh_bvh(m, 1 << 14)
        assert (nodes == golden[f"mesh{m}_nodes"]).all()
        assert np.float32(cost) == golden[f"mesh{m}_cost"][0]
    r.release()


@pytest.mark.parametrize("maker", [lambda: scenes.test_scene(40, 30, subdiv=3), scenes.sun_scene,
                                   lambda: scenes.glass_sphere_point(32, 32, subdiv=5),
                                   # 178,802 triangles: the multi-threaded build paths
                                   lambda: scenes.water_pool(64, 48, grid=300)])
def test_host_bvh_matches_reference(ref, in_tmpdir, maker):
    """Host SAH BVH (multi-threaded above 16k primitives) node arrays, triangle lists and
    traversal costs bit-identical to the reference's sequential build."""
    sc = maker()
    args = InitArgs(sc)
    args.call(ref.init)
    info_r = (C.c_float * 9)()
    ref.ref_prepare(info_r)
    r = Renderer(sc)
    info = r.prepare_host()
    assert (np.array(info_r, np.float32).view(np.uint32) == info.view(np.uint32)).all()
    for m in range(len(sc.meshes)):
        cap = 1 << 19
        nr = np.zeros((cap, 8), np.uint32)
        tr = np.zeros(cap, np.int32)
        cr = C.c_float()
        n = ref.ref_mesh_bvh(m, nr.ctypes.data, cap, tr.ctypes.data, cap, C.byref(cr))
        nodes, cost, idx = r.host_mesh_bvh(m, cap, with_index=True)
        assert (nodes == nr[:n]).all() and np.float32(cost) == np.float32(cr.value)
        nt = len(sc.meshes[m].tris)
        assert (idx[:nt + 1] == tr[:nt + 1]).all()
    ref.ref_release()
    r.release()


def test_errors_are_reported_not_crashes():
    lib = _native.lib()
    lib.rc_release()
    assert lib.main() == -1                       # no scene: reference would dereference null
    assert b"no scene" in lib.rc_last_error()
    cfg = abi.RcConfig()
    lib.rc_default_config(C.byref(cfg))
    assert cfg.max_path_length == 6 and cfg.exr_path == b"D:\\caustics.exr"
    bad = abi.RcConfig()
    lib.rc_default_config(C.byref(bad))
    bad.max_path_length = -1
    assert lib.rc_set_config(C.byref(bad)) == -2
    # a scene without lights fails in the host prepare with a message
    sc = scenes.test_scene(16, 16, subdiv=1)
    sc.lights = []
    r = Renderer(sc)
    with pytest.raises(_native.NativeError, match="no lights"):
        r.prepare_host()
    r.release()


def test_material_index_out_of_range_rejected_at_init():
    sc = scenes.test_scene(16, 16, subdiv=1)
    sc.meshes[0].slot_materials = [99]
    with pytest.raises(RuntimeError, match="material index"):
        Renderer(sc)
    _native.lib().rc_release()


def _bvh_obj_files(root):
    return {p.name: p.read_bytes() for p in sorted(root.iterdir()) if p.name.startswith("D:\\bvh\\Mesh_")}


def _single_mesh(sc):
    sc.meshes = sc.meshes[:1]
    return sc


@pytest.mark.parametrize("maker", [lambda: _single_mesh(scenes.glass_sphere_point(16, 16, subdiv=3)),
                                   lambda: _single_mesh(scenes.water_pool(16, 16, grid=40)),
                                   lambda: _single_mesh(scenes.gem_cluster(16, 16, n_gems=60))])
def test_debug_bvh_obj_matches_reference(ref, in_tmpdir, maker):
    """Debug view 5 (Vertex_Merging::run_debug_bvh): the OBJ files of the mesh BVHs' boxes,
    one per mesh and depth, byte for byte the reference's (host only: no GPU needed).
    Single-mesh scenes: with inner world nodes the reference reads past its mesh list and
    crashes (it walks every world node as a leaf); the library walks the leaves only."""
    sc = maker()
    args = InitArgs(sc)
    args.call(ref.init)
    assert ref.ref_prepare(None) == 0
    assert ref.ref_debug_bvh() == 0
    ref.ref_release()
    want = _bvh_obj_files(in_tmpdir)
    assert want
    for name in want:
        (in_tmpdir / name).unlink()
    lib = _native.lib()
    r = Renderer(sc)
    assert lib.rc_render_debug(5) == 0, lib.rc_last_error()
    r.release()
    got = _bvh_obj_files(in_tmpdir)
    assert sorted(got) == sorted(want)
    for name in want:
        assert got[name] == want[name], name


def test_main_debug_bvh_writes_obj_files_and_no_image(tmp_path):
    """init(debug_test=5) + main(): the BVH boxes as OBJ files beside the configured EXR
    path (in its "bvh" directory), no image, no GPU needed."""
    sc = _single_mesh(scenes.glass_sphere_point(16, 16, subdiv=2))
    lib = _native.lib()
    cfg = abi.RcConfig()
    lib.rc_default_config(C.byref(cfg))
    cfg.exr_path = str(tmp_path / "out.exr").encode()
    assert lib.rc_set_config(C.byref(cfg)) == 0
    (tmp_path / "bvh").mkdir()
    InitArgs(sc, debug_test=5).call(lib.init)
    assert lib.main() == 0, lib.rc_last_error()
    names = sorted(p.name for p in (tmp_path / "bvh").iterdir())
    assert names and names[0] == "Mesh_1_1.obj" and not (tmp_path / "out.exr").exists()
    first = (tmp_path / "bvh" / "Mesh_1_1.obj").read_text().splitlines()
    assert len(first) == 14 and first[0].startswith("v ") and first[8] == "f 1/ 5/ 7/ 3/"
