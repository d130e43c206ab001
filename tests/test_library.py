"""The C-ABI library: loads, exports every declared symbol, struct layouts match the
header, argument errors are reported without touching a GPU, host-side model logic."""

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from ffsrl import SimModelDO, _lib as L, meshgen as mg

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "ffsrl.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(ffsrl_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(built_lib):
    assert L.lib().ffsrl_abi_version() == 2


STRUCTS = {"ffsrl_model": L.Model, "ffsrl_params": L.Params, "ffsrl_bvh": L.Bvh, "ffsrl_render": L.Render,
           "ffsrl_batch_options": L.BatchOptions, "ffsrl_server_config": L.ServerConfig,
           "ffsrl_render_config": L.RenderConfig}


def test_struct_layouts_match_header(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.split("\n") if l)
    for cname, py in STRUCTS.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(py, f).offset, f"{cname}.{f}"


def test_argument_errors_need_no_gpu(built_lib):
    lib = L.lib()
    assert lib.ffsrl_step_model(None, None, None) == L.ERR_INVALID_ARGUMENT
    assert b"null" in lib.ffsrl_last_error()
    assert lib.ffsrl_remap(None, None, None, 5, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_batch_create(None, None, None, None, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_bvh_refit_fused(None, None, None, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_render_fused(None, None, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_grasp_nearest(None, None, None, None, None, 0.0, None, 3, None) == L.ERR_INVALID_ARGUMENT
    # serving, graphs and cutting check their arguments before touching a device
    h = C.c_void_p()
    assert lib.ffsrl_server_create(None, C.byref(h)) == L.ERR_INVALID_ARGUMENT and not h.value
    assert lib.ffsrl_server_create(C.byref(L.ServerConfig()), C.byref(h)) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_server_submit(None, 0, None, 1, 0, 7) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_server_poll(None, 0, None, None, None, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_server_destroy(None) == L.OK
    assert lib.ffsrl_create(None, None, 0, C.byref(h)) == L.ERR_INVALID_ARGUMENT and not h.value
    assert lib.ffsrl_create(C.byref(L.Model()), C.byref(L.Params()), 0, C.byref(h)) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_step(None, 1, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_attach_render(None, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_render_handle(None, None, None, 1, None, None, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_destroy(None) == L.OK
    assert lib.ffsrl_graph_begin(None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_graph_launch(None, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_graph_destroy(None) == L.OK
    assert lib.ffsrl_edge_breaker(None, None, None, None, None, 3, 1.0, 0.1, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_update_active_values(None, None, None, 0, 5, None) == L.ERR_INVALID_ARGUMENT
    assert lib.ffsrl_cut_edges(None, None, None, None, None, 2, None, 0, None, None, None, None, None, None,
                               None) == L.ERR_INVALID_ARGUMENT
    # empty work is a no-op
    assert lib.ffsrl_remap(None, None, None, 0, None) == L.OK
    assert lib.ffsrl_heat_propagation(None, None, None, None, 0, 0.1, 0.1, 0.1, None) == L.OK
    # out-of-range faces are rejected by the host BVH build
    pts = np.zeros((3, 3), dtype=np.float32)
    faces = np.array([[0, 1, 7]], dtype=np.int32)
    out = [np.zeros(2, dtype=np.int32) for _ in range(5)]
    nn, ml = C.c_int32(), C.c_int32()
    rc = lib.ffsrl_bvh_build_host(pts.ctypes.data, faces.ctypes.data, 3, 1, 8, *[o.ctypes.data for o in out],
                                  None, None, C.byref(nn), C.byref(ml))
    assert rc == L.ERR_INVALID_ARGUMENT


def test_cpu_model_refuses_gpu_entry_points():
    m = SimModelDO(mg.beam(nx=2, ny=1, nz=1), 2, "cpu")
    with pytest.raises(L.FFSRLError):
        m.transformSimMeshData()
    from ffsrl import SimIntegratorDO
    with pytest.raises(L.FFSRLError):
        SimIntegratorDO("cpu").stepModel(m)


def test_model_concatenation_offsets():
    a = mg.ellipsoid_for_tets(500, seed=1)
    b = mg.ellipsoid_for_tets(900, seed=2)
    m = SimModelDO([a, b, a], 3, "cpu")
    nv = [len(a["vertex"]), len(b["vertex"]), len(a["vertex"])]
    assert m.envVertexStart.tolist() == [0, nv[0], nv[0] + nv[1], sum(nv)]
    tet = m.host["tetrahedron"].reshape(-1, 4)
    env_of_tet = np.repeat(np.arange(3), [len(a["tetrahedron"]), len(b["tetrahedron"]), len(a["tetrahedron"])])
    lo, hi = m.envVertexStart[env_of_tet], m.envVertexStart[env_of_tet + 1]
    assert np.all((tet >= lo[:, None]) & (tet < hi[:, None]))
    ptv = m.host["pointToVertex"].reshape(-1, 2)
    np.testing.assert_array_equal(m.allVisPoint.numpy()[ptv[:, 0]], m.host["vertex"][ptv[:, 1]])
    assert m.envMesh == [0, 1, 0]
    assert m.triToEnv.numpy().tolist() == np.repeat(np.arange(3), [len(a["triangle"]), len(b["triangle"]),
                                                                   len(a["triangle"])]).tolist()


def test_generated_meshes_are_consistent():
    for mesh in (mg.beam(), mg.ellipsoid_for_tets(2000, seed=4)):
        x = mesh["rest_vertex"].astype(np.float64)
        t = mesh["tetrahedron"]
        s6 = np.einsum("ij,ij->i", np.cross(x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]]), x[t[:, 3]] - x[t[:, 0]])
        assert np.all(s6 < 0)
        np.testing.assert_allclose(mesh["tetrahedron_rest_volume"], np.abs(s6) / 6, rtol=1e-5)
        # every surface face is used by exactly one tet face, and the surface is closed
        f = np.sort(mesh["triangle"], axis=1)
        assert len(np.unique(f, axis=0)) == len(f)
        e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [0, 2]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        assert np.all(cnt == 2)
    assert len(mg.beam()["vertex"]) == 275 and len(mg.beam()["tetrahedron"]) == 800
