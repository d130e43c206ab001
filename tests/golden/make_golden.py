"""Writes the golden fixtures of this folder from the CPU oracle (the C++ restatement of
the reference kernels in oracle/); BVH topologies come from the host builder, which the
tests check against the numpy restatement of the reference build.

Run from the repository root:  python tests/golden/make_golden.py

Each fixture holds its inputs (mesh arrays, instrument, grasp flags, cameras) as well as
the outputs, so the tests rebuild every model from the fixture itself and do not depend
on the mesh generator giving the same floats on another machine.

  beam.npz    config-0 beam (275 vertices, 800 tets), reference step, 25 steps:
              positions and velocities in float32 and positions in float64
  liver3.npz  three small ellipsoids (Neo-Hookean + volume + distance + grasp + contact),
              5 steps: positions and contact counts
  render.npz  the liver3 end state: BVH topologies, refit boxes and 16x16 colour/depth
              images from per-env cameras
  scene.npz   three envs of one textured ellipsoid with a static rigid box under it and
              the instrument's visual mesh (the multi-object layout): the instrument moved
              by seeded actions, 3 steps, then visual points, the refit's face-shift
              table, BVH topology and boxes, and 16x16 images in the texture, vertex-colour
              and grayscale modes
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for p in (ROOT / "ff-srl_gb300", ROOT / "oracle"):
    sys.path.insert(0, str(p))

import torch  # noqa: E402

import oracle  # noqa: E402
from ffsrl import SimBVH, WarpRaycastRendererDO  # noqa: E402
from ffsrl import meshgen as mg  # noqa: E402
from ffsrl import scenarios as sc  # noqa: E402

MESH_KEYS = ("vertex", "rest_vertex", "inverse_mass", "tetrahedron", "tetrahedron_rest_volume",
             "tetrahedron_rest_volume_signed", "tetrahedron_dm_inv", "edge", "edge_rest_length", "triangle",
             "vis_face", "point_to_vertex", "vis_point_color", "fixed")
BEAM_STEPS = 25
LIVER_STEPS = 5
RES = 16
GRASP_RADIUS = 0.5


def pack_meshes(meshes) -> dict:
    out = {"num_meshes": np.int32(len(meshes))}
    for k, m in enumerate(meshes):
        for key in MESH_KEYS:
            out[f"mesh{k}_{key}"] = np.asarray(m[key])
    return out


def unpack_meshes(z) -> list:
    return [{key: np.asarray(z[f"mesh{k}_{key}"]) for key in MESH_KEYS} for k in range(int(z["num_meshes"]))]


def grasp_flags(model, radius: float = GRASP_RADIUS) -> np.ndarray:
    """The grasp of graspNearest on the host: per env, the surface vertex nearest the
    drag point (instrument entry 3) within ``radius``."""
    x = np.asarray(model.host["vertex"], dtype=np.float64).reshape(-1, 3)
    tip = np.asarray(model.toolHost["tip"], dtype=np.float64).reshape(-1, 3)
    ptv = np.asarray(model.host["pointToVertex"]).reshape(-1, 2)
    drag = np.zeros(model.numVertices, dtype=np.float32)
    for e in range(model.numEnvs):
        v0, v1 = int(model.envVertexStart[e]), int(model.envVertexStart[e + 1])
        cand = np.unique(ptv[:, 1][(ptv[:, 1] >= v0) & (ptv[:, 1] < v1)])
        d = np.linalg.norm(x[cand] - tip[4 * e + 3], axis=1)
        if len(d) and d.min() < radius:
            drag[cand[np.argmin(d)]] = 1.0
    return drag


def liver_model(device, meshes):
    return sc.liver_model(device, len(meshes), meshes=meshes, instrument_visual=False)[0]


def renderer(device, model, meshes):
    ap = sc.fov_aperture(60.0)
    r = WarpRaycastRendererDO(device, model, resolution=RES, mode="headless", verticalAperture=ap,
                              horizontalAperture=ap, lightPos=(0.3, 1.0, 0.5), lightIntensity=0.8)
    pos, rot = sc.env_cameras(meshes, seed=1)
    r.setCameras(pos, rot)
    return r


def make_beam() -> dict:
    mesh = mg.beam()
    m, _ = sc.beam_model("cpu", mesh=mesh)
    o = oracle.OracleSim(m)
    o.step(BEAM_STEPS)
    V = m.numVertices
    x64 = np.asarray(m.host["vertex"], dtype=np.float64).reshape(-1, 3).copy()
    xp64, v64 = np.zeros((V, 3)), np.zeros((V, 3))
    oracle.OracleSim(m).step_f64(BEAM_STEPS, x64, xp64, v64)
    return pack_meshes([mesh]) | {"steps": np.int32(BEAM_STEPS), "vertex": o.a["vertex"].copy(),
                                  "velocity": o.a["velocity"].copy(), "vertex_f64": x64}


def make_liver() -> tuple[dict, list, object, object]:
    pool = [mg.ellipsoid_for_tets(t, seed=20 + i) for i, t in enumerate((300, 550, 800))]
    m = liver_model("cpu", pool)
    drag = grasp_flags(m)
    o = oracle.OracleSim(m, {"active_drag_constraint": drag})
    o.step(LIVER_STEPS)
    fix = pack_meshes(pool) | {
        "steps": np.int32(LIVER_STEPS), "drag": drag, "tool_base": np.asarray(m.toolHost["base"], np.float32),
        "tool_tip": np.asarray(m.toolHost["tip"], np.float32),
        "tool_radius": np.asarray(m.toolHost["radius"], np.float32),
        "vertex": o.a["vertex"].copy(), "in_collision": o.a["laparoscope_in_collision"].copy()}
    return fix, pool, m, o


def make_render(pool, m, o) -> dict:
    bvh = SimBVH("cpu", m)  # topology from the rest-state visual points, as the tests build it
    vis = o.vis_points()
    lo, hi = oracle.refit(bvh, vis, m.host["allVisFace"])
    r = renderer("cpu", m, pool)
    col, dep, nrm = oracle.render(r, bvh, vis, aabb=(lo, hi))
    out = {"vis_point": vis, "aabb_min": lo, "aabb_max": hi, "color": col, "depth": dep, "normal": nrm,
           "camera_pos": r.cameraPosT.cpu().numpy(), "camera_rot": r.cameraRotT.cpu().numpy()}
    for k, t in enumerate(bvh.topologies):
        for key in ("left_node", "first_tri_id", "tri_count", "level", "tri_id"):
            out[f"topo{k}_{key}"] = np.asarray(t[key])
    return out


SCENE_STEPS = 3
SCENE_ENVS = 3
SCENE_MODES = (1, 3, 0)
INSTRUMENT_KEYS = ("points", "faces", "slot", "color")
TEXTURE_KEYS = ("texture", "tex_coords", "tex_indices")
RIGID_KEYS = ("vertex", "triangle", "color")


def scene_inputs() -> tuple[dict, dict]:
    """The scene's soft mesh (textured, one rigid box under it) and instrument mesh."""
    base = mg.ellipsoid_for_tets(500, seed=31)
    lo, hi = base["vertex"].min(axis=0), base["vertex"].max(axis=0)
    box = mg.rigid_box([lo[0] - 2.0, lo[1] - 1.0, lo[2] - 2.0], [hi[0] + 2.0, lo[1] - 0.5, hi[2] + 2.0])
    mesh = mg.with_rigids(mg.add_texture(base, size=16, seed=3), [box])
    return mesh, mg.instrument_mesh()


def pack_scene(mesh, inst) -> dict:
    out = pack_meshes([mesh])
    for key in TEXTURE_KEYS:
        out[f"mesh0_{key}"] = np.asarray(mesh[key])
    for key in RIGID_KEYS:
        out[f"rigid0_{key}"] = np.asarray(mesh["rigids"][0][key])
    for key in INSTRUMENT_KEYS:
        out[f"instrument_{key}"] = np.asarray(inst[key])
    return out


def unpack_scene(z) -> tuple[dict, dict]:
    mesh = unpack_meshes(z)[0]
    for key in TEXTURE_KEYS:
        mesh[key] = np.asarray(z[f"mesh0_{key}"])
    mesh["rigids"] = [{key: np.asarray(z[f"rigid0_{key}"]) for key in RIGID_KEYS}]
    return mesh, {key: np.asarray(z[f"instrument_{key}"]) for key in INSTRUMENT_KEYS}


def scene_model(device, mesh, inst):
    return sc.liver_model(device, SCENE_ENVS, meshes=[mesh] * SCENE_ENVS, instrumentMesh=inst)[0]


def make_scene() -> dict:
    mesh, inst = scene_inputs()
    m = scene_model("cpu", mesh, inst)
    # rest-state visual points with the instrument at its initial pose: the BVH build's input
    vis0 = oracle.OracleSim(m).vis_points(oracle.OracleInstrument.from_model(m))
    m.allVisPoint.copy_(torch.as_tensor(vis0))
    bvh = SimBVH("cpu", m)
    oi = oracle.OracleInstrument.from_model(m)
    rng = np.random.default_rng(5)
    for _ in range(4):
        a = rng.uniform(-0.05, 0.05, size=(SCENE_ENVS, 5)).astype(np.float32)
        a[:, 4] = 0.0  # the clamps stay closed
        oi.apply_actions(a)
    drag = grasp_flags(m)
    o = oracle.OracleSim(m, {"active_drag_constraint": drag, "laparoscope_base": oi.base,
                             "laparoscope_tip": oi.tip})
    o.step(SCENE_STEPS)
    vis = o.vis_points(oi)
    src = oracle.reference_refit_source(SCENE_ENVS, m.numEnvMeshesVisFaces, m.numEnvRigidsVisFaces,
                                        m.numEnvLaparoscopeVisFaces, m.envVisFaceStart[:-1])
    assert np.array_equal(bvh.refitSource.numpy(), src)
    lo, hi = oracle.refit(bvh, vis, m.host["allVisFace"])
    r = renderer("cpu", m, [mesh] * SCENE_ENVS)
    out = pack_scene(mesh, inst) | {
        "steps": np.int32(SCENE_STEPS), "drag": drag, "xform": oi.xform.copy(), "height": oi.height.copy(),
        "tool_base": oi.base.copy(), "tool_tip": oi.tip.copy(), "vertex": o.a["vertex"].copy(),
        "vis_point_rest": vis0, "vis_point": vis, "refit_source": src, "aabb_min": lo, "aabb_max": hi,
        "camera_pos": r.cameraPosT.cpu().numpy(), "camera_rot": r.cameraRotT.cpu().numpy()}
    for mode in SCENE_MODES:
        r.render_mode = mode
        col, dep, _ = oracle.render(r, bvh, vis, aabb=(lo, hi))
        out[f"color_mode{mode}"], out["depth"] = col, dep
    for key in ("left_node", "first_tri_id", "tri_count", "level", "tri_id"):
        out[f"topo0_{key}"] = np.asarray(bvh.topologies[0][key])
    return out


def main() -> None:
    np.savez_compressed(HERE / "beam.npz", **make_beam())
    fix, pool, m, o = make_liver()
    np.savez_compressed(HERE / "liver3.npz", **fix)
    np.savez_compressed(HERE / "render.npz", **make_render(pool, m, o))
    np.savez_compressed(HERE / "scene.npz", **make_scene())
    for f in ("beam.npz", "liver3.npz", "render.npz", "scene.npz"):
        print(f, (HERE / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
