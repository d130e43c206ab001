"""Synthetic workloads: the instrument stand-in and model builders for the benchmark
configurations (beam, liver-like ellipsoid, mixed-size pools).  Units: cm, g, s.

The reference drives its instrument (a dVRK laparoscope, 7 transforms per env,
``FF_SRL/FF_SRL/modelDO.py:26-416``) from USD; here each env's instrument is three
capsules plus a drag point around an effector point that the caller moves (a seeded
random walk in the benchmarks).  Entry layout per env, as the reference's
``laparoscopeBase/Tip/Radius`` arrays: 0 = rod, 1 = left clamp, 2 = right clamp (its tip
is the point ``dragConstraintsDO`` pulls grasped vertices to), 3 = drag point (the point
``updateClampsDragKernel`` measures from).
"""

from __future__ import annotations

import math

import numpy as np

from . import _lib as L
from . import meshgen as mg
from .model import SimModelDO

KPA = 1.0e4  # 1 kPa in barye (g / (cm s^2))
NH_E, NH_NU = 3.0 * KPA, 0.45


def lame(E: float, nu: float) -> tuple[float, float]:
    mu = E / (2.0 * (1.0 + nu))
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return mu, lam


def instrument_arrays(points, up=(0.0, 1.0, 0.0), radii=(0.3, 0.1, 0.1), rod=12.0, clamp=1.2):
    """base/tip [4N,3] and radius [4N] of instruments whose effector sits at ``points``."""
    p = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    u = np.asarray(up, dtype=np.float64)
    u = u / np.linalg.norm(u)
    side = np.cross(u, [0.0, 0.0, 1.0])
    if np.linalg.norm(side) < 1e-6:
        side = np.cross(u, [1.0, 0.0, 0.0])
    side = side / np.linalg.norm(side) * 0.2
    N = len(p)
    base = np.zeros((N, 4, 3))
    tip = np.zeros((N, 4, 3))
    base[:, 0], tip[:, 0] = p + u * (clamp + rod), p + u * clamp
    base[:, 1], tip[:, 1] = p + u * clamp - side, p - side
    base[:, 2], tip[:, 2] = p + u * clamp + side, p
    base[:, 3], tip[:, 3] = p, p
    rad = np.tile(np.array([radii[0], radii[1], radii[2], 0.0]), N)
    return base.reshape(-1, 3).astype(np.float32), tip.reshape(-1, 3).astype(np.float32), rad.astype(np.float32)


def _frame(z) -> np.ndarray:
    """Rotation whose third column is the unit vector z."""
    z = np.asarray(z, dtype=np.float64)
    z = z / np.linalg.norm(z)
    ref = np.array([1.0, 0.0, 0.0]) if abs(z[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    x = np.cross(ref, z)
    x /= np.linalg.norm(x)
    return np.stack([x, np.cross(z, x), z], axis=1)


def _rt(R, t) -> np.ndarray:
    M = np.eye(4)
    M[:3, :3], M[:3, 3] = R, t
    return M


def _rx(a) -> np.ndarray:
    c, s = np.cos(a), np.sin(a)
    return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])


def instrument_xforms(points, down=(0.0, -1.0, 0.0), radii=(0.3, 0.1, 0.1), rod=12.0, clamp=1.2,
                      clamp_angle=40.0, pivot_depth=None):
    """Kinematic laparoscopes whose drag point (effector) sits at ``points``.

    The instrument's local z runs along ``down`` toward the tissue.  Returns, per env, the
    7 transforms in the library's layout ([N, 112], row-major transposes of column-vector
    transforms; slots 0 rod capsule, 1/2 left/right clamp, 3 rotation centre, 4/5 clamp
    pivots, 6 rod), capsule heights [N, 4] (rod, clamp, clamp, 0), and the initial capsule
    ends base/tip [4N, 3] with radii [4N], computed on the host in float64 as the update
    kernel computes them from the transforms.  The rotation centre (the trocar) sits
    ``pivot_depth`` (default: the rod height) up the axis from the effector; the clamps
    stand at ``clamp_angle`` degrees about their pivots' x axes (40 = closed).
    """
    p = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    N = len(p)
    R = _frame(down)
    z = R[:, 2]
    depth = rod if pivot_depth is None else float(pivot_depth)
    th = np.radians(clamp_angle)
    xf = np.zeros((N, 7, 4, 4))
    ends_b = np.zeros((N, 4, 3))
    ends_t = np.zeros((N, 4, 3))
    for e in range(N):
        c0 = p[e] - z * (0.5 * rod + clamp)         # rod capsule centre
        X0 = _rt(R, c0)
        X3 = _rt(R, p[e] - z * depth)                 # rotation centre
        X4 = _rt(R @ _rx(-th), c0 + z * (0.5 * rod))  # clamp pivots at the rod's end
        X5 = _rt(R @ _rx(th), c0 + z * (0.5 * rod))
        X1 = X4 @ _rt(np.eye(3), np.array([0.0, 0.0, 0.5 * clamp]))
        X2 = X5 @ _rt(np.eye(3), np.array([0.0, 0.0, 0.5 * clamp]))
        for k, M in enumerate((X0, X1, X2, X3, X4, X5, X0)):
            xf[e, k] = M.T  # stored as the transpose, as the reference stores them
        for k, (M, h) in enumerate(((X0, rod), (X1, clamp), (X2, clamp))):
            ends_b[e, k] = (M @ np.array([0.0, 0.0, -h / 1.85, 1.0]))[:3]
            ends_t[e, k] = (M @ np.array([0.0, 0.0, h / 1.85, 1.0]))[:3]
        ends_b[e, 3] = (X0 @ np.array([0.0, 0.0, -0.5 * rod - clamp, 1.0]))[:3]
        ends_t[e, 3] = (X0 @ np.array([0.0, 0.0, 0.5 * rod + clamp, 1.0]))[:3]
    heights = np.tile(np.array([rod, clamp, clamp, 0.0], dtype=np.float32), (N, 1))
    rad = np.tile(np.array([radii[0], radii[1], radii[2], 0.0]), N).astype(np.float32)
    return (xf.reshape(N, 112).astype(np.float32), heights, ends_b.reshape(-1, 3).astype(np.float32),
            ends_t.reshape(-1, 3).astype(np.float32), rad)


def top_surface_point(mesh) -> np.ndarray:
    """The highest surface vertex of a mesh (the default grasp site)."""
    surf = mesh["point_to_vertex"][:, 1]
    v = mesh["vertex"][surf]
    return v[np.argmax(v[:, 1])].astype(np.float64)


def write_liver_scene(path, mesh, rigids=(), dip: float = 0.35, instrument_visual: bool = True) -> None:
    """An array scene file (``ffsrl.scene``) of one soft body with the synthetic instrument
    placed as ``place_instruments`` places it (effector ``dip`` below the highest surface
    point) and its visual mesh."""
    from . import scene as scene_io
    pt = top_surface_point(mesh) - np.array([0.0, dip, 0.0])
    xf, heights, b, t, r = instrument_xforms(pt[None])
    inst = {"transforms": xf.reshape(7, 16), "heights": heights[0], "radii": r, "bases": b, "tips": t}
    if instrument_visual:
        inst.update(mg.instrument_mesh())
    scene_io.write_scene(path, [mesh], rigids=rigids, instrument=inst)


def place_instruments(model: SimModelDO, meshes: list, dip: float = 0.35) -> np.ndarray:
    """Kinematic instrument of env e with its effector ``dip`` cm below mesh e's highest
    surface point, pointing down, clamps closed (their tips then touch the surface);
    returns the effector points."""
    pts = np.stack([top_surface_point(m) - np.array([0.0, dip, 0.0]) for m in meshes])
    xf, heights, b, t, r = instrument_xforms(pts)
    model.setTool(b, t, r)
    model.setInstrument(xf, heights)
    model.toolHost = {"base": b, "tip": t, "radius": r, "xform": xf, "height": heights}
    model.setEffectorInitialPosition()
    return pts


def beam_model(device, num_envs=1, neo=False, xpbd=False, mesh=None, **kw) -> tuple[SimModelDO, list]:
    """Config 0: 10x4x4 beam of 1 cm cubes, 275 vertices, 800 tets, x=0 face fixed,
    1 g/cm^3, dt 1/60, 8 substeps x 10 iterations.  Plain form: the reference DO step with
    kS = 1; the compliant form (xpbd=True) runs XPBD distance (alpha 1e-6) and volume
    (alpha 0)."""
    mesh = mg.beam() if mesh is None else mesh
    flags = L.REFERENCE_STEP
    if xpbd:
        flags = (flags & ~(L.DISTANCE | L.VOLUME)) | L.DISTANCE_XPBD | L.VOLUME_XPBD
    kw.setdefault("environmentGravity", mg.gravity_force(mesh))
    m = SimModelDO(mesh, num_envs, device, simSubsteps=8, simFrameRate=60, simConstraintsSteps=10,
                   environmentGroundLevel=-100.0, constraints=flags, distanceCompliance=1e-6,
                   volumeComplianceXPBD=0.0, **kw)
    return m, [mesh] * num_envs


def liver_model(device, num_envs, meshes=None, E=NH_E, nu=NH_NU, substeps=8, iterations=10, grasp=True,
                collide=True, instrument_visual=True, scene=None, **kw) -> tuple[SimModelDO, list]:
    """Config 1 (meshes=None: the 12/8/6 cm ellipsoid in every env) or a given list
    of meshes (configs 2/4): Neo-Hookean + volume + distance, grasp and contact.  With
    ``instrument_visual`` each env also renders its instrument (``meshgen.instrument_mesh``
    with the dimensions of ``instrument_xforms``).  ``scene``: an array scene file
    (``write_liver_scene``) in every env instead, its instrument included."""
    stage = meshes
    if scene is not None:
        from . import scene as scene_io
        meshes = [scene_io.read_scene(scene).mesh] * num_envs
        stage = scene
    elif meshes is None:
        meshes = stage = [mg.ellipsoid()] * num_envs
    mu, lam = lame(E, nu)
    flags = L.VOLUME | L.DISTANCE | L.NEOHOOKEAN | L.DRAG | (L.COLLIDE if collide else 0)
    kw.setdefault("environmentGravity", mg.gravity_force(meshes[0]))
    if instrument_visual and scene is None:
        kw.setdefault("instrumentMesh", mg.instrument_mesh())
    m = SimModelDO(stage, num_envs, device, simSubsteps=substeps, simFrameRate=60, simConstraintsSteps=iterations,
                   environmentGroundLevel=-100.0, constraints=flags, globalVolumeCompliance=1.0 / lam,
                   globalDeviatoricCompliance=1.0 / mu, globalLaparoscopeDragLookupRadius=0.5, **kw)
    if scene is None:
        place_instruments(m, meshes)
    return m, meshes


def mixed_meshes(num_envs: int, pool_size: int = 64, seed: int = 0, t_lo: int = 500, t_hi: int = 20000):
    """Config 2 pool: ``pool_size`` ellipsoids with tet targets log-uniform in [t_lo, t_hi],
    each env drawing one (seeded).  ``pool_size`` 0 (or the env count) gives every env a
    mesh of its own, as config 2 draws a tet count per env."""
    if pool_size <= 0 or pool_size == num_envs:
        pool = mg.mixed_pool(num_envs, seed=seed, t_lo=t_lo, t_hi=t_hi)
        return list(pool), pool
    pool = mg.mixed_pool(pool_size, seed=seed, t_lo=t_lo, t_hi=t_hi)
    rng = np.random.Generator(np.random.PCG64(seed + 17))
    pick = rng.integers(0, pool_size, size=num_envs)
    return [pool[k] for k in pick], pool


def random_walk_steps(num_envs: int, num_steps: int, step: float = 0.05, seed: int = 0) -> np.ndarray:
    """[num_steps, N, 3] effector displacements of length ``step`` in seeded random directions."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.normal(size=(num_steps, num_envs, 3))
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    return (d * step).astype(np.float32)


def env_cameras(meshes, seed: int = 0, distance: float | None = None):
    """Per-env pinhole poses looking at each mesh's centre from a seeded direction, at
    ``distance`` (default: 2.5 times the mesh's bounding radius)."""
    from .render import look_at_rotation
    rng = np.random.Generator(np.random.PCG64(seed))
    pos, rot = [], []
    for m in meshes:
        c = m["vertex"].mean(axis=0).astype(np.float64)
        dist = distance if distance is not None else 2.5 * float(np.linalg.norm(m["vertex"] - c, axis=1).max())
        az = rng.uniform(0, 2 * math.pi)
        el = rng.uniform(0.3, 1.0)
        d = np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
        p = c + d * dist
        pos.append(p)
        rot.append(look_at_rotation(p, c))
    return np.asarray(pos, dtype=np.float32), np.asarray(rot, dtype=np.float32)


def fov_aperture(fov_deg: float = 60.0) -> float:
    """vertical aperture giving the reference camera (focal 50) a vertical field of view."""
    return 2.0 * 50.0 * math.tan(math.radians(fov_deg) / 2.0)
