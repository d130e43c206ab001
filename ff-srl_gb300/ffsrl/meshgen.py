"""Synthetic tetrahedral meshes standing in for the reference's USD scenes.

The reference loads its soft bodies from USD (``FF_SRL/FF_SRL/modelDO.py:545-640``:
``extMesh:vertex``, ``extMesh:tetrahedron``, ``extMesh:edge``, rest volumes and rest
lengths, inverse masses, a separate visual mesh and its ``pointToVertex`` map).  USD
cannot be read here, and the reference ships no tetrahedraliser, so this module builds
the same arrays from two seeded generators:

* ``beam``: an nx*ny*nz grid of cubes, 5 tets per cube with alternating parity (a
  conforming split), the x=0 face fixed.
* ``ellipsoid``: a jittered cubic grid clipped to an ellipsoid, same 5-tet split, the
  lowest 5% of vertices (by y) fixed.

Units are centimetres, grams and seconds.  The reference's kernels assume centimetre
scenes: the ray/triangle test rejects |det| < 1e-4 (``FF_SRL/FF_SRL/render.py:677``),
depth is written as t/50 (``render.py:401``), and its demo camera sits at (0, 50, 50)
(``FF_SRL/FF_SRL/tests/testLiverRetraction.py:51``).

Conventions the reference's kernels depend on:

* Tets are oriented with NEGATIVE signed volume ``dot(cross(pB-pA, pC-pA), pD-pA)``.
  The reference's PBD volume constraint (``FF_SRL/FF_SRL/integrator.py:480-494``) uses
  ``C = V0 - |vol|`` with the unsigned gradient ``q_i``; it restores volume only for
  that orientation and pushes the other way for positively oriented tets.
* Inverse masses are lumped: ``m_v = rho * sum_{tets containing v} V0 / 4``; fixed
  vertices get 0.  (The reference reads ``extMesh:inverseMass`` from USD,
  ``FF_SRL/FF_SRL/modelDO.py:591``.)
* ``Dm^-1`` (inverse rest-shape matrix, columns = rest edge vectors) is computed in
  float64 and stored row-major as 9 float32 per tet.
* Edges are the unique tet edges; the surface is the set of tet faces used once,
  oriented outward; the visual mesh is the surface, with its own compact point index
  and a ``point_to_vertex`` map (``FF_SRL/FF_SRL/utils.py:32-42``).
"""

from __future__ import annotations

import numpy as np

# 5-tet split of a unit cube.  Corner (i,j,k) has local id i + 2j + 4k.
_EVEN = np.array([[0, 1, 2, 4], [3, 1, 2, 7], [5, 1, 4, 7], [6, 2, 4, 7], [1, 2, 4, 7]], dtype=np.int64)
_ODD = np.array([[1, 0, 3, 5], [2, 0, 3, 6], [4, 0, 5, 6], [7, 3, 5, 6], [0, 3, 5, 6]], dtype=np.int64)
_TET_FACES = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]], dtype=np.int64)
_TET_FACE_OPP = np.array([3, 2, 1, 0], dtype=np.int64)
_TET_EDGES = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]], dtype=np.int64)


def _grid_tets(cells: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Tets (as grid-point ids) for the boolean cell mask ``cells[nx,ny,nz]``."""
    nx, ny, nz = cells.shape
    gi, gj, gk = np.nonzero(cells)
    npy, npz = ny + 1, nz + 1

    def gid(i, j, k):
        return (i * npy + j) * npz + k

    corners = np.stack([gid(gi + (c & 1), gj + ((c >> 1) & 1), gk + ((c >> 2) & 1)) for c in range(8)], axis=1)
    parity = (gi + gj + gk) & 1
    tets = np.empty((len(gi), 5, 4), dtype=np.int64)
    even = parity == 0
    tets[even] = corners[even][:, _EVEN]
    tets[~even] = corners[~even][:, _ODD]
    return tets.reshape(-1, 4), np.array([nx + 1, ny + 1, nz + 1])


def _signed6(p: np.ndarray, t: np.ndarray) -> np.ndarray:
    a, b, c, d = (p[t[:, i]] for i in range(4))
    return np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a)


def finalize_mesh(points: np.ndarray, tets: np.ndarray, density: float, fixed: np.ndarray,
                  initial: np.ndarray | None = None, color=(0.75, 0.25, 0.2)) -> dict:
    """Build every per-mesh array the step, BVH and renderer read.

    ``points`` are the rest positions (float64), ``tets`` grid-point ids, ``fixed`` a
    boolean mask over ``points``.  Unused points are dropped.  ``initial`` (same shape
    as points) optionally gives starting positions that differ from the rest state.
    """
    used = np.zeros(len(points), dtype=bool)
    used[tets.ravel()] = True
    remap = -np.ones(len(points), dtype=np.int64)
    remap[used] = np.arange(used.sum())
    tets = remap[tets]
    rest = points[used]
    start = rest if initial is None else initial[used]
    fixed = fixed[used]

    # negative orientation (see module docstring)
    s6 = _signed6(rest, tets)
    flip = s6 > 0
    tets[flip] = tets[flip][:, [0, 2, 1, 3]]
    s6 = _signed6(rest, tets)
    assert np.all(s6 < 0), "degenerate tet in generator"
    rest_vol = np.abs(s6) / 6.0

    nv = len(rest)
    mass = np.zeros(nv)
    np.add.at(mass, tets.ravel(), np.repeat(rest_vol * density / 4.0, 4))
    inv_mass = np.where(fixed | (mass <= 0), 0.0, 1.0 / np.maximum(mass, 1e-300))

    # unique edges (sorted id pairs, lexicographic; one int64 key per pair)
    e = np.sort(tets[:, _TET_EDGES].reshape(-1, 2), axis=1)
    ekey = np.unique(e[:, 0] * nv + e[:, 1])
    edges = np.stack([ekey // nv, ekey % nv], axis=1)
    rest_len = np.linalg.norm(rest[edges[:, 1]] - rest[edges[:, 0]], axis=1)

    # boundary faces (used by one tet), oriented away from the opposite vertex
    faces = tets[:, _TET_FACES].reshape(-1, 3)
    opp = tets[:, _TET_FACE_OPP].reshape(-1)
    key = np.sort(faces, axis=1)
    fkey = (key[:, 0] * nv + key[:, 1]) * nv + key[:, 2]
    _, inv, cnt = np.unique(fkey, return_inverse=True, return_counts=True)
    bnd = cnt[inv.ravel()] == 1
    faces, opp = faces[bnd], opp[bnd]
    a, b, c = rest[faces[:, 0]], rest[faces[:, 1]], rest[faces[:, 2]]
    n = np.cross(b - a, c - a)
    inward = np.einsum("ij,ij->i", n, rest[opp] - a) > 0
    faces[inward] = faces[inward][:, [0, 2, 1]]
    # order faces by their lowest vertex for locality
    order = np.lexsort((faces[:, 2], faces[:, 1], faces.min(axis=1)))
    faces = faces[order]

    # Dm^-1, columns of Dm = rest edges from vertex A; float64 then float32
    pa = rest[tets[:, 0]]
    dm = np.stack([rest[tets[:, 1]] - pa, rest[tets[:, 2]] - pa, rest[tets[:, 3]] - pa], axis=2)
    dm_inv = np.linalg.inv(dm)

    # visual mesh = surface points, compact numbering in order of first use by vertex id
    surf_pts = np.unique(faces.ravel())
    vis_of = -np.ones(nv, dtype=np.int64)
    vis_of[surf_pts] = np.arange(len(surf_pts))
    vis_face = vis_of[faces]
    point_to_vertex = np.stack([np.arange(len(surf_pts)), surf_pts], axis=1)
    # deterministic per-point colour variation
    h = ((surf_pts * 2654435761) % 1000) / 1000.0
    colors = np.clip(np.array(color)[None, :] * (0.85 + 0.3 * h[:, None]), 0.0, 1.0)

    return {
        "vertex": start.astype(np.float32),
        "rest_vertex": rest.astype(np.float32),
        "inverse_mass": inv_mass.astype(np.float32),
        "tetrahedron": tets.astype(np.int32),
        "tetrahedron_rest_volume": rest_vol.astype(np.float32),
        "tetrahedron_rest_volume_signed": (s6 / 6.0).astype(np.float32),
        "tetrahedron_dm_inv": dm_inv.reshape(-1, 9).astype(np.float32),
        "edge": edges.astype(np.int32),
        "edge_rest_length": rest_len.astype(np.float32),
        "triangle": faces.astype(np.int32),
        "vis_face": vis_face.astype(np.int32),
        "point_to_vertex": point_to_vertex.astype(np.int32),
        "vis_point_color": colors.astype(np.float32),
        "fixed": fixed,
    }


def beam(nx: int = 10, ny: int = 4, nz: int = 4, h: float = 1.0, density: float = 1.0,
         jitter: float = 1e-2, seed: int = 0, origin=(0.0, 10.0, 0.0)) -> dict:
    """Cantilever beam: (nx+1)(ny+1)(nz+1) vertices, 5*nx*ny*nz tets, x=0 face fixed.

    Defaults: 1 cm cubes, 1 g/cm^3.  The rest state is the regular grid; the initial
    positions carry a seeded uniform jitter of +-``jitter`` cm (numpy PCG64, ``seed``).
    """
    cells = np.ones((nx, ny, nz), dtype=bool)
    tets, dims = _grid_tets(cells)
    ii, jj, kk = np.meshgrid(np.arange(dims[0]), np.arange(dims[1]), np.arange(dims[2]), indexing="ij")
    pts = np.stack([ii, jj, kk], axis=-1).reshape(-1, 3) * h + np.asarray(origin, dtype=np.float64)
    rng = np.random.Generator(np.random.PCG64(seed))
    init = pts + rng.uniform(-jitter, jitter, size=pts.shape)
    fixed = ii.reshape(-1) == 0
    return finalize_mesh(pts, tets, density, fixed, initial=init)


def _ellipsoid_cells(a: np.ndarray, h: float):
    n = np.ceil(2 * a / h).astype(int) + 2
    lo = -(n * h) / 2.0
    gx, gy, gz = (lo[d] + h * np.arange(n[d] + 1) for d in range(3))
    X, Y, Z = np.meshgrid(gx, gy, gz, indexing="ij")
    ins = ((X / a[0]) ** 2 + (Y / a[1]) ** 2 + (Z / a[2]) ** 2 <= 1.0).astype(np.int32)
    corner_count = sum(ins[di:di + n[0], dj:dj + n[1], dk:dk + n[2]]
                       for di in (0, 1) for dj in (0, 1) for dk in (0, 1))
    return corner_count >= 8, (X, Y, Z)


def ellipsoid(semi_axes=(12.0, 8.0, 6.0), h: float = 0.6, density: float = 1.06,
              jitter_frac: float = 0.1, seed: int = 0, fixed_frac: float = 0.05,
              origin=(0.0, 10.0, 0.0)) -> dict:
    """Ellipsoid on a jittered cubic grid (spacing ``h``), lowest ``fixed_frac`` by y fixed.

    A cell is kept when all 8 of its (unjittered) corners lie inside the ellipsoid.
    Grid points are jittered by U(+-jitter_frac*h) per axis; the jittered grid is the
    rest state.  For the default 12/8/6 cm, h = 0.6 cm this gives 11,102 vertices and
    46,640 tets.
    """
    a = np.asarray(semi_axes, dtype=np.float64)
    cells, (X, Y, Z) = _ellipsoid_cells(a, h)
    tets, dims = _grid_tets(cells)
    pts = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = pts + rng.uniform(-jitter_frac * h, jitter_frac * h, size=pts.shape)
    pts = pts + np.asarray(origin, dtype=np.float64)
    used = np.zeros(len(pts), dtype=bool)
    used[tets.ravel()] = True
    y = pts[:, 1]
    thr = np.quantile(y[used], fixed_frac)
    fixed = y <= thr
    return finalize_mesh(pts, tets, density, fixed)


def ellipsoid_for_tets(target_tets: int, seed: int = 0, h: float = 0.6, **kw) -> dict:
    """Ellipsoid with semi-axes 12/8/6 cm times one scale factor, chosen by bisection so
    that the tet count (5 per kept cell) is the closest to ``target_tets``."""
    base = np.array([12.0, 8.0, 6.0])
    lo, hi = 0.05, 3.0
    for _ in range(30):
        mid = 0.5 * (lo + hi)
        if 5 * int(_ellipsoid_cells(base * mid, h)[0].sum()) < target_tets:
            lo = mid
        else:
            hi = mid
    best = min((lo, hi), key=lambda s: abs(5 * int(_ellipsoid_cells(base * s, h)[0].sum()) - target_tets))
    return ellipsoid(semi_axes=tuple(base * best), h=h, seed=seed, **kw)


_WORKER_MODULE = "_ffsrl_meshgen_worker"


def _load_standalone():
    """This file as a module of its own (numpy only): what the pool workers run, so that
    they import neither torch nor the CUDA library."""
    import importlib.util
    import sys
    mod = sys.modules.get(_WORKER_MODULE)
    if mod is None:
        spec = importlib.util.spec_from_file_location(_WORKER_MODULE, __file__)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[_WORKER_MODULE] = mod
        spec.loader.exec_module(mod)
    return mod


def _ellipsoid_job(args):
    target, seed = args
    return ellipsoid_for_tets(target, seed=seed)


def mixed_pool(num_meshes: int, seed: int = 0, t_lo: int = 500, t_hi: int = 20000, workers: int = 0) -> list[dict]:
    """``num_meshes`` ellipsoids with tet targets drawn log-uniform in [t_lo, t_hi].

    ``workers`` > 1 builds them in that many spawned processes (0: one per host core for
    pools of 256 meshes or more); the meshes are the same either way."""
    rng = np.random.Generator(np.random.PCG64(seed))
    targets = np.exp(rng.uniform(np.log(t_lo), np.log(t_hi), size=num_meshes))
    jobs = [(int(t), seed * 1000 + i) for i, t in enumerate(targets)]
    if workers == 0:
        import os
        workers = (os.cpu_count() or 1) if num_meshes >= 256 else 1
    if workers <= 1:
        return [_ellipsoid_job(j) for j in jobs]
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    mod = _load_standalone()
    with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn"), initializer=_load_standalone) as ex:
        return list(ex.map(mod._ellipsoid_job, jobs, chunksize=max(1, len(jobs) // (4 * workers))))


def gravity_force(meshes, g: float = -981.0) -> tuple[float, float, float]:
    """The reference's ``gravity`` kernel multiplies the gravity vector by each vertex's
    inverse mass (``FF_SRL/FF_SRL/integrator.py:56``), so ``environmentGravity`` acts as a
    force per vertex.  This returns the force that gives a vertex of the mean (free)
    vertex mass of ``meshes`` the acceleration ``g`` along y."""
    if isinstance(meshes, dict):
        meshes = [meshes]
    inv = np.concatenate([m["inverse_mass"] for m in meshes])
    mbar = float(np.mean(1.0 / inv[inv > 0]))
    return (0.0, g * mbar, 0.0)


def tiny_mesh(vertex, tetrahedron=(), edge=(), triangle=(), inverse_mass=None) -> dict:
    """A hand-made mesh dict (for known-answer tests): rest state = ``vertex``; rest
    volumes, rest lengths and Dm^-1 follow from it; the visual mesh is ``triangle``."""
    x = np.asarray(vertex, dtype=np.float64).reshape(-1, 3)
    t = np.asarray(tetrahedron, dtype=np.int64).reshape(-1, 4)
    e = np.asarray(edge, dtype=np.int64).reshape(-1, 2)
    f = np.asarray(triangle, dtype=np.int64).reshape(-1, 3)
    nv = len(x)
    s6 = _signed6(x, t) if len(t) else np.zeros(0)
    if len(t):
        pa = x[t[:, 0]]
        dm = np.stack([x[t[:, 1]] - pa, x[t[:, 2]] - pa, x[t[:, 3]] - pa], axis=2)
        dm_inv = np.linalg.inv(dm).reshape(-1, 9)
    else:
        dm_inv = np.zeros((0, 9))
    surf = np.unique(f.ravel()) if len(f) else np.zeros(0, dtype=np.int64)
    vis_of = -np.ones(nv, dtype=np.int64)
    vis_of[surf] = np.arange(len(surf))
    inv = np.ones(nv) if inverse_mass is None else np.asarray(inverse_mass, dtype=np.float64)
    return {
        "vertex": x.astype(np.float32), "rest_vertex": x.astype(np.float32),
        "inverse_mass": inv.astype(np.float32),
        "tetrahedron": t.astype(np.int32),
        "tetrahedron_rest_volume": (np.abs(s6) / 6.0).astype(np.float32),
        "tetrahedron_rest_volume_signed": (s6 / 6.0).astype(np.float32),
        "tetrahedron_dm_inv": dm_inv.astype(np.float32),
        "edge": e.astype(np.int32),
        "edge_rest_length": np.linalg.norm(x[e[:, 1]] - x[e[:, 0]], axis=1).astype(np.float32) if len(e) else
        np.zeros(0, dtype=np.float32),
        "triangle": f.astype(np.int32),
        "vis_face": vis_of[f].astype(np.int32) if len(f) else np.zeros((0, 3), dtype=np.int32),
        "point_to_vertex": np.stack([np.arange(len(surf)), surf], axis=1).astype(np.int32) if len(surf) else
        np.zeros((0, 2), dtype=np.int32),
        "vis_point_color": np.full((len(surf), 3), 0.5, dtype=np.float32),
        "fixed": inv == 0,
    }


def add_texture(mesh: dict, size: int = 64, seed: int = 0, per_corner: bool = False) -> dict:
    """A copy of ``mesh`` with a texture, standing in for a USD material's diffuse texture
    (``FF_SRL/FF_SRL/modelDO.py:628-640``).

    ``texture`` [size, size, 3] in [0, 1] is a seeded smooth tissue-like pattern (stripes
    plus blotches).  ``tex_coords`` are a planar projection of the rest shape onto its x/z
    extent, one per visual point, and ``tex_indices`` is ``vis_face`` (the reference's
    default when the mesh carries no ``primvars:st:indices``).  With ``per_corner`` the
    coordinates are one per face corner instead, with their own ``tex_indices`` (the
    indexed-primvar form)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = np.linspace(0.0, 1.0, size)
    X, Y = np.meshgrid(g, g, indexing="ij")
    field = 0.5 + 0.25 * np.sin(2 * np.pi * (3 * X + rng.uniform())) * np.cos(2 * np.pi * (2 * Y + rng.uniform()))
    for _ in range(6):
        cx, cy, r = rng.uniform(0, 1), rng.uniform(0, 1), rng.uniform(0.05, 0.2)
        field += 0.2 * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * r * r))
    tint = np.array([0.75, 0.28, 0.25]) + rng.uniform(-0.05, 0.05, size=3)
    tex = np.clip(field[..., None] * tint[None, None, :] * 1.3, 0.0, 1.0).astype(np.float32)
    rest = mesh["rest_vertex"] if "rest_vertex" in mesh else mesh["vertex"]
    p = np.asarray(rest, dtype=np.float64)[np.asarray(mesh["point_to_vertex"])[:, 1]]
    lo, hi = p.min(axis=0), p.max(axis=0)
    span = np.where(hi - lo > 0, hi - lo, 1.0)
    uv = np.stack([(p[:, 0] - lo[0]) / span[0], (p[:, 2] - lo[2]) / span[2]], axis=1)
    out = dict(mesh)
    out["texture"] = tex
    if per_corner:
        out["tex_coords"] = uv[np.asarray(mesh["vis_face"]).reshape(-1)].astype(np.float32)
        out["tex_indices"] = np.arange(out["tex_coords"].shape[0], dtype=np.int32)
    else:
        out["tex_coords"] = uv.astype(np.float32)
        out["tex_indices"] = np.asarray(mesh["vis_face"], dtype=np.int32).reshape(-1)
    return out


def _outward(points: np.ndarray, faces: np.ndarray, centre) -> np.ndarray:
    """Flip the faces of a star-shaped surface (about ``centre``) whose normals point inward."""
    p = points[faces]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    inward = np.einsum("ij,ij->i", n, p.mean(axis=1) - np.asarray(centre)) < 0
    faces = faces.copy()
    faces[inward] = faces[inward][:, [0, 2, 1]]
    return faces


def capsule(radius: float = 1.0, height: float = 1.0, sections=(10, 10)) -> tuple[np.ndarray, np.ndarray]:
    """Triangle mesh of a capsule along z, centred at the origin: a cylinder of ``height``
    between two hemispheres of ``radius``.  ``sections`` = (latitude rings over both caps,
    segments around).  The reference generates its instrument capsules with
    ``trimesh.creation.capsule`` (``utils.py:105-107``, not available here); this is a
    tessellation of the same solid, with poles, ``sections[0] // 2`` rings per cap and
    outward faces."""
    nlat, nlon = max(1, int(sections[0]) // 2), max(3, int(sections[1]))
    rings = []
    for k in range(1, nlat + 1):          # bottom cap, from below the equator up to it
        a = -0.5 * np.pi + 0.5 * np.pi * k / nlat
        rings.append((-0.5 * height + radius * np.sin(a), radius * np.cos(a)))
    for k in range(0, nlat):              # top cap, from the equator up
        a = 0.5 * np.pi * k / nlat
        rings.append((0.5 * height + radius * np.sin(a), radius * np.cos(a)))
    phi = 2.0 * np.pi * np.arange(nlon) / nlon
    pts = [[0.0, 0.0, -0.5 * height - radius]]
    for zr, rr in rings:
        pts += [[rr * np.cos(f), rr * np.sin(f), zr] for f in phi]
    pts.append([0.0, 0.0, 0.5 * height + radius])
    pts = np.asarray(pts, dtype=np.float64)
    top = len(pts) - 1
    ring = lambda i, j: 1 + i * nlon + (j % nlon)
    faces = [[0, ring(0, j + 1), ring(0, j)] for j in range(nlon)]
    for i in range(len(rings) - 1):
        for j in range(nlon):
            a, b, c, d = ring(i, j), ring(i, j + 1), ring(i + 1, j + 1), ring(i + 1, j)
            faces += [[a, b, c], [a, c, d]]
    faces += [[top, ring(len(rings) - 1, j), ring(len(rings) - 1, j + 1)] for j in range(nlon)]
    return pts, _outward(pts, np.asarray(faces, dtype=np.int64), (0.0, 0.0, 0.0))


def instrument_mesh(rod: float = 12.0, clamp: float = 1.2, radii=(0.15, 0.05, 0.05), sections=(10, 10),
                    colors=((0.55, 0.55, 0.6), (0.75, 0.75, 0.8), (0.75, 0.75, 0.8)),
                    offsets=(0.0, 0.5, 0.5)) -> dict:
    """Visual mesh of a laparoscope: rod, left clamp and right clamp capsules
    (``laparoscope.py:388-422``), each in the frame of its transform slot -- 6 (rod), 4 and
    5 (clamp pivots), as ``modelDO.py:1031-1033`` assigns them -- and shifted along its z
    by ``offsets`` x its height.  The reference shifts its generated capsules by -h/2 to
    suit its USD frames (``laparoscope.py:402``); for the synthetic instrument of
    ``scenarios.instrument_xforms`` the rod frame is the capsule's centre (shift 0) and
    each clamp starts at its pivot (shift +h/2), so the visual mesh covers the contact
    capsules.  Visual radii are half the contact radii (the reference doubles them for
    contact, ``laparoscope.py:378``)."""
    pts, faces, slot, col = [], [], [], []
    n0 = 0
    for h, r, s, off, c in zip((rod, clamp, clamp), radii, (6, 4, 5), offsets, colors):
        p, f = capsule(r, h, sections)
        p = p + np.array([0.0, 0.0, off * h])
        pts.append(p)
        faces.append(f + n0)
        slot.append(np.full(len(p), s, dtype=np.int32))
        col.append(np.tile(np.asarray(c, dtype=np.float32), (len(p), 1)))
        n0 += len(p)
    return {"points": np.concatenate(pts).astype(np.float32), "faces": np.concatenate(faces).astype(np.int32),
            "slot": np.concatenate(slot), "color": np.concatenate(col)}


def rigid_box(lo, hi, color=(0.45, 0.35, 0.3)) -> dict:
    """A static axis-aligned box (12 outward triangles) as a rigid visual object, e.g. the
    table or the abdominal wall under an organ (the reference's ``SimRigidDO``)."""
    lo, hi = np.asarray(lo, dtype=np.float64), np.asarray(hi, dtype=np.float64)
    c = np.array([[(hi if (k >> d) & 1 else lo)[d] for d in range(3)] for k in range(8)])
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    f = np.array([[q[0], q[1], q[2]] for q in quads] + [[q[0], q[2], q[3]] for q in quads], dtype=np.int64)
    f = _outward(c, f, 0.5 * (lo + hi))
    return {"vertex": c.astype(np.float32), "triangle": f.astype(np.int32),
            "color": np.tile(np.asarray(color, dtype=np.float32), (8, 1))}


def with_rigids(mesh: dict, rigids) -> dict:
    """A copy of ``mesh`` carrying static rigid visual objects (``rigid_box`` dicts)."""
    out = dict(mesh)
    out["rigids"] = list(rigids)
    return out


def connect_meshes(a: dict, b: dict, radius: float, kind: str = "centroid") -> dict:
    """One soft body of two meshes with connectors (the reference's ``SimConnectorDO``,
    ``modelDO.py:723-770``): every surface vertex of ``a`` within ``radius`` of a surface
    triangle centroid of ``b`` is held to the nearest such centroid (barycentric
    (1/3, 1/3, 1/3)), its rest distance the current one.  Ids are those of the merged
    body (``a``'s vertices first)."""
    from .scene import merge_meshes
    out = dict(merge_meshes([a, b]))
    nva = len(a["vertex"])
    pa = np.asarray(a["vertex"], dtype=np.float64)
    pb = np.asarray(b["vertex"], dtype=np.float64)
    tri = np.asarray(b["triangle"], dtype=np.int64).reshape(-1, 3)
    cen = pb[tri].mean(axis=1)
    surf = np.unique(np.asarray(a["point_to_vertex"])[:, 1])
    vid, tid, dist = [], [], []
    for v in surf:
        d = np.linalg.norm(cen - pa[v], axis=1)
        k = int(np.argmin(d))
        if d[k] < radius:
            vid.append(int(v))
            tid.append(tri[k] + nva)
            dist.append(float(d[k]))
    c = len(vid)
    out["connector_vertex_id"] = np.asarray(vid, dtype=np.int32)
    out["connector_triangle_id"] = np.asarray(tid, dtype=np.int32).reshape(c, 3)
    out["connector_tri_bar"] = np.full((c, 3), 1.0 / 3.0, dtype=np.float32)
    out["connector_rest_dist"] = np.asarray(dist, dtype=np.float32)
    return out
