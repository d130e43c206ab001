"""The rounding bound behind the ray-cast's fast node test (render.cu, node_hit).

The traversal forms each slab distance as fma(lo, 1/rd, -(ro * (1/rd))) in float32 and
trusts its decision only when every part is farther from its threshold than the
difference to the reference's fl(fl(lo - ro) / rd) can be (intersectAABB,
render.py:588-609).  The kernel's comment states that difference as at most
4.01 u |t| + 1.02 u |ro/rd| with u = 2^-24.  This test checks that statement on seeded
float32 inputs spanning near and far boxes, small and large coordinates and nearly
axis-parallel rays.  The fma is emulated exactly: lo * (1/rd) of two float32 values is
exact in float64, and the difference to the float32 product rounds once more only when
the two are orders of magnitude apart, far below the bound's slack.
"""

import numpy as np

U = 2.0 ** -24


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    scale = 10.0 ** rng.uniform(-2, 3, size=(n, 1))
    ro = (rng.normal(size=(n, 3)) * scale).astype(np.float32)
    rd = rng.normal(size=(n, 3))
    # some nearly axis-parallel rays: tiny direction components
    tiny = rng.random(size=(n, 3)) < 0.1
    rd = np.where(tiny, rd * 1e-5, rd)
    rd = (rd / np.linalg.norm(rd, axis=1, keepdims=True)).astype(np.float32)
    reach = scale * 10.0 ** rng.uniform(-3, 1, size=(n, 1))
    lo = (ro + rng.normal(size=(n, 3)) * reach).astype(np.float32)
    return ro, rd, lo


def test_fma_slab_distance_stays_within_the_stated_bound():
    ro, rd, lo = _inputs(400_000, seed=7)
    with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
        inv = (np.float32(1.0) / rd).astype(np.float32)
        roinv = (ro * inv).astype(np.float32)
        t_fma = (lo.astype(np.float64) * inv.astype(np.float64) - roinv.astype(np.float64)).astype(np.float32)
        t_ref = ((lo - ro).astype(np.float32) / rd).astype(np.float32)
    ok = np.isfinite(t_fma) & np.isfinite(t_ref) & np.isfinite(roinv)
    assert ok.mean() > 0.99
    diff = np.abs(t_fma[ok].astype(np.float64) - t_ref[ok].astype(np.float64))
    bound = 4.01 * U * np.abs(t_fma[ok].astype(np.float64)) + 1.02 * U * np.abs(roinv[ok].astype(np.float64))
    ratio = diff / np.maximum(bound, np.finfo(np.float64).tiny)
    print(f"[slab] worst difference / bound = {ratio.max():.3f} over {ok.sum()} distances")
    assert (diff <= bound).all()


def test_guard_covers_every_decision():
    # node_hit compares tmax with 0 and with tmin, and tmin with the best hit; each part
    # differs from the reference's by at most two distance errors, which the guard
    # g = 8 u m + 4 u R (m: sum of the six |t|, R: sum of the three |ro/rd|) covers, and the
    # differences by 2 g
    ro, rd, lo = _inputs(50_000, seed=11)
    hi = (lo + np.abs(np.random.default_rng(3).normal(size=lo.shape)).astype(np.float32)
          * np.abs(lo - ro).max(axis=1, keepdims=True)).astype(np.float32)
    with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
        inv = (np.float32(1.0) / rd).astype(np.float32)
        roinv = (ro * inv).astype(np.float32)

        def fma_t(b):
            return (b.astype(np.float64) * inv.astype(np.float64) - roinv.astype(np.float64)).astype(np.float32)

        def ref_t(b):
            return ((b - ro).astype(np.float32) / rd).astype(np.float32)

        tf = np.concatenate([fma_t(lo), fma_t(hi)], axis=1)
        tr = np.concatenate([ref_t(lo), ref_t(hi)], axis=1)
    ok = np.isfinite(tf).all(axis=1) & np.isfinite(tr).all(axis=1) & np.isfinite(roinv).all(axis=1)
    tf, tr, R = tf[ok].astype(np.float64), tr[ok].astype(np.float64), np.abs(roinv[ok]).sum(axis=1)

    def span(t):
        t1, t2 = t[:, :3], t[:, 3:]
        return np.minimum(t1, t2).max(axis=1), np.maximum(t1, t2).min(axis=1)

    fmin, fmax = span(tf)
    rmin, rmax = span(tr)
    m = np.abs(tf).sum(axis=1)
    g = 8 * U * m + 4 * U * R
    assert (np.abs(fmax - rmax) <= g).all()
    assert (np.abs(fmin - rmin) <= g).all()
    assert (np.abs((fmax - fmin) - (rmax - rmin)) <= 2 * g).all()
