"""Shared rules of the hit-parity tests (GPU and the CPU run of the kernels).

the benchmark spec's bar: hit / miss and primitive id equal to the reference BVH's
except rays within 1e-6 of a primitive edge, t within 1e-5 relative (here:
t bit-identical wherever the primitive agrees).  "Within 1e-6" is measured
as a distance in scene units relative to the scale of the hit's float32
coordinates: the hit point lies closer to an edge than 1e-6 x (t + |P|max),
about 8 float32 ulps of the larger of the ray length and the hit point's
coordinates.  Below that, which of two adjoining triangles a ray enters is
decided by the rounding of two different FP32 formulas (the reference's
Moller-Trumbore against the watertight test), which no FP32 implementation
can reproduce bit for bit.  Every exclusion is counted and bounded per
scene.  Coplanar primitives are not excluded: where two of them meet a ray at
the same distance the reference keeps the one its BVH traversal reaches last,
and the kernels reproduce that order (tie_order.h), so the primitive ids must
agree there as everywhere else.
"""
import numpy as np

from cadise_gb300 import abi

EDGE = 1e-6
MAX_EXCLUDED = 0.005  # at most 0.5 % of the rays of a scene


def edge_distance(flat, prim, P):
    """Distance in scene units from points P (n, 3), projected into their
    primitives' planes, to the nearest edge of the primitive (inf for a
    sphere or a miss)."""
    m = np.full(len(prim), np.inf)
    for i, (p, x) in enumerate(zip(prim, P)):
        if p < 0:
            continue
        v = flat.vertices[p].reshape(3, 3).astype(np.float64)
        if flat.kind[p] == abi.CGPU_PRIM_SPHERE:
            continue  # no edges: the sphere test is the reference's own formula
        if flat.kind[p] == abi.CGPU_PRIM_TRIANGLE:
            e0, e1, w = v[1] - v[0], v[2] - v[0], x - v[0]
            d00, d01, d11 = e0 @ e0, e0 @ e1, e1 @ e1
            d20, d21 = w @ e0, w @ e1
            den = d00 * d11 - d01 * d01
            if den == 0:
                m[i] = 0
                continue
            b1 = (d11 * d20 - d01 * d21) / den
            b2 = (d00 * d21 - d01 * d20) / den
            b0 = 1 - b1 - b2
            area2 = np.sqrt(den)  # twice the triangle's area
            # a barycentric coordinate times the altitude onto its opposite edge
            alt = [area2 / np.linalg.norm(v[2] - v[1]), area2 / np.linalg.norm(e1), area2 / np.linalg.norm(e0)]
            m[i] = min(abs(b0) * alt[0], abs(b1) * alt[1], abs(b2) * alt[2])
        else:
            eA, eB = v[0] - v[1], v[2] - v[1]
            w = x - v[1]
            la, lb = np.linalg.norm(eA), np.linalg.norm(eB)
            a = w @ eA / (la * la)
            b = w @ eB / (lb * lb)
            m[i] = min(abs(a) * la, abs(1 - a) * la, abs(b) * lb, abs(1 - b) * lb)
    return m


def near_edge(flat, prim, rays, t):
    """Rays whose hit on `prim` at distance t lies within 1e-6 of an edge
    (relative to the hit's coordinate scale, see the module docstring)."""
    o, d = rays[:, :3].astype(np.float64), rays[:, 4:7].astype(np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    P = o + d * np.asarray(t, np.float64)[:, None]
    scale = np.abs(np.asarray(t, np.float64)) + np.abs(P).max(axis=1)
    return edge_distance(flat, prim, P) < EDGE * scale


def hit_exclusions(flat, rays, prim, t, ref_p, ref_t):
    """Rays excluded from the primitive-id comparison: those whose ids differ
    and whose hit on either primitive lies within 1e-6 of an edge."""
    near = np.zeros(len(prim), bool)
    diff = np.where(prim != ref_p)[0]
    if len(diff):
        near[diff] = near_edge(flat, ref_p[diff], rays[diff], ref_t[diff]) | \
                     near_edge(flat, prim[diff], rays[diff], t[diff])
    return near


def check_hits(flat, rays, prim, t, ref_p, ref_t, label=""):
    """Asserts the benchmark spec's hit parity; returns the excluded fraction."""
    near = hit_exclusions(flat, rays, prim, t, ref_p, ref_t)
    keep = ~near
    frac = 1.0 - keep.mean()
    assert frac <= MAX_EXCLUDED, (label, frac, near.sum())
    bad = np.where(prim[keep] != ref_p[keep])[0]
    assert len(bad) == 0, (label, np.where(keep)[0][bad][:10])
    both = (prim == ref_p) & (prim >= 0)
    assert np.array_equal(t[both], ref_t[both]), (label, np.abs(t - ref_t)[both].max())
    return frac
