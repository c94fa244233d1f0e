"""Comparison helpers shared by the GPU parity tests (hit records and image statistics)."""
import numpy as np
from oracle.oracle import mt32


def compare_bitexact(gpu, t_ref, uv_ref, id_ref, rays=None, tri32=None):
    """GPU hits against the fp32 restatement: every ray agrees bit for bit in (triangle index, t,
    u, v) except exact-t ties (two triangles at identical fp32 t: the kernel keeps the smaller
    index, accel_sahbvh.cpp:285-291 the later one). With `rays` and the oracle's fp32 triangle
    records `tri32`, a tie is confirmed by recomputing both triangles' fp32 t (needed when the
    reported t is the fp64-refined distance); without them, by equal reported t. Returns the
    number of ties."""
    g_id = gpu["prim"].astype(np.int64)
    same = g_id == id_ref
    hit = same & (g_id >= 0)
    cand = (~same) & (g_id >= 0) & (id_ref >= 0)
    ties = np.zeros_like(cand)
    if rays is not None and tri32 is not None:
        k = np.nonzero(cand)[0]
        if len(k):
            r = rays[k]
            ties[k] = mt32(r, tri32, g_id[k]) == mt32(r, tri32, id_ref[k])
    else:
        ties = cand & (gpu["t"] == t_ref.astype(np.float32))
    bad = ~(same | ties)
    assert bad.sum() == 0, f"{bad.sum()} of {len(g_id)} rays differ, e.g. {np.nonzero(bad)[0][:5]}"
    assert np.array_equal(gpu["t"][hit], t_ref[hit].astype(np.float32))
    assert np.array_equal(gpu["u"][hit], uv_ref[hit, 0].astype(np.float32))
    assert np.array_equal(gpu["v"][hit], uv_ref[hit, 1].astype(np.float32))
    return int(ties.sum())


def mt64(o, d, p1, e1, e2):
    """fp64 Moller-Trumbore without range checks: (t, u, v, |det|) per row."""
    p = np.cross(d, e2)
    tv = o - p1
    q = np.cross(tv, e1)
    det = np.sum(e1 * p, 1)
    ad = np.abs(det)
    s = np.sign(det)
    u = np.sum(tv * p, 1) * s / np.where(ad > 0, ad, 1)
    v = np.sum(d * q, 1) * s / np.where(ad > 0, ad, 1)
    t = np.sum(e2 * q, 1) / np.where(det != 0, det, 1)
    return t, u, v, ad


EPS32 = 2.0 ** -24


def fp32_bounds(o, d, tri_rows, k=16.0):
    """fp64 (t, u, v) of rays (o, d) against triangle rows (m, 3, 3) and the fp32 Moller-Trumbore
    test's error bounds for them (see classify_fp64_mismatches): (t, u, v, err_t, err_u, err_v)."""
    nd = np.linalg.norm(d, axis=1)
    p1 = tri_rows[:, 0]
    e1, e2 = tri_rows[:, 1] - p1, tri_rows[:, 2] - p1
    t, u, v, ad = mt64(o, d, p1, e1, e2)
    ad = np.maximum(ad, 1e-300)
    ntv, n1, n2 = np.linalg.norm(o - p1, axis=1), np.linalg.norm(e1, axis=1), np.linalg.norm(e2, axis=1)
    err_u = k * EPS32 * ntv * nd * n2 / ad
    err_v = k * EPS32 * nd * ntv * n1 / ad
    err_t = k * EPS32 * (n2 * ntv * n1 / ad + np.abs(t))
    return t, u, v, err_t, err_u, err_v


def classify_fp64_mismatches(rays, g, ids64, tri, k=16.0):
    """Rays whose GPU (fp32) triangle differs from the fp64 restatement's. Each must be one the
    fp32 test cannot decide within its rounding error: a near-tie (the two triangles' fp64 t
    closer than the fp32 error bound of t) or a grazing hit (a candidate's fp64 barycentric margin
    min(u, v, 1 - u - v), negative outside, within the fp32 error bound of the barycentrics).

    The bounds are k * 2^-24 times the magnitudes the fp32 formulas cancel (accel_sahbvh.cpp:58-75):
    u = (tv . (d x e2)) / det, v = (d . (tv x e1)) / det, t = (e2 . q) / det, with tv = o - p1 and
    det = e1 . (d x e2): err_u = k eps |tv| |d| |e2| / |det|, err_v = k eps |d| |tv| |e1| / |det|,
    err_t = k eps |e2| |tv| |e1| / |det|. k = 16 covers the chain's at most six roundings with margin.
    Far hits on small triangles make these bounds large: |tv| ~ t, while |det| ~ |e1| |e2| cos.
    Returns (near_ties, grazing, unexplained ray indices)."""
    mism = np.nonzero(g != ids64)[0]
    if len(mism) == 0:
        return 0, 0, []
    o = rays[mism, 0:3].astype(np.float64)
    d = rays[mism, 4:7].astype(np.float64)

    def test(c):
        valid = c >= 0
        t, u, v, err_t, err_u, err_v = fp32_bounds(o, d, tri[np.where(valid, c, 0)], k)
        margins = np.stack([u, v, 1 - u - v], 1)
        errs = np.stack([err_u, err_v, err_u + err_v], 1)
        graze = np.any(np.abs(margins) <= errs, axis=1)
        return valid, t, graze, err_t

    va, ta, ga, eta = test(g[mism])
    vb, tb, gb, etb = test(ids64[mism])
    near_tie = va & vb & (np.abs(ta - tb) <= np.maximum(eta, etb))
    grazing = (va & ga) | (vb & gb)
    ok = near_tie | grazing
    return int(near_tie.sum()), int((grazing & ~near_tie).sum()), [int(i) for i in mism[~ok]]


def check_against_fp64(gpu, t64, uv64, ids64, rays, tri, label):
    """GPU (fp32) hits against fp64 hits of the same rays (the reference's own, or the fp64
    restatement's). Where both pick the same triangle, t agrees within 1e-5 relative and u, v
    within 1e-5 absolute, or within the fp32 test's error bounds where those are larger (far,
    grazing hits). Every differing triangle choice is a near-tie or a grazing hit (see
    classify_fp64_mismatches). `tri` is the world-space triangles (n, 3, 3) in flattened order.
    Returns (fp64 hits, index mismatches, near-ties, grazing)."""
    g = gpu["prim"].astype(np.int64)
    ids64 = np.asarray(ids64, np.int64)
    both = np.nonzero((g >= 0) & (g == ids64))[0]
    if both.size:
        o = rays[both, 0:3].astype(np.float64)
        d = rays[both, 4:7].astype(np.float64)
        _, _, _, err_t, err_u, err_v = fp32_bounds(o, d, tri[g[both]])
        dt = np.abs(gpu["t"][both].astype(np.float64) - t64[both])
        du = np.abs(gpu["u"][both].astype(np.float64) - uv64[both, 0])
        dv = np.abs(gpu["v"][both].astype(np.float64) - uv64[both, 1])
        bad_t = dt > np.maximum(1e-5 * np.abs(t64[both]), err_t)
        bad_uv = (du > np.maximum(1e-5, err_u)) | (dv > np.maximum(1e-5, err_v))
        assert not bad_t.any(), f"{label}: t outside its bound at rays {both[bad_t][:10]}"
        assert not bad_uv.any(), f"{label}: u, v outside their bounds at rays {both[bad_uv][:10]}"
    near, graze, unexplained = classify_fp64_mismatches(rays, g, ids64, tri)
    assert not unexplained, f"{label}: unexplained index mismatches at rays {unexplained[:10]}"
    return int((ids64 >= 0).sum()), int((g != ids64).sum()), near, graze


def nmse(img, ref):
    """Normalized MSE: sum((img - ref)^2) / sum(ref^2) over every pixel and channel."""
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sum((img - ref) ** 2) / np.sum(ref ** 2))


def downsample(img, k):
    """Box filter over k x k pixel blocks. With pixel-window jitter this is exactly the image of
    the same camera at 1/k of the resolution with k*k times the samples per pixel."""
    h, w, c = img.shape
    return img.reshape(h // k, k, w // k, k, c).mean(axis=(1, 3))
