"""Test helper: a Python replica of the 8-wide traversal in csrc/lmgpu_dev.cuh (trace_bvh8).

It walks the node and triangle arrays that lmgpu_bvh8_build_host produces with the same slot
decoding, octant order and sibling-group stack as the kernel, and the same fp32 Moller-Trumbore
arithmetic (numpy float32 scalars round every operation to fp32, no fused multiply-add). The
CPU tests use it to check the data layout and the traversal logic against the oracle's
exhaustive test before any GPU run.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

f32 = np.float32


def build_host(native, tri_p: np.ndarray):
    tri_p = np.ascontiguousarray(tri_p, np.float32).reshape(-1, 9)
    n = tri_p.shape[0]
    nodes = np.zeros(20 * max(n, 1), np.uint32)
    tris = np.zeros(12 * n, np.float32)
    nn = C.c_int64()
    depth = C.c_int32()
    from lightmetrica import _native as N
    N.check(native.lmgpu_bvh8_build_host(N.fptr(tri_p), n, nodes.ctypes.data_as(C.POINTER(C.c_uint32)), N.fptr(tris),
                                         C.byref(nn), C.byref(depth)))
    return nodes[:20 * nn.value].reshape(-1, 20), tris.reshape(-1, 12), depth.value


def build_gpu(native, tri_p: np.ndarray):
    """The same arrays from the GPU builder (lmgpu_bvh8_build_gpu; needs a device)."""
    tri_p = np.ascontiguousarray(tri_p, np.float32).reshape(-1, 9)
    n = tri_p.shape[0]
    nodes = np.zeros(20 * max(n, 1), np.uint32)
    tris = np.zeros(12 * n, np.float32)
    nn = C.c_int64()
    depth = C.c_int32()
    from lightmetrica import _native as N
    N.check(native.lmgpu_bvh8_build_gpu(N.fptr(tri_p), n, nodes.ctypes.data_as(C.POINTER(C.c_uint32)), N.fptr(tris),
                                        C.byref(nn), C.byref(depth)))
    return nodes[:20 * nn.value].reshape(-1, 20), tris.reshape(-1, 12), depth.value


def decode(w: np.ndarray) -> dict:
    u = w.astype(np.uint64)
    org = w[0:3].view(np.float32)
    eb = [(int(w[3]) >> (8 * a)) & 0xFF for a in range(3)]
    scale = [np.uint32(e << 23).view(np.float32) for e in eb]
    imask = int(w[3]) >> 24
    meta = [(int(w[6 + s // 4]) >> (8 * (s % 4))) & 0xFF for s in range(8)]
    qlo = [[(int(w[8 + 2 * a + s // 4]) >> (8 * (s % 4))) & 0xFF for s in range(8)] for a in range(3)]
    qhi = [[(int(w[14 + 2 * a + s // 4]) >> (8 * (s % 4))) & 0xFF for s in range(8)] for a in range(3)]
    del u
    return {"origin": org, "scale": scale, "imask": imask, "child_base": int(w[4]), "tri_base": int(w[5]),
            "meta": meta, "qlo": qlo, "qhi": qhi}


def child_box(nd: dict, s: int):
    """Dequantized planes rounded to fp32: fmaf(q, scale, origin). q * scale is exact in fp32
    (q < 256, scale a power of two), so one fp32 addition gives the fused result."""
    lo = [f32(nd["origin"][a] + f32(f32(nd["qlo"][a][s]) * nd["scale"][a])) for a in range(3)]
    hi = [f32(nd["origin"][a] + f32(f32(nd["qhi"][a][s]) * nd["scale"][a])) for a in range(3)]
    return lo, hi


def _cross(x, y):
    return (f32(x[1] * y[2]) - f32(y[1] * x[2]), f32(x[2] * y[0]) - f32(y[2] * x[0]), f32(x[0] * y[1]) - f32(y[0] * x[1]))


def _dot(a, b):
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def tri_test(o, d, p1, e1, e2, tl, th):
    """accel_sahbvh.cpp:58-75 in fp32."""
    p = tuple(f32(v) for v in _cross(d, e2))
    tv = (f32(o[0] - p1[0]), f32(o[1] - p1[1]), f32(o[2] - p1[2]))
    q = tuple(f32(v) for v in _cross(tv, e1))
    det = _dot(e1, p)
    ad = f32(abs(det))
    s = f32(math.copysign(1.0, det))
    u = f32(_dot(tv, p) * s)
    v = f32(_dot(d, q) * s)
    if ad < f32(1e-8) or u < 0 or v < 0 or f32(u + v) > ad:
        return None
    t = f32(_dot(e2, q) / det)
    if t < tl or th < t:
        return None
    return t, f32(u / ad), f32(v / ad)


def _oct_permute(m: int, oct_: int) -> int:
    if oct_ & 1:
        m = ((m & 0x55) << 1) | ((m >> 1) & 0x55)
    if oct_ & 2:
        m = ((m & 0x33) << 2) | ((m >> 2) & 0x33)
    if oct_ & 4:
        m = ((m & 0x0F) << 4) | ((m >> 4) & 0x0F)
    return m


def trace(nodes: np.ndarray, tris: np.ndarray, depth: int, ray: np.ndarray, any_hit: bool = False):
    """Returns (t, u, v, id, visited) with id = -1 on a miss; same rules as trace_bvh8."""
    o = tuple(f32(x) for x in ray[0:3])
    tmin = f32(ray[3])
    d = tuple(f32(x) for x in ray[4:7])
    # the kernel's slab reciprocals: zero or tiny components become +-1e-20 (sign kept)
    ds = tuple(x if abs(x) > 1e-20 else math.copysign(1e-20, x) for x in d)
    oct_ = sum((1 << a) for a in range(3) if math.copysign(1.0, d[a]) < 0)
    best_t, best_u, best_v, best_id = f32(ray[7]), f32(0), f32(0), -1
    stack = []
    node = 0
    visited = 0
    decoded = {}
    while True:
        visited += 1
        assert visited <= len(nodes)
        nd = decoded.get(node)
        if nd is None:
            nd = decoded[node] = decode(nodes[node])
        hitmask = 0
        for s in range(8):
            if nd["meta"][s] == 0:
                continue
            # exact plane positions p + q*s (in double) with the kernel's 2^-18 far-side widening
            tn, tf = [], []
            for a in range(3):
                lo = float(nd["origin"][a]) + nd["qlo"][a][s] * float(nd["scale"][a])
                hi = float(nd["origin"][a]) + nd["qhi"][a][s] * float(nd["scale"][a])
                near, far = (hi, lo) if (oct_ >> a) & 1 else (lo, hi)
                tn.append((near - float(o[a])) / float(ds[a]))
                tf.append((far - float(o[a])) / float(ds[a]))
            tnv = max(max(tn), float(tmin))
            tfv = min(tf + [float(best_t)]) * (1 + 2.0 ** -18)
            if tnv <= tfv:
                hitmask |= 1 << s
        leaves = hitmask & ~nd["imask"]
        for s in range(8):
            if not (leaves >> s) & 1:
                continue
            meta = nd["meta"][s]
            cnt, off = meta >> 5, meta & 31
            for j in range(cnt):
                rec = tris[nd["tri_base"] + off + j]
                p1, e1, e2 = rec[0:3], rec[3:6], rec[6:9]
                r = tri_test(o, d, p1, e1, e2, tmin, best_t)
                if r is None:
                    continue
                tid = int(rec[9:10].view(np.uint32)[0])
                if any_hit:
                    return r[0], r[1], r[2], tid, visited
                if r[0] < best_t or best_id < 0 or tid < best_id:
                    best_t, best_u, best_v, best_id = r[0], r[1], r[2], tid
        inner = _oct_permute(hitmask & nd["imask"], oct_)
        base, imask = nd["child_base"], nd["imask"]
        if inner == 0:
            if not stack:
                break
            base, imask, inner = stack.pop()
        k = (inner & -inner).bit_length() - 1
        inner &= inner - 1
        slot = k ^ oct_
        node = base + bin(imask & ((1 << slot) - 1)).count("1")
        if inner:
            assert len(stack) < depth
            stack.append((base, imask, inner))
    return (best_t if best_id >= 0 else f32(0)), best_u, best_v, best_id, visited
