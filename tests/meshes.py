"""Closed triangle meshes for the STL point-in-mesh tests."""
import numpy as np


def cube(lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0)):
    """12 triangles, outward winding."""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    c = np.array([[lo[0] if (i >> 0) & 1 == 0 else hi[0], lo[1] if (i >> 1) & 1 == 0 else hi[1],
                   lo[2] if (i >> 2) & 1 == 0 else hi[2]] for i in range(8)])
    quads = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    tris = []
    for a, b, cc, d in quads:
        tris.append([c[a], c[b], c[cc]])
        tris.append([c[a], c[cc], c[d]])
    return np.array(tris).reshape(-1, 9)


def icosphere(radius=1.0, center=(0.0, 0.0, 0.0), levels=1):
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(x, float) / np.linalg.norm(x) for x in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(levels):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    V = np.array(v) * radius + np.asarray(center, float)
    return np.array([[V[a], V[b], V[c]] for a, b, c in f]).reshape(-1, 9)


def l_shape():
    """Non-convex: two boxes sharing a face, meshed as their union's boundary
    (here simply two closed boxes; a point inside either is inside)."""
    return np.concatenate([cube((0, 0, 0), (2, 1, 1)), cube((0, 1.0001, 0), (1, 2, 1))])
