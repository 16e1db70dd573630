"""Surface meshes for the BEM hot path: icospheres, jittered rounded cubes, and
GMSH 2.2 ASCII ``.msh`` files.

The reference reads meshes produced by GMSH (libs/libscuff/ParseMeshFiles.cc:69);
the same ``.msh`` file written here feeds both this library and the reference,
so coordinates are written with 17 significant digits (exact round trip).
"""
from __future__ import annotations

import numpy as np

__all__ = ["icosphere", "rounded_cube", "write_msh", "read_msh", "write_scuffgeo"]


def icosphere(subdivisions: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Icosahedron subdivided ``subdivisions`` times, vertices projected onto the
    sphere.  Returns (V[nv,3] float64, P[np,3] int32) with outward-oriented panels.
    Panel count 20*4**s, vertex count 10*4**s + 2, interior edges 30*4**s."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
         (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
         (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
         (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        nf = []
        for (a, b, c) in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    Va = np.array(V) * radius + np.asarray(center, dtype=np.float64)
    Pa = np.array(F, dtype=np.int32)
    # orient outward
    c = Va[Pa].mean(axis=1) - np.asarray(center)
    n = np.cross(Va[Pa[:, 1]] - Va[Pa[:, 0]], Va[Pa[:, 2]] - Va[Pa[:, 0]])
    flip = (n * c).sum(axis=1) < 0
    Pa[flip] = Pa[flip][:, [0, 2, 1]]
    return Va, Pa


def rounded_cube(target_panels: int, side: float = 1.0, rounding: float = 0.2,
                 jitter: float = 0.1, seed: int = 0):
    """Seeded jittered triangulation of a cube of side ``side`` with rounded edges.

    Each face is an n x n grid split into triangles (12 n^2 panels, n chosen so
    the count is near ``target_panels``); interior grid vertices are jittered by
    up to ``jitter`` times the grid spacing, then all vertices are projected onto
    the rounded-cube surface (the set of points at distance ``rounding*side/2``
    from a shrunken cube)."""
    n = max(1, int(round((target_panels / 12.0) ** 0.5)))
    rng = np.random.default_rng(seed)
    h = side / 2.0
    verts = {}
    V = []

    def vid(p):
        key = tuple(np.round(p, 9))
        if key not in verts:
            verts[key] = len(V)
            V.append(np.array(p, dtype=np.float64))
        return verts[key]

    P = []
    axes = [(0, 1, 2), (1, 2, 0), (2, 0, 1)]
    g = np.linspace(-h, h, n + 1)
    for (a, b, c) in axes:
        for sgn in (-1.0, 1.0):
            ids = np.empty((n + 1, n + 1), dtype=np.int64)
            for i in range(n + 1):
                for j in range(n + 1):
                    p = np.zeros(3)
                    p[a], p[b], p[c] = g[i], g[j], sgn * h
                    ids[i, j] = vid(p)
            for i in range(n):
                for j in range(n):
                    v00, v10, v01, v11 = ids[i, j], ids[i + 1, j], ids[i, j + 1], ids[i + 1, j + 1]
                    P.append((v00, v10, v11))
                    P.append((v00, v11, v01))
    V = np.array(V)
    # jitter vertices not on cube edges, tangentially
    dx = side / n
    onedge = (np.abs(np.abs(V) - h) < 1e-9).sum(axis=1) >= 2
    J = rng.uniform(-jitter * dx, jitter * dx, size=V.shape)
    for k in range(len(V)):
        if onedge[k]:
            continue
        face_axis = int(np.argmax(np.abs(V[k])))
        J[k, face_axis] = 0.0
        V[k] += J[k]
    # project onto rounded cube
    rr = rounding * h
    core = h - rr
    Q = np.clip(V, -core, core)
    d = V - Q
    nd = np.linalg.norm(d, axis=1, keepdims=True)
    V = Q + d / np.maximum(nd, 1e-300) * rr
    P = np.array(P, dtype=np.int32)
    c = V[P].mean(axis=1)
    nrm = np.cross(V[P[:, 1]] - V[P[:, 0]], V[P[:, 2]] - V[P[:, 0]])
    flip = (nrm * c).sum(axis=1) < 0
    P[flip] = P[flip][:, [0, 2, 1]]
    return V, P


def write_msh(path, V, P):
    """Write a GMSH 2.2 ASCII mesh (1-based node and element numbers)."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(V))
        for i, v in enumerate(V):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, v[0], v[1], v[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % len(P))
        for i, p in enumerate(P):
            f.write("%d 2 2 1 1 %d %d %d\n" % (i + 1, p[0] + 1, p[1] + 1, p[2] + 1))
        f.write("$EndElements\n")


def read_msh(path):
    """Read triangles of a GMSH 2.x mesh (legacy or 2.2 ASCII) into (V, P),
    merging vertices closer than 1e-6 as the reference does
    (ParseMeshFiles.cc:136-150)."""
    with open(path) as f:
        lines = f.read().splitlines()
    i = 0
    while not (lines[i].startswith("$Nodes") or lines[i].startswith("$NOD")):
        i += 1
    nn = int(lines[i + 1])
    ids, V = [], []
    for k in range(nn):
        t = lines[i + 2 + k].split()
        ids.append(int(t[0]))
        V.append([float(t[1]), float(t[2]), float(t[3])])
    V = np.array(V)
    g2h = {nid: k for k, nid in enumerate(ids)}
    # merge coincident vertices onto the first occurrence
    from collections import defaultdict
    grid = defaultdict(list)
    remap = np.arange(nn)
    for k in range(nn):
        key = tuple(np.floor(V[k] / 1e-5).astype(np.int64))
        hit = -1
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                        if np.linalg.norm(V[j] - V[k]) < 1e-6 and (hit < 0 or j < hit):
                            hit = j
        if hit >= 0:
            remap[k] = hit
        else:
            grid[key].append(k)
    j = i + 2 + nn
    while not (lines[j].startswith("$Elements") or lines[j].startswith("$ELM")):
        j += 1
    ne = int(lines[j + 1])
    P = []
    legacy = lines[j].startswith("$ELM")
    for k in range(ne):
        t = [int(x) for x in lines[j + 2 + k].split()]
        if t[1] != 2:
            continue
        vi = t[5:8] if legacy else t[3 + t[2]:3 + t[2] + 3]
        P.append([remap[g2h[v]] for v in vi])
    return V, np.array(P, dtype=np.int32)


def write_scuffgeo(path, objects, materials=None):
    """Write a .scuffgeo file.  ``objects``: list of (label, meshfile, material
    or None for PEC); ``materials``: dict name -> constant epsilon (complex)."""
    with open(path, "w") as f:
        for name, eps in (materials or {}).items():
            f.write("MATERIAL %s\n  Eps(w) = %r + %r*i;\nENDMATERIAL\n\n" % (name, eps.real, eps.imag))
        for label, mesh, mat in objects:
            f.write("OBJECT %s\n  MESHFILE %s\n" % (label, mesh))
            if mat is not None:
                f.write("  MATERIAL %s\n" % mat)
            f.write("ENDOBJECT\n\n")
