"""Synthetic meshes of the benchmark workloads (seeded, numpy only).

  grid2d(33)            33x33 vertex grid on the unit square, each cell split along
                        its (i,j)-(i+1,j+1) diagonal: 1089 vertices, 2048 triangles
  kuhn_cube(65, ...)    65^3 lattice on the unit cube, every cube Kuhn-split into 6
                        tets along its (0,0,0)-(1,1,1) diagonal (274,625 vertices,
                        1,572,864 tets); interior vertices jittered by U(-0.2h, 0.2h)^3
  log_uniform_speeds    per-element speed exp(U(ln lo, ln hi))
  icosphere(level)      unit icosahedron subdivided `level` times (10*4^L + 2 vertices)
  batch_workload(256)   the batching workload: icospheres of levels U{2..6}, 1-8
                        seeds each, per-triangle speed 1 + 0.5 sin(3x) cos(2y) sin(z)
  sliver_cube / anisotropic_metrics   the precision workload (49^3 cube with
                        10% sliver tets and per-tet SPD metrics R diag(1,a,b) R^T)

Vertex numbering is lexicographic (index = i + n*j [+ n*n*k]) so the reference's
structured-grid tiling applies to the grids.
"""
import concurrent.futures as _fut
import os

import numpy as np


def grid2d(n=33):
    h = 1.0 / (n - 1)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    xyz = np.stack([i.ravel() * h, j.ravel() * h, np.zeros(n * n)], axis=1).astype(np.float32)
    ci, cj = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="xy")
    v00 = (cj * n + ci).ravel()
    v10 = v00 + 1
    v01 = v00 + n
    v11 = v00 + n + 1
    faces = np.concatenate([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 0).astype(np.int32)
    return xyz, faces


_KUHN = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def kuhn_cube(n=65, jitter=0.2, seed=1):
    """Vertices (n^3 x 3 float32) and tets (6 (n-1)^3 x 4 int32) of a jittered unit cube."""
    h = 1.0 / (n - 1)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    xyz = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64) * h
    if jitter > 0:
        rng = np.random.Generator(np.random.PCG64(seed))
        d = rng.uniform(-jitter * h, jitter * h, size=xyz.shape)
        ii, jj, kk = i.ravel(), j.ravel(), k.ravel()
        interior = (ii > 0) & (ii < n - 1) & (jj > 0) & (jj < n - 1) & (kk > 0) & (kk < n - 1)
        xyz[interior] += d[interior]
    xyz = xyz.astype(np.float32)
    m = n - 1
    ck, cj, ci = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    base = (ci + n * cj + n * n * ck).ravel()
    step = [1, n, n * n]
    tets = []
    for p in _KUHN:
        a = base
        b = a + step[p[0]]
        c = b + step[p[1]]
        d = c + step[p[2]]
        tets.append(np.stack([a, b, c, d], 1))
    tets = np.stack(tets, 1).reshape(-1, 4).astype(np.int32)
    return xyz, tets


def center_vertex(n):
    c = n // 2
    return c + n * c + n * n * c


def log_uniform_speeds(count, lo=0.5, hi=2.0, seed=2):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.float32)


_ICO_CACHE = {}


def icosphere(level):
    """Unit icosphere: (10*4^level + 2) x 3 float32 vertices, 20*4^level x 3 int32 faces."""
    if level not in _ICO_CACHE:
        _ICO_CACHE[level] = _icosphere(level)
    v, f = _ICO_CACHE[level]
    return v.copy(), f.copy()


def _icosphere(level):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = np.array(f, dtype=np.int64)
    for _ in range(level):
        cache = {}
        vl = list(verts)

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = vl[a] + vl[b]
                vl.append(m / np.linalg.norm(m))
                cache[key] = len(vl) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        verts = vl
        faces = np.array(nf, dtype=np.int64)
    return np.array(verts, dtype=np.float32), faces.astype(np.int32)


def batch_speed(xyz, faces):
    """Per-triangle speed 1 + 0.5 sin(3x) cos(2y) sin(z) at the centroid."""
    c = xyz[faces].mean(axis=1).astype(np.float64)
    return (1.0 + 0.5 * np.sin(3 * c[:, 0]) * np.cos(2 * c[:, 1]) * np.sin(c[:, 2])).astype(np.float32)


def batch_workload(count=256, level_seed=3, seed_seed=4, lo=2, hi=6):
    """Independent 2D solves of uneven size: per instance (xyz, faces, speeds, seeds)
    with the icosphere level drawn uniformly from {lo..hi} (PCG64 seed level_seed),
    1-8 distinct seed vertices (PCG64 seed seed_seed) and batch_speed speeds."""
    rl = np.random.Generator(np.random.PCG64(level_seed))
    rs = np.random.Generator(np.random.PCG64(seed_seed))
    levels = rl.integers(lo, hi + 1, size=count)
    out = []
    for lv in levels:
        xyz, faces = icosphere(int(lv))
        k = int(rs.integers(1, 9))
        seeds = np.sort(rs.choice(xyz.shape[0], size=k, replace=False)).astype(np.int32)
        out.append((xyz, faces, batch_speed(xyz, faces), seeds))
    return out


def random_rotations(count, rng):
    q = rng.normal(size=(count, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)


def anisotropic_metrics(count, seed=6, lo=1.0, hi=100.0):
    """6 entries M00 M01 M02 M11 M12 M22 per tet of M = R diag(1, a, b) R^T."""
    rng = np.random.Generator(np.random.PCG64(seed))
    R = random_rotations(count, rng)
    ab = np.exp(rng.uniform(np.log(lo), np.log(hi), size=(count, 2)))
    D = np.zeros((count, 3, 3))
    D[:, 0, 0] = 1.0
    D[:, 1, 1] = ab[:, 0]
    D[:, 2, 2] = ab[:, 1]
    M = R @ D @ np.transpose(R, (0, 2, 1))
    return np.stack([M[:, 0, 0], M[:, 0, 1], M[:, 0, 2], M[:, 1, 1], M[:, 1, 2], M[:, 2, 2]], 1).astype(np.float32)


def _min_dihedral(P):
    """Minimum dihedral angle (radians) of tets P (t x 4 x 3)."""
    faces = [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]
    normals = []
    for a, b, c in faces:
        nrm = np.cross(P[:, b] - P[:, a], P[:, c] - P[:, a])
        normals.append(nrm / np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-300))
    best = np.full(P.shape[0], np.pi)
    for x in range(4):
        for y in range(x + 1, 4):
            cosang = -np.sum(normals[x] * normals[y], axis=1)
            best = np.minimum(best, np.arccos(np.clip(cosang, -1, 1)))
    return best


def _tet_volumes(P):
    return np.einsum("...j,...j->...", np.cross(P[..., 1, :] - P[..., 0, :], P[..., 2, :] - P[..., 0, :]),
                     P[..., 3, :] - P[..., 0, :])


def _has_small_dihedral(P, lim):
    """True where a tet (... x 4 x 3) has a dihedral angle below `lim` radians."""
    faces = [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]
    nr = []
    for a, b, c in faces:
        x = np.cross(P[..., b, :] - P[..., a, :], P[..., c, :] - P[..., a, :])
        nr.append(x / np.maximum(np.linalg.norm(x, axis=-1, keepdims=True), 1e-300))
    c = np.cos(lim)
    out = np.zeros(P.shape[:-2], dtype=bool)
    for x in range(4):
        for y in range(x + 1, 4):
            out |= -np.sum(nr[x] * nr[y], axis=-1) > c
    return out


def sliver_cube(n=49, fraction=0.10, seed=5, max_deg=5.0, directions=12,
                steps=(0.9, 0.95, 0.98, 0.995), rounds=3):
    """Jittered Kuhn cube (as kuhn_cube(n, 0.2, seed=1)) with about `fraction` of
    its tets flattened into slivers: minimum dihedral angle below `max_deg`
    degrees, every tet keeping its orientation and at least 1e-3 of its volume.

    A conforming mesh has no vertex unique to one tet, so slivers come from moving
    interior vertices toward the opposite face of a tet of their ring.  Vertices
    are taken by lattice parity class (same-parity vertices share no tet, so a
    class moves at once); for each vertex, `directions` random ring tets times
    `steps` (fractions of the distance to that tet's opposite face) are tried and
    the valid move that most raises the ring's sliver count is kept.  Rounds over
    the classes (each round in a random order, PCG64 seed `seed`) run until the
    slivers reach the target.
    Returns xyz (float32), tets, sliver mask (final dihedral test of every tet)."""
    xyz, tets = kuhn_cube(n, 0.2, seed=1)
    xyz = xyz.astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(seed))
    nt = tets.shape[0]
    target = int(fraction * nt)
    lim = np.deg2rad(max_deg)
    vol0 = _tet_volumes(xyz[tets])
    order = np.argsort(tets.ravel(), kind="stable")
    tet_of = order // 4
    starts = np.searchsorted(tets.ravel()[order], np.arange(xyz.shape[0] + 1))
    ii = np.arange(xyz.shape[0])
    gi, gj, gk = ii % n, (ii // n) % n, ii // (n * n)
    interior = (gi > 0) & (gi < n - 1) & (gj > 0) & (gj < n - 1) & (gk > 0) & (gk < n - 1)
    if not interior.any():
        return xyz.astype(np.float32), tets, np.zeros(nt, dtype=bool)
    R = int((starts[1:] - starts[:-1])[interior].max())
    made = int(_has_small_dihedral(xyz[tets], lim).sum())
    classes = [c for _ in range(rounds) for c in rng.permutation(8)]
    for cls in classes:
        if made >= target:
            break
        sel = np.nonzero(interior & (gi % 2 == (cls & 1)) & (gj % 2 == ((cls >> 1) & 1)) & (gk % 2 == (cls >> 2)))[0]
        sel = rng.permutation(sel)
        rings = np.stack([tet_of[starts[v]:starts[v] + R] for v in sel])  # S x R
        T = tets[rings]
        pos = T == sel[:, None, None]
        P0 = xyz[T]
        v0 = vol0[rings]
        def trial(r):
            # the best valid step toward the opposite face of ring tet r, per vertex
            F = xyz[T[:, r][~pos[:, r]].reshape(len(sel), 3)]
            nrm = np.cross(F[:, 1] - F[:, 0], F[:, 2] - F[:, 0])
            nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
            dist = np.einsum("ij,ij->i", xyz[sel] - F[:, 0], nrm)
            bc = np.zeros(len(sel), dtype=np.int64)
            bp = xyz[sel].copy()
            for f in steps:
                newp = xyz[sel] - (f * dist)[:, None] * nrm
                P = P0.copy()
                P[pos] = np.repeat(newp, R, axis=0)
                vn = _tet_volumes(P)
                ok = np.all((vn * v0 > 0) & (np.abs(vn) >= 1e-3 * np.abs(v0)), axis=1)
                cnt = np.where(ok, _has_small_dihedral(P, lim).sum(axis=1), 0)
                upd = cnt > bc
                bc[upd] = cnt[upd]
                bp[upd] = newp[upd]
            return bc, bp

        dirs = rng.choice(R, size=min(directions, R), replace=False)
        with _fut.ThreadPoolExecutor(max_workers=min(len(dirs), os.cpu_count() or 1)) as ex:
            trials = list(ex.map(trial, dirs))
        cur = _has_small_dihedral(P0, lim).sum(axis=1)  # ring slivers where the vertex is now
        best = cur.astype(np.int64)
        best_pos = xyz[sel].copy()
        for bc, bp in trials:  # in direction order: ties keep the earlier direction
            upd = bc > best
            best[upd] = bc[upd]
            best_pos[upd] = bp[upd]
        gain = best - cur
        take = (gain > 0) & (np.cumsum(gain) <= max(0, target - made))
        xyz[sel[take]] = best_pos[take]
        made = int(_has_small_dihedral(xyz[tets], lim).sum())
    xyz32 = xyz.astype(np.float32)
    return xyz32, tets, _has_small_dihedral(xyz32[tets].astype(np.float64), lim)
