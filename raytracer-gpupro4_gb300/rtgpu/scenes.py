"""Seeded synthetic scenes for the LBVH workloads.

The reference loads OBJ models (Common/Scenes/Model.cpp:210-381) that are
not available here; these generators stand in for them with the sizes of the
five workloads.  Every generator returns a de-indexed fp32 triangle soup of
shape (n, 9) (A, B, C), the layout the C ABI consumes.  Vertices shared by
neighbouring triangles are bit-identical, so meshes are watertight.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from ._lib import Camera


# ---------------------------------------------------------------------------
def look_at(eye, target, up_hint=(0.0, 1.0, 0.0), vfov_deg=60.0, width=512, height=512) -> Camera:
    """Pinhole camera with an orthonormal basis (computed in float64, stored fp32)."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up_hint, np.float64))
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    cam = Camera()
    for name, v in (("eye", eye), ("right", right), ("up", up), ("fwd", fwd)):
        arr = getattr(cam, name)
        for c in range(3):
            arr[c] = float(np.float32(v[c]))
    cam.tan_half_fovy = float(np.float32(math.tan(math.radians(vfov_deg) / 2)))
    cam.width = width
    cam.height = height
    return cam


def deindex(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(verts.astype(np.float32)[faces].reshape(len(faces), 9))


# ---------------------------------------------------------------------------
def torus(n_major: int = 256, n_minor: int = 128, R: float = 1.0, r: float = 0.3, jitter: float = 0.002,
          seed: int = 1) -> np.ndarray:
    """Tessellated torus ring in the xy plane: 2 * n_major * n_minor triangles
    (65,536 by default), vertex jitter N(0, jitter) from PCG64(seed)."""
    u = np.arange(n_major) * (2 * np.pi / n_major)
    v = np.arange(n_minor) * (2 * np.pi / n_minor)
    U, V = np.meshgrid(u, v, indexing="ij")
    P = np.stack([(R + r * np.cos(V)) * np.cos(U), (R + r * np.cos(V)) * np.sin(U), r * np.sin(V)], axis=-1)
    P = P.reshape(-1, 3)
    rng = np.random.Generator(np.random.PCG64(seed))
    P = P + rng.normal(0.0, jitter, size=P.shape)
    i = np.arange(n_major)[:, None]
    j = np.arange(n_minor)[None, :]
    a = i * n_minor + j
    b = ((i + 1) % n_major) * n_minor + j
    c = ((i + 1) % n_major) * n_minor + (j + 1) % n_minor
    d = i * n_minor + (j + 1) % n_minor
    faces = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return deindex(P, faces)


# ---------------------------------------------------------------------------
_ICO_V = None


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return V, F


def geodesic_sphere(freq: int):
    """Class-I geodesic subdivision of the icosahedron: 20 * freq^2 faces,
    10 * freq^2 + 2 shared vertices on the unit sphere."""
    V0, F0 = _icosahedron()
    f = freq
    edges = {}
    for tri in F0:
        for a, b in ((tri[0], tri[1]), (tri[1], tri[2]), (tri[0], tri[2])):
            key = (min(a, b), max(a, b))
            if key not in edges:
                edges[key] = len(edges)
    n_edge_pts = f - 1
    n_face_pts = (f - 1) * (f - 2) // 2
    base_e = 12
    base_f = base_e + len(edges) * n_edge_pts
    nverts = base_f + 20 * n_face_pts
    P = np.zeros((nverts, 3), np.float64)
    P[:12] = V0
    t = np.arange(1, f) / f
    for (a, b), e in edges.items():
        P[base_e + e * n_edge_pts: base_e + (e + 1) * n_edge_pts] = V0[a][None] * (1 - t)[:, None] + V0[b][None] * t[:, None]
    # grid (i, j) on a face with corners (A, B, C): point = (k A + i B + j C) / f, k = f - i - j
    I, J = np.meshgrid(np.arange(f + 1), np.arange(f + 1), indexing="ij")
    mask = I + J <= f
    Ii, Jj = I[mask], J[mask]
    Kk = f - Ii - Jj
    interior = (Ii > 0) & (Jj > 0) & (Kk > 0)
    faces = []
    lin = -np.ones((f + 1, f + 1), np.int64)
    for fi, (A, B, C) in enumerate(F0):
        idx = np.empty(len(Ii), np.int64)
        # corners
        idx[(Ii == 0) & (Jj == 0)] = A
        idx[(Ii == f) & (Jj == 0)] = B
        idx[(Ii == 0) & (Jj == f)] = C

        def edge_pts(p, q, s):  # point at parameter s/f from corner p to corner q
            e = edges[(min(p, q), max(p, q))]
            s2 = np.where(p < q, s, f - s)
            return base_e + e * n_edge_pts + (s2 - 1)

        m = (Jj == 0) & (Ii > 0) & (Ii < f)            # edge A-B, parameter i
        idx[m] = edge_pts(A, B, Ii[m])
        m = (Ii == 0) & (Jj > 0) & (Jj < f)            # edge A-C, parameter j
        idx[m] = edge_pts(A, C, Jj[m])
        m = (Kk == 0) & (Ii > 0) & (Jj > 0)            # edge B-C, parameter j
        idx[m] = edge_pts(B, C, Jj[m])
        fb = base_f + fi * n_face_pts
        ids = fb + np.arange(int(interior.sum()))
        idx[interior] = ids
        P[ids] = (Kk[interior, None] * V0[A] + Ii[interior, None] * V0[B] + Jj[interior, None] * V0[C]) / f
        lin[Ii, Jj] = idx
        # triangles of the face grid
        gi, gj = np.meshgrid(np.arange(f), np.arange(f), indexing="ij")
        up = gi + gj <= f - 1
        a = lin[gi[up], gj[up]]
        b = lin[gi[up] + 1, gj[up]]
        c = lin[gi[up], gj[up] + 1]
        faces.append(np.stack([a, b, c], -1))
        dn = gi + gj <= f - 2
        a = lin[gi[dn] + 1, gj[dn]]
        b = lin[gi[dn] + 1, gj[dn] + 1]
        c = lin[gi[dn], gj[dn] + 1]
        faces.append(np.stack([a, b, c], -1))
    P /= np.linalg.norm(P, axis=1, keepdims=True)
    return P, np.concatenate(faces)


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343) ^ iy.astype(np.uint64) * np.uint64(0xD8163841)
         ^ iz.astype(np.uint64) * np.uint64(0xCB1AB31F) ^ np.uint64((seed * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF))
    h ^= h >> np.uint64(33)
    h *= np.uint64(0xFF51AFD7ED558CCD)
    h ^= h >> np.uint64(33)
    h *= np.uint64(0xC4CEB9FE1A85EC53)
    h ^= h >> np.uint64(33)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) * 2.0 - 1.0


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded 3D value noise in [-1, 1]: lattice values from an integer hash,
    smoothstep-weighted trilinear interpolation."""
    fl = np.floor(p)
    f = p - fl
    w = f * f * (3 - 2 * f)
    i = fl.astype(np.int64)
    out = np.zeros(len(p))
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1 - w[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1 - w[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out += wx * wy * wz * _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
    return out


def fbm(p: np.ndarray, seed: int, octaves: int = 6, lacunarity: float = 2.0, gain: float = 0.5,
        base_freq: float = 2.0) -> np.ndarray:
    total = np.zeros(len(p))
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        total += amp * value_noise(p * freq, seed + 7919 * o)
        norm += amp
        amp *= gain
        freq *= lacunarity
    return total / norm


@dataclass
class Icosphere:
    verts: np.ndarray   # (V, 3) float64, displaced
    faces: np.ndarray   # (F, 3) int64
    seed: int

    @property
    def n_tris(self) -> int:
        return len(self.faces)

    def frame(self, k: int, sigma: float = 1e-3) -> np.ndarray:
        """Soup of frame k: every shared vertex perturbed by N(0, sigma), seed = seed + k."""
        if sigma == 0.0:
            return deindex(self.verts, self.faces)
        rng = np.random.Generator(np.random.PCG64(self.seed + 1 + k))
        return deindex(self.verts + rng.normal(0.0, sigma, size=self.verts.shape), self.faces)


def icosphere(freq: int = 324, amplitude: float = 0.15, octaves: int = 6, seed: int = 2) -> Icosphere:
    """Geodesic icosphere, class I frequency `freq` (324 -> 2,099,520 triangles),
    radius 1 + amplitude * fBm(value noise, `octaves` octaves)."""
    P, F = geodesic_sphere(freq)
    P = P * (1.0 + amplitude * fbm(P, seed, octaves))[:, None]
    return Icosphere(P, F, seed)


# ---------------------------------------------------------------------------
def random_soup(n: int, seed: int, lo_len: float = 0.005, hi_len: float = 0.03) -> np.ndarray:
    """n triangles with centroids U[0,1]^3; each vertex = centroid + l * u,
    l ~ U(lo_len, hi_len), u uniform on the unit sphere."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.random((n, 1, 3))
    u = rng.normal(size=(n, 3, 3))
    u /= np.linalg.norm(u, axis=2, keepdims=True)
    ln = rng.uniform(lo_len, hi_len, size=(n, 3, 1))
    return np.ascontiguousarray((c + ln * u).reshape(n, 9).astype(np.float32))


@dataclass
class GIScene:
    tris: np.ndarray      # (n, 9) fp32
    albedo: np.ndarray    # (n, 3) fp32
    emission: np.ndarray  # (n, 3) fp32
    n_box: int
    n_emitter: int


def _quad(p0, p1, p2, p3):
    return [p0 + p1 + p2, p0 + p2 + p3]


def gi_box(n_soup: int = 262144, seed: int = 3, radiance: float = 10.0, wall_albedo: float = 0.75) -> GIScene:
    """Closed box [-0.1, 1.1]^3 (12 triangles), an emitting quad under the
    ceiling (2 triangles, radiance `radiance`) and `n_soup` random triangles
    with Lambertian albedo U[0.2, 0.8]^3: 262,158 triangles by default."""
    lo, hi = -0.1, 1.1
    c = [[lo, lo, lo], [hi, lo, lo], [hi, hi, lo], [lo, hi, lo], [lo, lo, hi], [hi, lo, hi], [hi, hi, hi], [lo, hi, hi]]
    box = []
    for q in ((0, 1, 2, 3), (4, 7, 6, 5), (0, 4, 5, 1), (3, 2, 6, 7), (0, 3, 7, 4), (1, 5, 6, 2)):
        box += _quad(*[c[k] for k in q])
    y = 1.09
    em = _quad([0.35, y, 0.35], [0.85, y, 0.35], [0.85, y, 0.85], [0.35, y, 0.85])
    fixed = np.array(box + em, np.float32)
    soup = random_soup(n_soup, seed)
    tris = np.ascontiguousarray(np.concatenate([fixed, soup]))
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    albedo = np.concatenate([np.full((12, 3), wall_albedo, np.float32), np.full((2, 3), 0.5, np.float32),
                             rng.uniform(0.2, 0.8, size=(n_soup, 3)).astype(np.float32)])
    emission = np.zeros((len(tris), 3), np.float32)
    emission[12:14] = radiance
    return GIScene(tris, np.ascontiguousarray(albedo), emission, 12, 2)


def gi_camera(width: int = 1024, height: int = 1024) -> Camera:
    return look_at((0.5, 0.55, -0.08), (0.5, 0.5, 1.0), vfov_deg=60.0, width=width, height=height)


def batch_sizes(n_scenes: int = 256, lo: int = 1000, hi: int = 200000, seed: int = 4) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.round(np.exp(rng.uniform(math.log(lo), math.log(hi), size=n_scenes))).astype(np.int64)


def batch_scene(sizes, seed_base: int = 1000) -> np.ndarray:
    """Concatenated soups of a batch: scene s = random_soup(sizes[s], seed_base + s)."""
    return np.ascontiguousarray(np.concatenate([random_soup(int(n), seed_base + i) for i, n in enumerate(sizes)]))


def batch_views(n_scenes: int, width: int = 256, height: int = 256):
    """One camera per scene, circling the unit cube of the soups at distance
    1.7 from its centre, and a light above the cube."""
    cams, lights = [], []
    for s in range(n_scenes):
        a = 2.0 * math.pi * s / max(1, n_scenes)
        eye = (0.5 + 1.7 * math.sin(a), 0.8, 0.5 - 1.7 * math.cos(a))
        cams.append(look_at(eye, (0.5, 0.5, 0.5), vfov_deg=60.0, width=width, height=height))
        lights.append((0.5 + 0.3 * math.cos(a), 2.5, 0.5 + 0.3 * math.sin(a)))
    return cams, np.asarray(lights, np.float32)


# Workload cameras / lights
TORUS_LIGHT = (1.0, 2.0, 3.0)


def torus_camera(width: int = 512, height: int = 512) -> Camera:
    return look_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), vfov_deg=60.0, width=width, height=height)


def sphere_camera(width: int = 1920, height: int = 1080) -> Camera:
    return look_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), vfov_deg=60.0, width=width, height=height)
