"""Seeded synthetic RGB-D workloads for the pose solver.

The reference runs on the ACCV/LINEMOD captures (main.cu:1231-1241), which
are not available here; these procedural scenes stand in for them with the
shapes, sizes and value distributions of the benchmark configurations:
perturbed icospheres, boxes and capped cylinders; a 640x480 pinhole camera
(fx=fy=525, cx=319.5, cy=239.5); uint16 depth in mm over a plane at 1300 mm
tilted by 10 degrees; Gaussian noise sigma = 1.5 (z/1000)^2 mm and 5% of the
pixels zeroed.  Meshes are returned in the loadOBJ3 SoA layout, in metres.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SCENE_LIB = os.path.join(HERE, "_build", "libqpso_scene.so")

W, H = 640, 480
FX = FY = 525.0
CX, CY = 319.5, 239.5
PLANE_Z_MM = 1300.0
PLANE_TILT_DEG = 10.0

_lib = None


def build_scene_lib(force: bool = False) -> str:
    src = os.path.join(HERE, "csrc", "scene.cpp")
    if not force and os.path.exists(SCENE_LIB) and os.path.getmtime(SCENE_LIB) >= os.path.getmtime(src):
        return SCENE_LIB
    os.makedirs(os.path.dirname(SCENE_LIB), exist_ok=True)
    tmp = SCENE_LIB + ".tmp%d" % os.getpid()
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-o", tmp], check=True)
    os.replace(tmp, SCENE_LIB)
    return SCENE_LIB


def _scene_lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_scene_lib())
        _lib.qs_render_depth.restype = None
    return _lib


# --------------------------------------------------------------------------
# meshes (vertices V [n,3] in metres, faces Fc [m,3] int)

def icosphere(level: int):
    t = (1.0 + 5 ** 0.5) / 2
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    Fc = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                   [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                   [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                   [8, 6, 7], [9, 8, 1]], np.int64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    for _ in range(level):
        e = np.concatenate([Fc[:, [0, 1]], Fc[:, [1, 2]], Fc[:, [2, 0]]])
        es = np.sort(e, axis=1)
        uniq, inv = np.unique(es, axis=0, return_inverse=True)
        mid = V[uniq[:, 0]] + V[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(V)
        V = np.concatenate([V, mid])
        m = len(Fc)
        a = base + inv[:m]
        b = base + inv[m:2 * m]
        c = base + inv[2 * m:]
        v0, v1, v2 = Fc[:, 0], Fc[:, 1], Fc[:, 2]
        Fc = np.concatenate([np.stack([v0, a, c], 1), np.stack([v1, b, a], 1),
                             np.stack([v2, c, b], 1), np.stack([a, b, c], 1)])
    return V, Fc


def uv_ellipsoid(n_faces: int):
    """Latitude-longitude sphere with about n_faces triangles."""
    n_lon = max(4, int(round(math.sqrt(n_faces))))
    n_lat = max(2, int(round(n_faces / (2 * n_lon))) + 1)
    th = np.linspace(0, math.pi, n_lat + 1)
    ph = np.linspace(0, 2 * math.pi, n_lon, endpoint=False)
    V = [[0, 0, 1.0]]
    for i in range(1, n_lat):
        for j in range(n_lon):
            V.append([math.sin(th[i]) * math.cos(ph[j]), math.sin(th[i]) * math.sin(ph[j]),
                      math.cos(th[i])])
    V.append([0, 0, -1.0])
    V = np.array(V)
    F = []
    ring = lambda i, j: 1 + (i - 1) * n_lon + (j % n_lon)
    for j in range(n_lon):
        F.append([0, ring(1, j), ring(1, j + 1)])
    for i in range(1, n_lat - 1):
        for j in range(n_lon):
            a, b = ring(i, j), ring(i, j + 1)
            c, d = ring(i + 1, j), ring(i + 1, j + 1)
            F.append([a, c, d])
            F.append([a, d, b])
    last = len(V) - 1
    for j in range(n_lon):
        F.append([last, ring(n_lat - 1, j + 1), ring(n_lat - 1, j)])
    return V, np.array(F, np.int64)


def box(n: int):
    """Unit cube [-1,1]^3 with each face split into n x n quads."""
    Vs, Fs, off = [], [], 0
    g = np.linspace(-1, 1, n + 1)
    uu, vv = np.meshgrid(g, g, indexing="ij")
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            P = np.zeros(((n + 1) ** 2, 3))
            a1, a2 = (axis + 1) % 3, (axis + 2) % 3
            P[:, axis] = sgn
            P[:, a1] = uu.ravel()
            P[:, a2] = vv.ravel()
            idx = lambda i, j: off + i * (n + 1) + j
            for i in range(n):
                for j in range(n):
                    q = [idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)]
                    if sgn > 0:
                        Fs += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
                    else:
                        Fs += [[q[0], q[2], q[1]], [q[0], q[3], q[2]]]
            Vs.append(P)
            off += len(P)
    return np.concatenate(Vs), np.array(Fs, np.int64)


def capped_cylinder(segments: int, rings: int):
    """Cylinder of radius 1 along z in [-1, 1] with fan caps."""
    ph = np.linspace(0, 2 * math.pi, segments, endpoint=False)
    zs = np.linspace(-1, 1, rings + 1)
    V = [[math.cos(p), math.sin(p), z] for z in zs for p in ph]
    bot, top = len(V), len(V) + 1
    V += [[0, 0, -1.0], [0, 0, 1.0]]
    F = []
    for r in range(rings):
        for s in range(segments):
            a = r * segments + s
            b = r * segments + (s + 1) % segments
            c = a + segments
            d = b + segments
            F += [[a, b, d], [a, d, c]]
    for s in range(segments):
        F.append([bot, (s + 1) % segments, s])
        F.append([top, rings * segments + s, rings * segments + (s + 1) % segments])
    return np.array(V), np.array(F, np.int64)


def _perlin_perm(seed: int):
    p = np.random.default_rng(seed).permutation(256)
    return np.concatenate([p, p])


def perlin3(P: np.ndarray, seed: int) -> np.ndarray:
    """Improved gradient noise (K. Perlin, SIGGRAPH 2002) at points P [n,3]."""
    perm = _perlin_perm(seed)
    Pi = np.floor(P).astype(np.int64)
    f = P - Pi
    Pi &= 255
    fade = lambda t: t * t * t * (t * (t * 6 - 15) + 10)
    u, v, w = fade(f[:, 0]), fade(f[:, 1]), fade(f[:, 2])
    X, Y, Z = Pi[:, 0], Pi[:, 1], Pi[:, 2]

    def grad(h, x, y, z):
        h = h & 15
        a = np.where(h < 8, x, y)
        b = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
        return np.where(h & 1, -a, a) + np.where(h & 2, -b, b)

    A = perm[X] + Y
    AA, AB = perm[A] + Z, perm[A + 1] + Z
    B = perm[X + 1] + Y
    BA, BB = perm[B] + Z, perm[B + 1] + Z
    x, y, z = f[:, 0], f[:, 1], f[:, 2]
    lerp = lambda t, a, b: a + t * (b - a)
    return lerp(w, lerp(v, lerp(u, grad(perm[AA], x, y, z), grad(perm[BA], x - 1, y, z)),
                        lerp(u, grad(perm[AB], x, y - 1, z), grad(perm[BB], x - 1, y - 1, z))),
                lerp(v, lerp(u, grad(perm[AA + 1], x, y, z - 1), grad(perm[BA + 1], x - 1, y, z - 1)),
                     lerp(u, grad(perm[AB + 1], x, y - 1, z - 1),
                          grad(perm[BB + 1], x - 1, y - 1, z - 1))))


def bump(V: np.ndarray, amp: float, freq: float, seed: int) -> np.ndarray:
    """Radial displacement by +-amp (same units as V) of seeded Perlin noise."""
    r = np.linalg.norm(V, axis=1, keepdims=True)
    n = perlin3(V * freq, seed)
    return V * (1 + amp * n[:, None] / np.maximum(r, 1e-12))


def to_soa(V: np.ndarray, Fc: np.ndarray) -> np.ndarray:
    """loadOBJ3 layout (main.h:620-679): soa[f + j*F + c*3F] = V[Fc[f,j], c]."""
    Fn = len(Fc)
    soa = np.empty(9 * Fn, np.float32)
    for c in range(3):
        for j in range(3):
            soa[(3 * c + j) * Fn:(3 * c + j + 1) * Fn] = V[Fc[:, j], c]
    return soa


def make_mesh(kind: str, n_faces: int, extent_mm: float, seed: int, bump_mm: float = 3.0):
    """Procedural mesh scaled to `extent_mm` (largest dimension) with radial
    Perlin bumps of +-bump_mm.  Returns (soa, F)."""
    rng = np.random.default_rng(seed)
    if kind == "icosphere":
        level = max(0, int(round(math.log(max(n_faces, 20) / 20, 4))))
        V, Fc = icosphere(level)
        axes = np.array([1.0, rng.uniform(0.55, 1.0), rng.uniform(0.4, 0.9)])
    elif kind == "ellipsoid":
        V, Fc = uv_ellipsoid(n_faces)
        axes = np.array([1.0, rng.uniform(0.55, 1.0), rng.uniform(0.4, 0.9)])
    elif kind == "box":
        n = max(1, int(round(math.sqrt(n_faces / 12))))
        V, Fc = box(n)
        axes = np.array([1.0, rng.uniform(0.5, 1.0), rng.uniform(0.3, 0.8)])
    elif kind == "cylinder":
        seg = max(8, int(round(math.sqrt(n_faces / 2))))
        rings = max(1, int(round((n_faces - 2 * seg) / (2 * seg))))
        V, Fc = capped_cylinder(seg, rings)
        axes = np.array([rng.uniform(0.35, 0.6), rng.uniform(0.35, 0.6), 1.0])
    else:
        raise ValueError(kind)
    V = V * axes
    half = extent_mm / 2.0 / 1000.0
    V = V * (half / np.abs(V).max())
    if bump_mm > 0:
        V = bump(V, bump_mm / 1000.0, 8.0 / (extent_mm / 1000.0) / 8.0, seed + 7)
    return to_soa(V, Fc), len(Fc)


def ellipsoid_c1(seed: int = 0):
    """1280-triangle icosphere (subdivision 3) scaled to 60x40x30 mm semi-axes
    with +-3 mm Perlin bumps."""
    V, Fc = icosphere(3)
    V = V * np.array([0.060, 0.040, 0.030])
    V = bump(V, 0.003, 25.0, seed + 7)
    return to_soa(V, Fc), len(Fc)


# --------------------------------------------------------------------------
# poses and frames

def random_quat(rng) -> np.ndarray:
    """Uniform on SO(3) (Shoemake), scalar first, q0 >= 0."""
    u1, u2, u3 = rng.uniform(size=3)
    q = np.array([math.sqrt(u1) * math.cos(2 * math.pi * u3),
                  math.sqrt(1 - u1) * math.sin(2 * math.pi * u2),
                  math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3)])
    return q if q[0] >= 0 else -q


def camera_K():
    return np.array([FX, FY, CX, CY], np.float32)


def plane_depth(w=W, h=H, z_mm=PLANE_Z_MM, tilt_deg=PLANE_TILT_DEG) -> np.ndarray:
    """Depth (mm) of a plane through (0,0,z_mm) whose normal is tilted about x."""
    t = math.radians(tilt_deg)
    n = np.array([0.0, math.sin(t), math.cos(t)])
    uu, vv = np.meshgrid(np.arange(w), np.arange(h))
    rx, ry = (uu - CX) / FX, (vv - CY) / FY
    return (n[2] * z_mm) / (n[0] * rx + n[1] * ry + n[2])


def render_gt(soa, F, pose, zbuf, labels, label_value):
    L = _scene_lib()
    p = np.ascontiguousarray(pose, np.float32)
    K = camera_K()
    s = np.ascontiguousarray(soa, np.float32)
    L.qs_render_depth(s.ctypes.data_as(C.c_void_p), C.c_uint32(F), p.ctypes.data_as(C.c_void_p),
                      K.ctypes.data_as(C.c_void_p), C.c_int32(zbuf.shape[1]), C.c_int32(zbuf.shape[0]),
                      zbuf.ctypes.data_as(C.c_void_p), labels.ctypes.data_as(C.c_void_p),
                      C.c_int32(label_value))


def finish_depth(zf: np.ndarray, rng) -> np.ndarray:
    z = zf + rng.normal(size=zf.shape) * 1.5 * (zf / 1000.0) ** 2
    z = np.clip(np.rint(z), 0, 65535).astype(np.uint16)
    z[rng.uniform(size=z.shape) < 0.05] = 0
    return z


def compose_frame(objects, seed: int, with_rgb: bool = False):
    """objects: list of (soa, F, pose7).  Returns depth uint16 [H,W], labels
    int32 [H,W] (-1 = plane), rgb uint8 [H,W,3] or None."""
    rng = np.random.default_rng(seed)
    zf = plane_depth().astype(np.float32)
    labels = np.full((H, W), -1, np.int32)
    for k, (soa, F, pose) in enumerate(objects):
        render_gt(soa, F, pose, zf, labels, k)
    depth = finish_depth(zf, rng)
    rgb = None
    if with_rgb:
        base = rng.integers(40, 216, size=(len(objects) + 1, 3))
        rgb = base[labels + 1].astype(np.float64) + rng.normal(0, 8, size=(H, W, 3))
        rgb = np.clip(np.rint(rgb), 0, 255).astype(np.uint8)
    return depth, labels, rgb


def cluster_info(depth: np.ndarray, labels: np.ndarray, k: int):
    """SegResults-like record of cluster k (GraphCannySeg.h:594-618):
    pixel count, bounding rectangle (max exclusive) and 3D centroid (mm)."""
    m = labels == k
    ys, xs = np.nonzero(m)
    if len(xs) == 0:
        return None
    z = depth[ys, xs].astype(np.float64)
    v = z > 0
    X = (xs[v] - CX) * z[v] / FX
    Y = (ys[v] - CY) * z[v] / FY
    cen = [float(X.mean()), float(Y.mean()), float(z[v].mean())] if v.any() else [0.0, 0.0, 1000.0]
    return {"label": k, "num_points": int(m.sum()), "aabb": (int(xs.min()), int(xs.max()) + 1,
                                                            int(ys.min()), int(ys.max()) + 1),
            "centroid_mm": cen}


def place_pose(rng, soa, F, z_range=(0.6, 1.0), margin_px=10, taken=None, tries=200):
    """Pose with q uniform on SO(3), z in z_range (m), and the projected mesh
    inside the frame (and, if `taken` masks are given, not overlapping)."""
    V = np.stack([soa[0:F], soa[3 * F:4 * F], soa[6 * F:7 * F]], 1).astype(np.float64)
    for _ in range(tries):
        q = random_quat(rng)
        z = rng.uniform(*z_range)
        u = rng.uniform(margin_px + 40, W - margin_px - 40)
        v = rng.uniform(margin_px + 40, H - margin_px - 40)
        t = np.array([(u - CX) * z / FX, (v - CY) * z / FY, z])
        q0, q1, q2, q3 = q
        R = np.array([[1 - 2 * (q2 * q2 + q3 * q3), 2 * (q1 * q2 - q0 * q3), 2 * (q1 * q3 + q0 * q2)],
                      [2 * (q1 * q2 + q0 * q3), 1 - 2 * (q1 * q1 + q3 * q3), 2 * (q2 * q3 - q0 * q1)],
                      [2 * (q1 * q3 - q0 * q2), 2 * (q2 * q3 + q0 * q1), 1 - 2 * (q1 * q1 + q2 * q2)]])
        P = V @ R.T + t
        pu = CX + FX * P[:, 0] / P[:, 2]
        pv = CY + FY * P[:, 1] / P[:, 2]
        box = (pu.min() - margin_px, pu.max() + margin_px, pv.min() - margin_px, pv.max() + margin_px)
        if box[0] < 0 or box[2] < 0 or box[1] >= W or box[3] >= H:
            continue
        if taken is not None and any(not (box[1] < b[0] or b[1] < box[0] or box[3] < b[2] or b[3] < box[2])
                                     for b in taken):
            continue
        if taken is not None:
            taken.append(box)
        return np.array([*t, *q], np.float32)
    raise RuntimeError("could not place object")


# --------------------------------------------------------------------------
# benchmark workloads

def workload_c1(seed: int = 0):
    """Plain single solve, small: one 1280-face ellipsoid, one cluster,
    64 particles x 50 iterations, Philox seed 0."""
    rng = np.random.default_rng(1000 + seed)
    soa, F = ellipsoid_c1(seed)
    pose = place_pose(rng, soa, F)
    depth, labels, _ = compose_frame([(soa, F, pose)], seed=2000 + seed)
    info = cluster_info(depth, labels, 0)
    return {"meshes": [(soa, F)], "frames": [(depth, labels, None)],
            "solves": [dict(mesh=0, frame=0, cluster=info, particles=64, iterations=50, seed=0,
                            stream=0, gt_pose=pose)]}


def workload_c2(seed: int = 0, frames: int = 1, particles: int = 256, iterations: int = 100):
    """Production size: per frame 8 non-overlapping objects drawn from 4
    procedural meshes (5k faces, 50-200 mm), RGB with per-object colour."""
    rng = np.random.default_rng(3000 + seed)
    kinds = ["icosphere", "box", "cylinder", "ellipsoid"]
    meshes = [make_mesh(k, 5000 if k != "icosphere" else 5120, rng.uniform(50, 200), seed * 10 + i)
              for i, k in enumerate(kinds)]
    fr, solves = [], []
    for fi in range(frames):
        taken = []
        objs, mids = [], []
        for k in range(8):
            mi = int(rng.integers(0, 4))
            soa, F = meshes[mi]
            pose = place_pose(rng, soa, F, margin_px=4, taken=taken, tries=2000)
            objs.append((soa, F, pose))
            mids.append(mi)
        depth, labels, rgb = compose_frame(objs, seed=4000 + seed * 100 + fi, with_rgb=True)
        fr.append((depth, labels, rgb))
        for k in range(8):
            info = cluster_info(depth, labels, k)
            if info is None:
                continue
            solves.append(dict(mesh=mids[k], frame=fi, cluster=info, particles=particles,
                               iterations=iterations, seed=seed, stream=len(solves),
                               gt_pose=objs[k][2]))
    return {"meshes": meshes, "frames": fr, "solves": solves}


def workload_c3(seed: int = 0, n_frames: int = 8, per_frame: int = 8, iterations: int = 100,
                particle_choices=(128, 256, 512, 1024)):
    """Batching: 64 clusters from 8 frames, meshes log-uniform in 1k-50k
    faces, cluster windows 40x40 .. 300x300 px, particles in {128..1024}."""
    rng = np.random.default_rng(5000 + seed)
    kinds = ["ellipsoid", "box", "cylinder"]
    meshes, fr, solves = [], [], []
    for fi in range(n_frames):
        taken, objs, mids = [], [], []
        k = 0
        while k < per_frame:
            nf = int(round(math.exp(rng.uniform(math.log(1000), math.log(50000)))))
            win = math.exp(rng.uniform(math.log(40), math.log(300)))
            z = rng.uniform(0.6, 1.0)
            extent = win * z * 1000.0 / FX
            soa, F = make_mesh(kinds[int(rng.integers(0, 3))], nf, extent, seed * 1000 + len(meshes))
            try:
                pose = place_pose(rng, soa, F, z_range=(z, z), margin_px=2, taken=taken, tries=400)
            except RuntimeError:
                continue
            meshes.append((soa, F))
            objs.append((soa, F, pose))
            mids.append(len(meshes) - 1)
            k += 1
        depth, labels, _ = compose_frame(objs, seed=6000 + seed * 100 + fi)
        fr.append((depth, labels, None))
        for j in range(per_frame):
            info = cluster_info(depth, labels, j)
            if info is None:
                continue
            solves.append(dict(mesh=mids[j], frame=fi, cluster=info,
                               particles=int(rng.choice(particle_choices)), iterations=iterations,
                               seed=seed, stream=len(solves), gt_pose=objs[j][2]))
    return {"meshes": meshes, "frames": fr, "solves": solves}


def workload_c4(seed: int = 0, n_meshes: int = 16, n_frames: int = 32, per_frame: int = 4,
                iterations: int = 100, particle_choices=(256, 1024)):
    """Serving pool: 16 resident procedural meshes (log-uniform 2k-100k
    faces, 50-200 mm) and 32 resident 640x480 frames, each showing
    `per_frame` objects drawn from the pool.  Every (frame, cluster) pair is
    a possible request, solved with the mesh that made the cluster."""
    rng = np.random.default_rng(9000 + seed)
    kinds = ["ellipsoid", "box", "cylinder"]
    meshes = []
    for i in range(n_meshes):
        nf = int(round(math.exp(rng.uniform(math.log(2000), math.log(100000)))))
        meshes.append(make_mesh(kinds[i % 3], nf, rng.uniform(50, 200), seed * 100 + i))
    fr, solves = [], []
    for fi in range(n_frames):
        taken, objs, mids = [], [], []
        while len(objs) < per_frame:
            mi = int(rng.integers(0, n_meshes))
            soa, F = meshes[mi]
            try:
                pose = place_pose(rng, soa, F, margin_px=2, taken=taken, tries=400)
            except RuntimeError:
                continue
            objs.append((soa, F, pose))
            mids.append(mi)
        depth, labels, _ = compose_frame(objs, seed=9500 + seed * 100 + fi)
        fr.append((depth, labels, None))
        for j in range(per_frame):
            info = cluster_info(depth, labels, j)
            if info is None:
                continue
            solves.append(dict(mesh=mids[j], frame=fi, cluster=info,
                               particles=int(rng.choice(particle_choices)), iterations=iterations,
                               seed=seed, stream=len(solves), gt_pose=objs[j][2]))
    return {"meshes": meshes, "frames": fr, "solves": solves}


def segmentation_frame_c5(seed: int = 0, n_objects: int = 15):
    """The stress configuration's segmentation input: one 640x480 RGB-D
    frame with 15 non-overlapping objects (procedural meshes of 2k-3k faces,
    40-120 mm) over the tilted plane, each object with its own base colour
    and sigma=8 per-channel noise, depth noise and 5% dropout.  Returns
    (depth uint16, ground-truth labels int32, bgr uint8)."""
    rng = np.random.default_rng(11000 + seed)
    kinds = ["icosphere", "box", "cylinder", "ellipsoid"]
    meshes = [make_mesh(k, 2560 if k == "icosphere" else 2400, rng.uniform(40, 120), seed * 10 + i)
              for i, k in enumerate(kinds)]
    taken, objs = [], []
    while len(objs) < n_objects:
        soa, F = meshes[int(rng.integers(0, len(meshes)))]
        try:
            pose = place_pose(rng, soa, F, margin_px=3, taken=taken, tries=400)
        except RuntimeError:
            continue
        objs.append((soa, F, pose))
    depth, labels, rgb = compose_frame(objs, seed=12000 + seed, with_rgb=True)
    return depth, labels, rgb


def workload_c5(seed: int = 0, particles: int = 4096, iterations: int = 200, level: int = 7):
    """Stress: one noise-displaced level-7 icosphere (250 mm extent) and a
    full 640x480 fitness window (cluster AABB = the frame)."""
    rng = np.random.default_rng(7000 + seed)
    V, Fc = icosphere(level)
    V = V * 0.125
    V = bump(V, 0.004, 12.0, seed + 11)
    soa, F = to_soa(V, Fc), len(Fc)
    pose = place_pose(rng, soa, F, z_range=(0.8, 1.0))
    depth, labels, _ = compose_frame([(soa, F, pose)], seed=8000 + seed)
    info = cluster_info(depth, labels, 0)
    info["aabb"] = (0, W, 0, H)
    return {"meshes": [(soa, F)], "frames": [(depth, labels, None)],
            "solves": [dict(mesh=0, frame=0, cluster=info, particles=particles,
                            iterations=iterations, seed=seed, stream=0, gt_pose=pose)]}


def solve_fields(s: dict) -> dict:
    """SolveDesc fields (except mesh/frame ids) for a workload solve entry:
    the cluster record of the segmentation and the reference's translation
    box of +-0.3 m around the centroid (main.cu:1285-1323)."""
    c = s["cluster"]
    cen = c["centroid_mm"]
    lo = [np.float32(np.float32(x) * np.float32(0.001)) - np.float32(0.3) for x in cen]
    hi = [np.float32(np.float32(x) * np.float32(0.001)) + np.float32(0.3) for x in cen]
    x0, x1, y0, y1 = c["aabb"]
    return dict(cluster_label=c["label"], cl_min_x=x0, cl_max_x=x1, cl_min_y=y0, cl_max_y=y1,
                num_points=c["num_points"], t_lo=[float(v) for v in lo], t_hi=[float(v) for v in hi],
                num_particles=s["particles"], iterations=s["iterations"], seed=s["seed"],
                stream=s["stream"])


def camera_tuple():
    return (FX, FY, CX, CY, W, H)


def masked_depth(depth: np.ndarray, labels: np.ndarray, k: int) -> np.ndarray:
    return np.where(labels == k, depth, 0).astype(np.uint16)
