"""ctypes view of the reference's own CUDA kernels rebuilt for sm_103a.

TEST INFRASTRUCTURE ONLY: imported by tests/ and bench.py's baseline legs,
never by the product package.  The cubins come from the reference sources
(oracle/build.py, only where they are present); the harness that drives them
(oracle/ref_gpu/ref_gpu.cu) is this project's code.  The kernels run the
reference's fixed shape: 1024 particles, 640x480 depth buffers, the ACCV
intrinsics compiled into main.h, 512 table uniforms per particle.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

NPARTICLE = 1024
RAND_STRIDE = 512
ROWS, COLS = 480, 640
OK, ERR_CUDA, ERR_ARG, OUT_OF_FRAME = 0, 1, 2, 3

_f = C.POINTER(C.c_float)
_i32 = C.POINTER(C.c_int32)
_u32 = C.POINTER(C.c_uint32)


class Params(C.Structure):
    _fields_ = [("x_lo", C.c_float * 3), ("x_hi", C.c_float * 3), ("num_points", C.c_uint32),
                ("aabb_min_x", C.c_int32), ("aabb_max_x", C.c_int32),
                ("aabb_min_y", C.c_int32), ("aabb_max_y", C.c_int32)]


class RefError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%d: %s" % (status, msg))
        self.status = status


def cubin_path(kind: str = "ieee") -> str:
    return _build.REF_CUBINS[kind]


def available(kind: str = "ieee") -> bool:
    """The cubin exists (built from the reference sources) and nvcc can build
    the harness."""
    return os.path.exists(cubin_path(kind))


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build_refgpu())
        L.rg_last_error.restype = C.c_char_p
        L.rg_last_error.argtypes = [C.c_void_p]
        L.rg_close.argtypes = [C.c_void_p]
        for fn in ("rg_set_scene", "rg_set_rand_table", "rg_init", "rg_get_state", "rg_set_state",
                   "rg_render_score", "rg_best_and_update", "rg_solve"):
            getattr(L, fn).restype = C.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def uniform_table(seed: int, stream: int) -> np.ndarray:
    """d_randGen filled with the oracle's Philox draws (qo_uniform, here
    vectorised): row j, column p = draw j of particle p (the reference reads
    d_randGen[p + j*1024])."""
    M = np.uint64(0xFFFFFFFF)
    blocks = RAND_STRIDE // 4
    c0 = np.repeat(np.arange(blocks, dtype=np.uint64)[:, None], NPARTICLE, axis=1)
    c1 = np.repeat(np.arange(NPARTICLE, dtype=np.uint64)[None, :], blocks, axis=0)
    c2 = np.full_like(c0, np.uint64(stream))
    c3 = np.zeros_like(c0)
    k0, k1 = np.uint64(seed & 0xFFFFFFFF), np.uint64((seed >> 32) & 0xFFFFFFFF)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(0x9E3779B9)) & M
            k1 = (k1 + np.uint64(0xBB67AE85)) & M
        p0 = np.uint64(0xD2511F53) * c0
        p1 = np.uint64(0xCD9E8D57) * c2
        c0, c1, c2, c3 = (p1 >> np.uint64(32)) ^ c1 ^ k0, p1 & M, (p0 >> np.uint64(32)) ^ c3 ^ k1, p0 & M
    out = np.stack([c0, c1, c2, c3], axis=1).reshape(RAND_STRIDE, NPARTICLE)  # row 4b+lane = draw
    return ((out >> np.uint64(8)).astype(np.float32) * np.float32(2.0 ** -24)).astype(np.float32)


class RefKernels:
    """One loaded cubin and its device buffers."""

    def __init__(self, kind: str = "ieee"):
        self.L = lib()
        self.h = C.c_void_p()
        st = self.L.rg_open(cubin_path(kind).encode(), C.byref(self.h))
        if st != OK:
            msg = self.L.rg_last_error(self.h).decode() if self.h else "open failed"
            self.close()
            raise RefError(st, msg)

    def close(self):
        if self.h:
            self.L.rg_close(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        if st != OK:
            raise RefError(st, self.L.rg_last_error(self.h).decode())

    def set_scene(self, mesh, F, depth, t_lo, t_hi, num_points, aabb):
        mesh = np.ascontiguousarray(mesh, np.float32)
        depth = np.ascontiguousarray(depth, np.int32)
        assert depth.shape == (ROWS, COLS)
        prm = Params((C.c_float * 3)(*t_lo), (C.c_float * 3)(*t_hi), int(num_points), *[int(v) for v in aabb])
        self._check(self.L.rg_set_scene(self.h, _p(mesh, _f), C.c_uint32(F), _p(depth, _i32), C.byref(prm)))

    def set_rand_table(self, table):
        table = np.ascontiguousarray(table, np.float32)
        assert table.shape == (RAND_STRIDE, NPARTICLE)
        self._check(self.L.rg_set_rand_table(self.h, _p(table, _f)))

    def init(self):
        self._check(self.L.rg_init(self.h))

    def get_state(self) -> dict:
        s = {k: np.empty((7, NPARTICLE), np.float32) for k in ("pos", "vel", "pbest")}
        s.update(fit=np.empty(NPARTICLE, np.float32), pbest_fit=np.empty(NPARTICLE, np.float32),
                 best_fit=np.empty(1, np.float32), best_pose=np.empty(7, np.float32),
                 cursor=np.empty(NPARTICLE, np.uint32))
        self._check(self.L.rg_get_state(self.h, _p(s["pos"], _f), _p(s["vel"], _f), _p(s["pbest"], _f),
                                        _p(s["fit"], _f), _p(s["pbest_fit"], _f), _p(s["best_fit"], _f),
                                        _p(s["best_pose"], _f), _p(s["cursor"], _u32)))
        return s

    def set_state(self, pos=None, vel=None, pbest=None, fit=None, pbest_fit=None, best_fit=None,
                  best_pose=None, cursor=None):
        def a(x, shape, dt):
            if x is None:
                return None
            x = np.ascontiguousarray(x, dt)
            assert x.size == int(np.prod(shape))
            return x

        st7 = (7, NPARTICLE)
        pos, vel, pbest = a(pos, st7, np.float32), a(vel, st7, np.float32), a(pbest, st7, np.float32)
        fit, pbest_fit = a(fit, (NPARTICLE,), np.float32), a(pbest_fit, (NPARTICLE,), np.float32)
        best_fit, best_pose = a(best_fit, (1,), np.float32), a(best_pose, (7,), np.float32)
        cursor = a(cursor, (NPARTICLE,), np.uint32)
        self._check(self.L.rg_set_state(self.h, _p(pos, _f), _p(vel, _f), _p(pbest, _f), _p(fit, _f),
                                        _p(pbest_fit, _f), _p(best_fit, _f), _p(best_pose, _f),
                                        _p(cursor, _u32)))

    def render_score(self, n: int, want_depth: bool = False):
        """Depth buffers as rendered (n x 480 x 640, or None), render boxes
        (n x 4: minX, maxX, minY, maxY) and fitness (n)."""
        depth = np.empty((n, ROWS, COLS), np.int32) if want_depth else None
        aabb = np.empty((n, 4), np.int32)
        self._check(self.L.rg_render_score(self.h, C.c_uint32(n), _p(depth, _i32), _p(aabb, _i32)))
        return depth, aabb, self.get_state()["fit"][:n].copy()

    def best_and_update(self):
        self._check(self.L.rg_best_and_update(self.h))

    def solve(self, iterations: int) -> dict:
        trace = np.zeros(iterations, np.float32)
        ms = C.c_double(0.0)
        done = C.c_uint32(0)
        st = self.L.rg_solve(self.h, C.c_uint32(iterations), _p(trace, _f), C.byref(ms), C.byref(done))
        out = {"status": st, "trace": trace[:done.value], "ms": ms.value, "done": done.value,
               "error": self.L.rg_last_error(self.h).decode() if st != OK else ""}
        if st not in (OK, OUT_OF_FRAME):
            raise RefError(st, out["error"])
        return out


def in_frame(mesh, F, poses, margin: float = 8.0, min_z: float = 0.05) -> np.ndarray:
    """Mirror of the harness's in-frame check (ref_gpu.cu, check_in_frame)
    for poses (n x 7): True where all eight object-box corners project at
    least `margin` px inside the image with the reference's ACCV camera."""
    m = np.asarray(mesh, np.float64).reshape(3, 3 * F)
    lo, hi = m.min(axis=1), m.max(axis=1)
    ok = np.ones(len(poses), bool)
    for i, s in enumerate(np.asarray(poses, np.float64)):
        u = s[4:7]
        for k in range(8):
            v = np.array([hi[0] if k & 1 else lo[0], hi[1] if k & 2 else lo[1], hi[2] if k & 4 else lo[2]])
            t = 2 * np.cross(u, v)
            w = v + s[3] * t + np.cross(u, t) + s[:3]
            if not w[2] >= min_z:
                ok[i] = False
                break
            x = 325.26110 + 572.41140 * (w[0] / w[2])
            y = 242.04899 + 573.57043 * (w[1] / w[2])
            if not (margin <= x <= COLS - margin and margin <= y <= ROWS - margin):
                ok[i] = False
                break
    return ok
