"""ctypes view of the oracle and of the reference pin library.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline arm, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

NDIM = 7
DEPTH_BG = 60000
GUARD = 1024

_f = C.POINTER(C.c_float)
_i32 = C.POINTER(C.c_int32)
_u16 = C.POINTER(C.c_uint16)


class Camera(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("width", C.c_int32), ("height", C.c_int32), ("proj", C.c_int32)]


PROJ_FP32, PROJ_REF_ACCV = 0, 1


class Params(C.Structure):
    _fields_ = [("c1", C.c_float), ("c2", C.c_float), ("w", C.c_double), ("vdot", C.c_float),
                ("ang_lo", C.c_float), ("ang_hi", C.c_float), ("qinit", C.c_float * 4),
                ("t_lo", C.c_float * 3), ("t_hi", C.c_float * 3),
                ("cl_min_x", C.c_int32), ("cl_max_x", C.c_int32),
                ("cl_min_y", C.c_int32), ("cl_max_y", C.c_int32),
                ("num_points", C.c_uint32), ("num_particles", C.c_uint32),
                ("iterations", C.c_uint32), ("seed", C.c_uint64), ("stream", C.c_uint32),
                ("raster_mode", C.c_uint32)]


RASTER_REF, RASTER_EDGE = 0, 1


class Score(C.Structure):
    _fields_ = [("n_rendered", C.c_uint32), ("n_no_obs", C.c_uint32),
                ("n_seg_rendered", C.c_uint32), ("n_seg_not_rendered", C.c_uint32),
                ("sq_lo", C.c_uint64), ("sq_hi", C.c_uint64),
                ("r_min_x", C.c_int32), ("r_max_x", C.c_int32),
                ("r_min_y", C.c_int32), ("r_max_y", C.c_int32),
                ("w_min_x", C.c_int32), ("w_max_x", C.c_int32),
                ("w_min_y", C.c_int32), ("w_max_y", C.c_int32),
                ("partial_len", C.c_int32), ("fit", C.c_float)]


class Result(C.Structure):
    _fields_ = [("gbest_fit", C.c_float), ("gbest", C.c_float * 7), ("raster_writes", C.c_uint64)]


_lib = None
_pin = None
_segpin = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.qo_uniform.restype = C.c_float
        L.qo_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        for fn in ("qo_sin", "qo_cos", "qo_acos"):
            getattr(L, fn).restype = C.c_double
            getattr(L, fn).argtypes = [C.c_double]
        for fn in ("qo_sinf", "qo_cosf", "qo_acosf"):
            getattr(L, fn).restype = C.c_float
            getattr(L, fn).argtypes = [C.c_float]
        L.qo_raster_face.restype = C.c_int64
        L.qo_render.restype = C.c_int64
        L.qo_raster_face_mode.restype = C.c_int64
        L.qo_render_mode.restype = C.c_int64
        L.qo_fitness_from_counts.restype = C.c_float
        L.qo_fitness_from_counts.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64,
                                             C.c_uint64, C.c_uint32]
        L.qo_fitness_fp64.restype = C.c_double
        L.qo_domain_w.restype = C.c_int32
        L.qo_domain_h.restype = C.c_int32
        L.qo_solve.restype = C.c_int
        L.qo_solve_mt.restype = C.c_int
        L.qo_edge_weight.restype = C.c_float
        L.qo_segment_graph.restype = C.c_int32
        L.qo_segment_graph.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_float, C.c_float,
                                       C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def pin():
    """The reference's main.h helpers compiled for the host (None where the
    reference sources are absent)."""
    global _pin
    if _pin is None:
        path = _build.build_ref_pin()
        if path is None:
            return None
        _pin = C.CDLL(path)
    return _pin


def segpin():
    """The reference's segmentation core (union-find forest, segment_graph,
    small-component merge, collectSets) compiled for the host (None where
    the reference sources are absent)."""
    global _segpin
    if _segpin is None:
        path = _build.build_seg_pin()
        if path is None:
            return None
        _segpin = C.CDLL(path)
        _segpin.sp_segment.restype = C.c_int
    return _segpin


def ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def camera(fx=525.0, fy=525.0, cx=319.5, cy=239.5, width=640, height=480, proj=PROJ_FP32) -> Camera:
    return Camera(fx, fy, cx, cy, width, height, proj)


def camera_ref_accv() -> Camera:
    """The reference's compiled-in ACCV camera (main.h:30-33), projected in
    double as its kernels do."""
    return Camera(572.41140, 573.57043, 325.26110, 242.04899, 640, 480, PROJ_REF_ACCV)


def default_params() -> Params:
    p = Params()
    lib().qo_default_params(C.byref(p))
    return p


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().qo_philox4x32_10(c, k, o)
    return list(o)


def uniform(seed, stream, particle, draw) -> float:
    return lib().qo_uniform(seed, stream, particle, draw)


def zbuf_new(cam: Camera) -> np.ndarray:
    L = lib()
    return np.full((L.qo_domain_h(C.byref(cam)), L.qo_domain_w(C.byref(cam))), DEPTH_BG,
                   dtype=np.int32)


def project(s7, v3, cam: Camera):
    s = np.ascontiguousarray(s7, dtype=np.float32)
    v = np.ascontiguousarray(v3, dtype=np.float32)
    o = np.zeros(3, np.float32)
    lib().qo_project(ptr(s, _f), ptr(v, _f), C.byref(cam), ptr(o, _f))
    return o


def raster_face(v1, v2, v3, cam: Camera, zbuf: np.ndarray, box=None, mode: int = RASTER_REF):
    a = np.ascontiguousarray(v1, np.float32)
    b = np.ascontiguousarray(v2, np.float32)
    c = np.ascontiguousarray(v3, np.float32)
    if box is None:
        box = np.array([50000, -1, 50000, -1], np.int32)
    n = lib().qo_raster_face_mode(ptr(a, _f), ptr(b, _f), ptr(c, _f), C.byref(cam),
                                  ptr(zbuf, _i32), ptr(box, _i32), C.c_uint32(mode))
    return n, box


def render(mesh: np.ndarray, num_faces: int, s7, cam: Camera, zbuf: np.ndarray | None = None,
           mode: int = RASTER_REF):
    if zbuf is None:
        zbuf = zbuf_new(cam)
    s = np.ascontiguousarray(s7, np.float32)
    box = np.zeros(4, np.int32)
    m = np.ascontiguousarray(mesh, np.float32)
    n = lib().qo_render_mode(ptr(m, _f), C.c_uint32(num_faces), ptr(s, _f), C.byref(cam),
                             ptr(zbuf, _i32), ptr(box, _i32), C.c_uint32(mode))
    return zbuf, box, n


def render_cpu(mesh: np.ndarray, num_faces: int, s7, cam: Camera) -> np.ndarray:
    """The reference's host render of a pose (RenderCPU): float depth over
    the image, background 60000."""
    out = np.empty((cam.height, cam.width), np.float32)
    s = np.ascontiguousarray(s7, np.float32)
    m = np.ascontiguousarray(mesh, np.float32)
    lib().qo_render_cpu(ptr(m, _f), C.c_uint32(num_faces), ptr(s, _f), C.byref(cam), ptr(out, _f))
    return out


def raster_face_cpu(v1, v2, v3, cam: Camera, depth: np.ndarray) -> None:
    a, b, c = (np.ascontiguousarray(v, np.float32) for v in (v1, v2, v3))
    lib().qo_raster_face_cpu(ptr(a, _f), ptr(b, _f), ptr(c, _f), C.byref(cam), ptr(depth, _f))


def score(zbuf: np.ndarray, box: np.ndarray, obs: np.ndarray, cam: Camera, prm: Params) -> Score:
    sc = Score()
    o = np.ascontiguousarray(obs, np.uint16)
    b = np.ascontiguousarray(box, np.int32)
    lib().qo_score_zbuf(ptr(zbuf, _i32), ptr(b, _i32), ptr(o, _u16), C.byref(cam),
                        C.byref(prm), C.byref(sc))
    return sc


def fitness_fp64(sc: Score, num_points: int) -> float:
    return lib().qo_fitness_fp64(C.byref(sc), C.c_uint32(num_points))


def init_particle(prm: Params, p: int, pos, vel, pb):
    lib().qo_init_particle(C.byref(prm), C.c_uint32(p), ptr(pos, _f), ptr(vel, _f), ptr(pb, _f))


def update_particle(prm: Params, p: int, it: int, pos, vel, pb, gb):
    g = np.ascontiguousarray(gb, np.float32)
    lib().qo_update_particle(C.byref(prm), C.c_uint32(p), C.c_uint32(it), ptr(pos, _f),
                             ptr(vel, _f), ptr(pb, _f), ptr(g, _f))


def solve(mesh: np.ndarray, num_faces: int, obs: np.ndarray, cam: Camera, prm: Params,
          trace: bool = False, threads: int = 1):
    P = prm.num_particles
    pos = np.zeros((NDIM, P), np.float32)
    vel = np.zeros((NDIM, P), np.float32)
    pb = np.zeros((NDIM, P), np.float32)
    pbf = np.zeros(P, np.float32)
    res = Result()
    tg = np.zeros((prm.iterations, 8), np.float32) if trace else None
    tf = np.zeros((prm.iterations, P), np.float32) if trace else None
    m = np.ascontiguousarray(mesh, np.float32)
    o = np.ascontiguousarray(obs, np.uint16)
    rc = lib().qo_solve_mt(ptr(m, _f), C.c_uint32(num_faces), ptr(o, _u16), C.byref(cam),
                           C.byref(prm), ptr(pos, _f), ptr(vel, _f), ptr(pb, _f), ptr(pbf, _f),
                           C.byref(res), ptr(tg, _f) if trace else None,
                           ptr(tf, _f) if trace else None, C.c_int(threads))
    if rc != 0:
        raise RuntimeError("qo_solve failed: %d" % rc)
    out = {"fit": res.gbest_fit, "pose": np.array(res.gbest[:], np.float32), "pos": pos,
           "vel": vel, "pbest": pb, "pbest_fit": pbf, "raster_writes": res.raster_writes}
    if trace:
        out["trace_gbest"] = tg
        out["trace_fit"] = tf
    return out


def sin(x):
    return lib().qo_sin(x)


def cos(x):
    return lib().qo_cos(x)


def acos(x):
    return lib().qo_acos(x)


def sinf(x):
    return lib().qo_sinf(x)


def cosf(x):
    return lib().qo_cosf(x)


def acosf(x):
    return lib().qo_acosf(x)


EDGE_DTYPE = np.dtype([("w", np.float32), ("a", np.int32), ("b", np.int32)])


def edges_array(a, b, w) -> np.ndarray:
    e = np.empty(len(w), EDGE_DTYPE)
    e["a"], e["b"], e["w"] = a, b, w
    return e


def segment_graph(n_vertices: int, edges: np.ndarray, k: float, min_size: float, merge: bool = True,
                  presorted: bool = False):
    """The oracle's segmentation core.  edges: EDGE_DTYPE array (a copy is
    sorted).  Returns (lists, num_sets, sorted_edges): lists is the
    collectSets listing, one int32 array per set in the order of its
    smallest pixel, each [first pixel, its parent, the rest of the set]."""
    e = np.ascontiguousarray(edges, EDGE_DTYPE).copy()
    offsets = np.zeros(n_vertices + 1, np.int32)
    points = np.zeros(2 * n_vertices, np.int32)
    ns = C.c_int32(0)
    n = lib().qo_segment_graph(n_vertices, len(e), e.ctypes.data, int(presorted), k, min_size, int(merge),
                               offsets.ctypes.data, points.ctypes.data, C.byref(ns))
    if n < 0:
        raise ValueError("qo_segment_graph refused its arguments")
    return [points[offsets[i]:offsets[i + 1]].copy() for i in range(n)], ns.value, e


def segment_graph_reference(H: int, W: int, edges: np.ndarray, k: float, min_size: float, merge: bool = True):
    """The same through the reference's own code (segpin); None where the
    reference sources are absent."""
    sp = segpin()
    if sp is None:
        return None
    n_vertices, m = H * W, len(edges)
    ea = np.ascontiguousarray(edges["a"], np.int32)
    eb = np.ascontiguousarray(edges["b"], np.int32)
    ew = np.ascontiguousarray(edges["w"], np.float32)
    sa, sb, sw = np.zeros(max(m, 1), np.int32), np.zeros(max(m, 1), np.int32), np.zeros(max(m, 1), np.float32)
    offsets = np.zeros(n_vertices + 1, np.int32)
    points = np.zeros(2 * n_vertices, np.int32)
    nl, ns = C.c_int(0), C.c_int(0)
    rc = sp.sp_segment(C.c_int(n_vertices), C.c_int(m), C.c_void_p(ea.ctypes.data), C.c_void_p(eb.ctypes.data),
                       C.c_void_p(ew.ctypes.data), C.c_float(k), C.c_float(min_size), C.c_int(int(merge)),
                       C.c_int(H), C.c_int(W), C.c_void_p(sa.ctypes.data), C.c_void_p(sb.ctypes.data),
                       C.c_void_p(sw.ctypes.data), C.c_void_p(offsets.ctypes.data), C.c_void_p(points.ctypes.data),
                       C.byref(nl), C.byref(ns))
    if rc != 0:
        raise ValueError("sp_segment refused its arguments")
    lists = [points[offsets[i]:offsets[i + 1]].copy() for i in range(nl.value)]
    return lists, ns.value, edges_array(sa[:m], sb[:m], sw[:m])


def grid_edges(H: int, W: int, weight) -> np.ndarray:
    """The reference's pixel graph (GraphCannySeg.cpp segment_image): for
    each pixel (x, y) in row-major order, the edges to (x+1, y), (x, y+1),
    (x+1, y+1) and (x+1, y-1) that lie inside the image, in that order;
    weight(a, b) gives each edge's weight from the two pixel indices."""
    a, b = [], []
    for y in range(H):
        for x in range(W):
            i = y * W + x
            if x < W - 1:
                a.append(i); b.append(i + 1)
            if y < H - 1:
                a.append(i); b.append(i + W)
            if x < W - 1 and y < H - 1:
                a.append(i); b.append(i + W + 1)
            if x < W - 1 and y > 0:
                a.append(i); b.append(i - W + 1)
    a, b = np.array(a, np.int32), np.array(b, np.int32)
    return edges_array(a, b, np.asarray(weight(a, b), np.float32))


class SegParams(C.Structure):
    _fields_ = [("sigma", C.c_float), ("k", C.c_float), ("min_size", C.c_float), ("kx", C.c_float),
                ("ky", C.c_float), ("ks", C.c_float), ("kdv", C.c_float), ("kdc", C.c_float)]


def seg_params(**kw) -> SegParams:
    """The reference main's segmentation constants (main.h:58-65,
    main.cu:1214-1217), with keyword overrides."""
    sp = SegParams()
    lib().qo_seg_default_params(C.byref(sp))
    for k, v in kw.items():
        setattr(sp, k, v)
    return sp


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def smooth(plane: np.ndarray, sigma: float) -> np.ndarray:
    src = _f32(plane)
    H, W = src.shape
    dst = np.empty_like(src)
    if lib().qo_smooth(src.ctypes.data_as(C.c_void_p), W, H, C.c_float(sigma), dst.ctypes.data_as(C.c_void_p)):
        raise ValueError("qo_smooth refused its arguments")
    return dst


def depth_norm(depth: np.ndarray) -> np.ndarray:
    d = np.ascontiguousarray(depth, np.uint16)
    H, W = d.shape
    out = np.empty((H, W), np.float32)
    lib().qo_depth_norm(d.ctypes.data_as(C.c_void_p), W, H, out.ctypes.data_as(C.c_void_p))
    return out


def graph_edges(sh, ss, sv, dnorm, sal, sp: SegParams) -> np.ndarray:
    """The pixel graph's edges (EDGE_DTYPE) over smoothed planes."""
    sh, ss, sv, dnorm, sal = (_f32(x) for x in (sh, ss, sv, dnorm, sal))
    H, W = sh.shape
    out = np.empty(4 * W * H, EDGE_DTYPE)
    n = lib().qo_graph_edges(*(x.ctypes.data_as(C.c_void_p) for x in (sh, ss, sv, dnorm, sal)), W, H,
                             C.byref(sp), out.ctypes.data_as(C.c_void_p))
    return out[:n].copy()


def segment_planes(h8, s8, v8, depth, sal, sp: SegParams):
    """End to end from 8-bit HSV planes, depth (mm) and saliency to the
    collectSets lists and the set count."""
    h8, s8, v8 = (np.ascontiguousarray(x, np.uint8) for x in (h8, s8, v8))
    d = np.ascontiguousarray(depth, np.uint16)
    sal = _f32(sal)
    H, W = h8.shape
    offsets = np.zeros(W * H + 1, np.int32)
    points = np.zeros(2 * W * H, np.int32)
    ns = C.c_int32(0)
    n = lib().qo_segment_planes(*(x.ctypes.data_as(C.c_void_p) for x in (h8, s8, v8, d, sal)), W, H,
                                C.byref(sp), offsets.ctypes.data_as(C.c_void_p), points.ctypes.data_as(C.c_void_p),
                                C.byref(ns))
    if n < 0:
        raise ValueError("qo_segment_planes refused its arguments")
    return [points[offsets[i]:offsets[i + 1]].copy() for i in range(n)], ns.value


def smooth_reference(plane: np.ndarray, sigma: float):
    """The reference's smooth() (segpin); None without the reference."""
    sp_ = segpin()
    if sp_ is None:
        return None
    src = _f32(plane)
    H, W = src.shape
    dst = np.empty_like(src)
    if sp_.sp_smooth(C.c_int(W), C.c_int(H), C.c_void_p(src.ctypes.data), C.c_float(sigma),
                     C.c_void_p(dst.ctypes.data)):
        raise ValueError("sp_smooth refused its arguments")
    return dst


def graph_reference(h8, s8, v8, depth, sal, sp: SegParams):
    """The reference's segment_image graph (segpin): (edges, smoothed planes
    [3, H, W], normalised depth); None without the reference."""
    lib_ = segpin()
    if lib_ is None:
        return None
    h8, s8, v8 = (np.ascontiguousarray(x, np.uint8) for x in (h8, s8, v8))
    d = np.ascontiguousarray(depth, np.uint16)
    sal = _f32(sal)
    H, W = h8.shape
    ea, eb = np.zeros(4 * W * H, np.int32), np.zeros(4 * W * H, np.int32)
    ew = np.zeros(4 * W * H, np.float32)
    sm = np.zeros((3, H, W), np.float32)
    dn = np.zeros((H, W), np.float32)
    m = lib_.sp_graph(C.c_int(W), C.c_int(H), *(C.c_void_p(x.ctypes.data) for x in (h8, s8, v8, d, sal)),
                      C.c_float(sp.sigma), C.c_float(sp.kdv), C.c_float(sp.kdc), C.c_float(sp.kx),
                      C.c_float(sp.ky), C.c_float(sp.ks), *(C.c_void_p(x.ctypes.data) for x in (ea, eb, ew, sm, dn)))
    if m < 0:
        raise ValueError("sp_graph refused its arguments")
    return edges_array(ea[:m], eb[:m], ew[:m]), sm, dn


# ---- the stages around the graph segmentation (qpso_seg_front.c) ----

class SegFrontParams(C.Structure):
    _fields_ = [("beta", C.c_float), ("gamma", C.c_float), ("inpaint_radius", C.c_int32),
                ("canny_low", C.c_float), ("canny_high", C.c_float), ("dth", C.c_int32),
                ("plus_d", C.c_int32), ("point_3d", C.c_int32), ("g_angle", C.c_float),
                ("l_angle", C.c_float), ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float),
                ("cy", C.c_float), ("far_obj_z", C.c_float), ("max_ecc", C.c_float),
                ("max_l1", C.c_float), ("max_l2", C.c_float)]


class SegCluster(C.Structure):
    _fields_ = [("label", C.c_int32), ("num_points", C.c_uint32), ("pixels", C.c_uint32),
                ("min_x", C.c_int32), ("max_x", C.c_int32), ("min_y", C.c_int32), ("max_y", C.c_int32),
                ("centroid_mm", C.c_float * 3), ("nan_ratio", C.c_float), ("dark_ratio", C.c_float),
                ("eig", C.c_double * 2), ("eccentricity", C.c_double), ("far", C.c_int32),
                ("kept", C.c_int32)]


def seg_front_params(**kw) -> SegFrontParams:
    """The reference main's constants for the stages around the graph
    segmentation (main.h:51-77, main.cu:1214-1221), with overrides."""
    fp = SegFrontParams()
    lib().qo_seg_front_default_params(C.byref(fp))
    for k, v in kw.items():
        setattr(fp, k, v)
    return fp


def _vp(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def bgr_to_hsv_gray(bgr: np.ndarray):
    """(h, s, v, gray) 8-bit planes of an H x W x 3 BGR image."""
    b = np.ascontiguousarray(bgr, np.uint8)
    H, W = b.shape[:2]
    out = [np.empty((H, W), np.uint8) for _ in range(4)]
    lib().qo_bgr_to_hsv_gray(_vp(b), W * H, *(_vp(x) for x in out))
    return tuple(out)


def depth_smooth(depth: np.ndarray, fp: SegFrontParams | None = None, with_maps: bool = False):
    fp = fp or seg_front_params()
    d = np.ascontiguousarray(depth, np.uint16)
    H, W = d.shape
    out = np.empty((H, W), np.uint16)
    cm = np.empty((H, W), np.uint8)
    rm = np.empty((H, W), np.float32)
    L = lib()
    L.qo_depth_smooth.restype = C.c_int32
    if L.qo_depth_smooth(_vp(d), W, H, C.c_float(fp.beta), C.c_float(fp.gamma), _vp(out), _vp(cm), _vp(rm)):
        raise ValueError("qo_depth_smooth refused its arguments")
    return (out, cm, rm) if with_maps else out


def telea(img: np.ndarray, mask: np.ndarray, radius: int = 20) -> np.ndarray:
    a = np.ascontiguousarray(img, np.uint8).copy()
    m = np.ascontiguousarray(mask, np.uint8)
    h, w = a.shape
    if lib().qo_telea(_vp(a), _vp(m), w, h, radius) < 0:
        raise ValueError("qo_telea refused its arguments")
    return a


def resize_bilinear_u8(src: np.ndarray, dw: int, dh: int) -> np.ndarray:
    s = np.ascontiguousarray(src, np.uint8)
    sh, sw = s.shape
    out = np.empty((dh, dw), np.uint8)
    lib().qo_resize_bilinear_u8(_vp(s), sw, sh, _vp(out), dw, dh)
    return out


def inpaint_depth(smoothed: np.ndarray, fp: SegFrontParams | None = None, with_small: bool = False):
    fp = fp or seg_front_params()
    sm = np.ascontiguousarray(smoothed, np.uint16)
    H, W = sm.shape
    out = np.empty((H, W), np.uint16)
    small = np.zeros((H // 5 + 1) * (W // 5 + 1), np.uint8)
    sw, sh = C.c_int32(0), C.c_int32(0)
    if lib().qo_inpaint_depth(_vp(sm), W, H, fp.inpaint_radius, _vp(out), _vp(small), C.byref(sw), C.byref(sh)):
        raise ValueError("qo_inpaint_depth refused its arguments")
    if with_small:
        return out, small[:sw.value * sh.value].reshape(sh.value, sw.value).copy()
    return out


def gauss_taps(ksize: int) -> np.ndarray:
    t = np.zeros(31, np.int32)
    n = lib().qo_gauss_taps(ksize, _vp(t))
    return t[:n].copy()


def blur_u8(src: np.ndarray, ksize: int) -> np.ndarray:
    s = np.ascontiguousarray(src, np.uint8)
    H, W = s.shape
    out = np.empty_like(s)
    lib().qo_blur_u8(_vp(s), W, H, ksize, _vp(out))
    return out


def orient_bin(x: int, y: int) -> int:
    return lib().qo_orient_bin(C.c_int32(x), C.c_int32(y))


def canny_saliency(gray: np.ndarray, inpainted: np.ndarray, fp: SegFrontParams | None = None,
                   with_edges: bool = False):
    fp = fp or seg_front_params()
    g = np.ascontiguousarray(gray, np.uint8)
    z = np.ascontiguousarray(inpainted, np.uint16)
    H, W = g.shape
    sal = np.empty((H, W), np.float32)
    edges = np.empty((H, W), np.uint8)
    if lib().qo_canny_saliency(_vp(g), _vp(z), W, H, C.byref(fp), _vp(sal), _vp(edges)):
        raise ValueError("qo_canny_saliency refused its arguments")
    return (sal, edges) if with_edges else sal


def seg_clusters(labels: np.ndarray, n_sets: int, inpainted: np.ndarray, v8: np.ndarray,
                 fp: SegFrontParams | None = None, keep_all: bool = False) -> list:
    fp = fp or seg_front_params()
    lab = np.ascontiguousarray(labels, np.int32)
    z = np.ascontiguousarray(inpainted, np.uint16)
    v = np.ascontiguousarray(v8, np.uint8)
    H, W = lab.shape
    out = (SegCluster * max(1, n_sets))()
    n = lib().qo_seg_clusters(_vp(lab), n_sets, _vp(z), _vp(v), W, H, C.byref(fp), out, int(keep_all))
    if n < 0:
        raise ValueError("qo_seg_clusters refused its arguments")
    return list(out[:n])


def labels_from_lists(lists, H: int, W: int) -> np.ndarray:
    """Label map (set k for the pixels of the k-th collectSets list, -1
    elsewhere) of segment_graph / segment_planes output."""
    lab = np.full(H * W, -1, np.int32)
    for k, pts in enumerate(lists):
        lab[pts] = k
    return lab.reshape(H, W)


def segment_rgbd(bgr: np.ndarray, depth: np.ndarray, sp: SegParams | None = None,
                 fp: SegFrontParams | None = None) -> dict:
    """GraphCannySeg<hsv>::run from a BGR image and a depth map (mm): the
    colour conversions, depth smoothing, inpainting, Canny saliency, the
    graph segmentation and the cluster filter, each stage's output kept."""
    sp = sp or seg_params()
    fp = fp or seg_front_params()
    h8, s8, v8, gray = bgr_to_hsv_gray(bgr)
    smoothed = depth_smooth(depth, fp)
    inp = inpaint_depth(smoothed, fp)
    sal = canny_saliency(gray, inp, fp)
    lists, n_sets = segment_planes(h8, s8, v8, inp, sal, sp)
    H, W = gray.shape
    labels = labels_from_lists(lists, H, W)
    clusters = seg_clusters(labels, len(lists), inp, v8, fp)
    return {"h": h8, "s": s8, "v": v8, "gray": gray, "smoothed": smoothed, "inpainted": inp,
            "saliency": sal, "labels": labels, "n_sets": len(lists), "clusters": clusters}


# ---- post-PSO refinement (the search of qpso_refine, replayed) ----

_MASK64 = (1 << 64) - 1


def _splitmix64(state: int):
    state = (state + 0x9E3779B97F4A7C15) & _MASK64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
    return state, z ^ (z >> 31)


def _uniform_pm1(state: int):
    state, z = _splitmix64(state)
    u = np.float32(z >> 40) * np.float32(5.9604644775390625e-8)
    return state, np.float32(u * np.float32(2.0) - np.float32(1.0))


def _rotate_small(q, hx, hy, hz):
    f = np.float32
    a0, a1, a2, a3 = f(1.0), f(hx), f(hy), f(hz)
    b0, b1, b2, b3 = (f(v) for v in q)
    r = [f(f(f(a0 * b0 - a1 * b1) - a2 * b2) - a3 * b3),
         f(f(f(a0 * b1 + a1 * b0) + a2 * b3) - a3 * b2),
         f(f(f(a0 * b2 - a1 * b3) + a2 * b0) + a3 * b1),
         f(f(f(a0 * b3 + a1 * b2) - a2 * b1) + a3 * b0)]
    n = np.sqrt(f(f(f(r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]) + r[3] * r[3]))
    sgn = f(-1.0) if r[0] < 0 else f(1.0)
    return [f(sgn * f(x / n)) for x in r]


def refine(mesh, num_faces, obs, cam: Camera, prm: Params, pose0, seed: int, stream: int, rounds: int = 32,
           candidates: int = 128, step_t: float = 0.03, step_rot: float = 0.5, mode: int = RASTER_EDGE):
    """The oracle's replay of qpso_refine: the same candidates, scored by
    the oracle's render and fitness in `mode`.  Returns (pose, fitness)."""
    f = np.float32

    def fitness(p):
        zbuf, box, _ = render(mesh, num_faces, np.array(p, np.float32), cam, mode=mode)
        return f(score(zbuf, box, obs, cam, prm).fit)

    pose = [f(v) for v in pose0[:3]] + _rotate_small(pose0[3:], 0.0, 0.0, 0.0)
    fit = fitness(pose)
    rng = (seed ^ (stream << 32) ^ 0x5245464E45) & _MASK64
    st, sr = f(step_t), f(step_rot)
    for _ in range(rounds):
        cands = []
        for i in range(candidates):
            c = list(pose)
            if i < 6:
                c[i // 2] = f(c[i // 2] + (-st if i & 1 else st))
            elif i < 12:
                h = [f(0.0)] * 3
                h[(i - 6) // 2] = f((-sr if i & 1 else sr) * f(0.5))
                c[3:] = _rotate_small(c[3:], *h)
            else:
                for k in range(3):
                    rng, u = _uniform_pm1(rng)
                    c[k] = f(c[k] + f(u * st))
                h = []
                for k in range(3):
                    rng, u = _uniform_pm1(rng)
                    h.append(f(f(u * sr) * f(0.5)))
                c[3:] = _rotate_small(c[3:], *h)
            cands.append(c)
        fits = [fitness(c) for c in cands]
        j = int(np.argmin(fits))  # first minimum
        if fits[j] < fit:
            fit, pose = fits[j], cands[j]
        else:
            st, sr = f(st * f(0.5)), f(sr * f(0.5))
    return np.array(pose, np.float32), fit
