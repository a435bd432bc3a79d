"""Python view of the C ABI in include/qpso.h (ctypes over the in-tree
``_build/libqpso_gb300.so``).

This mirrors the reference's host-side workflow (main.cu:1198-1780): upload
the mesh (loadOBJ3 layout) and the observed depth, describe the cluster and
the PSO constants, solve, read back the global best.  Every call goes to the
sm_103a library; there is no CPU path, and loading fails loudly when the
library is missing or no GB300-class GPU is present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqpso_gb300.so")

OK, ERR_ARG, ERR_NOMEM, ERR_CUDA, ERR_TIMEOUT, ERR_BUSY, ERR_NOT_FOUND, ERR_INTERNAL = range(8)
STATUS_NAMES = ["OK", "ERR_ARG", "ERR_NOMEM", "ERR_CUDA", "ERR_TIMEOUT", "ERR_BUSY",
                "ERR_NOT_FOUND", "ERR_INTERNAL"]
ERR_BIT_BOUND, ERR_BIT_TIMEOUT, ERR_BIT_ARG = 1, 2, 4

# Functions declared in include/qpso.h (checked by the CPU test suite).
EXPORTS = [
    "qpso_version", "qpso_create", "qpso_destroy", "qpso_last_error", "qpso_mesh_upload",
    "qpso_mesh_release", "qpso_frame_upload", "qpso_frame_release", "qpso_solve_desc_init",
    "qpso_box_from_centroid", "qpso_set_launch_config", "qpso_get_launch_config", "qpso_solve",
    "qpso_solve_traced", "qpso_solve_batch", "qpso_score_poses", "qpso_render",
    "qpso_barrier_selftest", "qpso_frame_update", "qpso_host_alloc", "qpso_host_free",
    "qpso_get_stream", "qpso_set_profiling", "qpso_get_profile", "qpso_timer_record",
    "qpso_timer_elapsed", "qpso_scrub_l2", "qpso_score_poses_noalloc", "qpso_autotune",
    "qpso_server_start", "qpso_server_submit", "qpso_server_poll", "qpso_server_wait",
    "qpso_server_stats_get", "qpso_server_stop", "qpso_render_depth_f32", "qpso_frame_clusters",
    "qpso_obj_load", "qpso_image_u16_load", "qpso_seg_params_init", "qpso_segment_num_edges",
    "qpso_segment_edge_ends", "qpso_segment_gauss_mask", "qpso_segment_edges", "qpso_segment_planes",
    "qpso_seg_front_params_init", "qpso_segment_rgbd", "qpso_segment_clusters", "qpso_image_bgr8_load",
    "qpso_image_jpeg_write",
    "qpso_refine_params_init", "qpso_refine",
]


class Camera(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("width", C.c_int32), ("height", C.c_int32), ("projection", C.c_int32)]


# qpso_camera.projection: fp32 with the given intrinsics, or the reference's
# own double-precision projection with its compiled-in ACCV intrinsics
PROJ_FP32, PROJ_REF_ACCV = 0, 1


class SolveDesc(C.Structure):
    _fields_ = [("mesh_id", C.c_uint32), ("frame_id", C.c_uint32), ("cluster_label", C.c_int32),
                ("cl_min_x", C.c_int32), ("cl_max_x", C.c_int32), ("cl_min_y", C.c_int32),
                ("cl_max_y", C.c_int32), ("num_points", C.c_uint32), ("t_lo", C.c_float * 3),
                ("t_hi", C.c_float * 3), ("num_particles", C.c_uint32), ("iterations", C.c_uint32),
                ("c1", C.c_float), ("c2", C.c_float), ("w", C.c_double), ("vdot", C.c_float),
                ("ang_lo", C.c_float), ("ang_hi", C.c_float), ("qinit", C.c_float * 4),
                ("seed", C.c_uint64), ("stream", C.c_uint32), ("raster_mode", C.c_uint32)]


RASTER_REF, RASTER_EDGE = 0, 1


class Result(C.Structure):
    _fields_ = [("fit", C.c_float), ("pose", C.c_float * 7), ("flags", C.c_uint32),
                ("reserved", C.c_uint32), ("raster_writes", C.c_uint64),
                ("tile_passes", C.c_uint64)]


class LaunchConfig(C.Structure):
    _fields_ = [("threads", C.c_int32), ("tile_px", C.c_int32), ("ppb", C.c_int32)]


class Profile(C.Structure):
    _fields_ = [("step_launches", C.c_uint64), ("step_ms", C.c_double),
                ("batch_launches", C.c_uint64), ("batch_ms", C.c_double),
                ("prep_launches", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("max_slots", C.c_uint32), ("hbm_budget_bytes", C.c_uint64),
                ("iters_per_epoch", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("failed", C.c_uint64), ("pending", C.c_uint32), ("active", C.c_uint32),
                ("peak_active", C.c_uint32), ("bytes_in_use", C.c_uint64), ("peak_bytes", C.c_uint64),
                ("budget_bytes", C.c_uint64), ("epochs", C.c_uint64), ("launches", C.c_uint64)]


class Cluster(C.Structure):
    _fields_ = [("label", C.c_int32), ("num_points", C.c_uint32), ("min_x", C.c_int32),
                ("max_x", C.c_int32), ("min_y", C.c_int32), ("max_y", C.c_int32),
                ("depth_points", C.c_uint32), ("centroid_mm", C.c_float * 3)]


class SegParams(C.Structure):
    _fields_ = [("sigma", C.c_float), ("k", C.c_float), ("min_size", C.c_float), ("kx", C.c_float),
                ("ky", C.c_float), ("ks", C.c_float), ("kdv", C.c_float), ("kdc", C.c_float)]


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


class SegFrameOut(C.Structure):
    _fields_ = [("h", C.c_void_p), ("s", C.c_void_p), ("v", C.c_void_p), ("gray", C.c_void_p),
                ("smoothed", C.c_void_p), ("inpainted", C.c_void_p), ("saliency", C.c_void_p),
                ("edges", C.c_void_p)]


class RefineParams(C.Structure):
    _fields_ = [("rounds", C.c_uint32), ("candidates", C.c_uint32), ("step_t", C.c_float),
                ("step_rot", C.c_float), ("raster_mode", C.c_uint32)]


class QpsoError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES[status] if 0 <= status < 8 else status, msg))
        self.status = status


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("qpso CUDA library not built: %s (run __graft_entry__.build())" % path)
    L = C.CDLL(path)
    vp = C.c_void_p
    L.qpso_version.argtypes = []
    L.qpso_version.restype = C.c_char_p
    L.qpso_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.qpso_destroy.argtypes = [vp]
    L.qpso_destroy.restype = None
    L.qpso_last_error.argtypes = [vp]
    L.qpso_last_error.restype = C.c_char_p
    L.qpso_mesh_upload.argtypes = [vp, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)]
    L.qpso_mesh_release.argtypes = [vp, C.c_uint32]
    L.qpso_frame_upload.argtypes = [vp, C.c_void_p, C.c_void_p, C.POINTER(Camera),
                                    C.POINTER(C.c_uint32)]
    L.qpso_frame_release.argtypes = [vp, C.c_uint32]
    L.qpso_solve_desc_init.argtypes = [C.POINTER(SolveDesc)]
    L.qpso_solve_desc_init.restype = None
    L.qpso_box_from_centroid.argtypes = [C.POINTER(C.c_float), C.c_float, C.c_float,
                                         C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.qpso_box_from_centroid.restype = None
    L.qpso_set_launch_config.argtypes = [vp, C.POINTER(LaunchConfig), C.POINTER(LaunchConfig)]
    L.qpso_get_launch_config.argtypes = [vp, C.POINTER(LaunchConfig), C.POINTER(LaunchConfig)]
    L.qpso_solve.argtypes = [vp, C.POINTER(SolveDesc), C.POINTER(Result)]
    L.qpso_solve_traced.argtypes = [vp, C.POINTER(SolveDesc), C.POINTER(Result), C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.qpso_solve_batch.argtypes = [vp, C.POINTER(SolveDesc), C.c_uint32, C.POINTER(Result)]
    L.qpso_score_poses.argtypes = [vp, C.POINTER(SolveDesc), C.c_void_p, C.c_uint32, C.c_void_p]
    L.qpso_render.argtypes = [vp, C.c_uint32, C.POINTER(Camera), C.c_void_p, C.c_int32,
                              C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    L.qpso_render_depth_f32.argtypes = [vp, C.c_uint32, C.POINTER(Camera), C.c_void_p, C.c_void_p]
    L.qpso_frame_clusters.argtypes = [vp, C.c_uint32, C.POINTER(Cluster), C.c_uint32, C.POINTER(C.c_uint32)]
    L.qpso_obj_load.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)]
    L.qpso_image_u16_load.argtypes = [C.c_char_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]
    L.qpso_image_bgr8_load.argtypes = [C.c_char_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_uint32)]
    L.qpso_image_jpeg_write.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32]
    L.qpso_barrier_selftest.argtypes = [vp, C.c_uint64, C.POINTER(C.c_uint32)]
    L.qpso_frame_update.argtypes = [vp, C.c_uint32, C.c_void_p, C.c_void_p]
    L.qpso_host_alloc.argtypes = [C.c_uint64]
    L.qpso_host_alloc.restype = C.c_void_p
    L.qpso_host_free.argtypes = [C.c_void_p]
    L.qpso_host_free.restype = None
    L.qpso_get_stream.argtypes = [vp]
    L.qpso_get_stream.restype = C.c_void_p
    L.qpso_set_profiling.argtypes = [vp, C.c_int]
    L.qpso_get_profile.argtypes = [vp, C.POINTER(Profile), C.c_int]
    L.qpso_timer_record.argtypes = [vp, C.c_uint32]
    L.qpso_timer_elapsed.argtypes = [vp, C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]
    L.qpso_scrub_l2.argtypes = [vp, C.c_uint64]
    L.qpso_server_start.argtypes = [vp, C.POINTER(ServerConfig), C.POINTER(vp)]
    L.qpso_server_submit.argtypes = [vp, C.POINTER(SolveDesc), C.POINTER(C.c_uint64)]
    L.qpso_server_poll.argtypes = [vp, C.c_uint64, C.POINTER(C.c_int), C.POINTER(Result),
                                   C.POINTER(C.c_double)]
    L.qpso_server_wait.argtypes = [vp, C.c_uint64, C.c_uint64, C.POINTER(Result),
                                   C.POINTER(C.c_double)]
    L.qpso_server_stats_get.argtypes = [vp, C.POINTER(ServerStats)]
    L.qpso_server_stop.argtypes = [vp]
    L.qpso_autotune.argtypes = [vp, C.POINTER(SolveDesc), C.c_uint32, C.c_int, C.c_uint32,
                                C.POINTER(LaunchConfig), C.POINTER(C.c_float)]
    L.qpso_score_poses_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                           C.POINTER(Camera), C.POINTER(SolveDesc), C.c_void_p,
                                           C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.qpso_seg_params_init.argtypes = [C.POINTER(SegParams)]
    L.qpso_seg_params_init.restype = None
    L.qpso_segment_num_edges.argtypes = [C.c_uint32, C.c_uint32]
    L.qpso_segment_num_edges.restype = C.c_uint64
    L.qpso_segment_edge_ends.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    L.qpso_segment_gauss_mask.argtypes = [C.c_float, C.c_void_p, C.c_int32]
    L.qpso_segment_edges.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.POINTER(SegParams), C.c_void_p,
                                     C.POINTER(C.c_uint32)]
    L.qpso_segment_planes.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_uint32, C.c_uint32, C.POINTER(SegParams), C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_uint32)]
    L.qpso_segment_rgbd.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(SegParams),
                                    C.POINTER(SegFrontParams), C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p,
                                    C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(SegFrameOut)]
    L.qpso_seg_front_params_init.argtypes = [C.POINTER(SegFrontParams)]
    L.qpso_refine_params_init.argtypes = [C.POINTER(RefineParams)]
    L.qpso_refine.argtypes = [vp, C.POINTER(SolveDesc), C.POINTER(RefineParams), C.c_void_p, C.c_void_p,
                              C.POINTER(C.c_float)]
    L.qpso_segment_clusters.argtypes = [vp, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                        C.c_uint32, C.POINTER(SegFrontParams), C.c_int, C.c_void_p, C.c_uint32,
                                        C.POINTER(C.c_uint32)]
    for fn in EXPORTS:
        if fn not in ("qpso_version", "qpso_destroy", "qpso_last_error", "qpso_solve_desc_init",
                      "qpso_box_from_centroid", "qpso_host_alloc", "qpso_host_free",
                      "qpso_get_stream", "qpso_seg_params_init", "qpso_segment_num_edges",
                      "qpso_seg_front_params_init", "qpso_refine_params_init"):
            getattr(L, fn).restype = C.c_int32
    _lib = L
    return L


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def solve_desc(**kw) -> SolveDesc:
    """A descriptor with the reference's defaults, fields overridden by kw."""
    d = SolveDesc()
    load_library().qpso_solve_desc_init(C.byref(d))
    for k, v in kw.items():
        if k in ("t_lo", "t_hi"):
            setattr(d, k, (C.c_float * 3)(*v))
        elif k == "qinit":
            setattr(d, k, (C.c_float * 4)(*v))
        else:
            setattr(d, k, v)
    return d


def box_from_centroid(centroid_mm, bound=0.3, bound_z=0.3):
    c = (C.c_float * 3)(*centroid_mm)
    lo = (C.c_float * 3)()
    hi = (C.c_float * 3)()
    load_library().qpso_box_from_centroid(c, bound, bound_z, lo, hi)
    return list(lo), list(hi)


class Context:
    """One GPU context (qpso_create / qpso_destroy)."""

    def __init__(self, device: int = 0):
        self.L = load_library()
        self.device = device
        self.h = C.c_void_p()
        st = self.L.qpso_create(device, C.byref(self.h))
        if st != OK:
            raise QpsoError(st, "qpso_create(device=%d) failed (no sm_100+ GPU?)" % device)

    def close(self):
        if self.h:
            self.L.qpso_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != OK:
            raise QpsoError(st, self.L.qpso_last_error(self.h).decode())

    def mesh_upload(self, soa: np.ndarray, num_faces: int) -> int:
        a = _f32(soa)
        if a.size != 9 * num_faces:
            raise ValueError("mesh must hold 9*num_faces floats")
        mid = C.c_uint32()
        self._check(self.L.qpso_mesh_upload(self.h, a.ctypes.data, num_faces, C.byref(mid)))
        return mid.value

    def mesh_release(self, mid: int):
        self._check(self.L.qpso_mesh_release(self.h, mid))

    def frame_upload(self, depth_mm: np.ndarray, cam: Camera, labels: np.ndarray | None = None) -> int:
        d = np.ascontiguousarray(depth_mm, dtype=np.uint16)
        lab = None if labels is None else np.ascontiguousarray(labels, dtype=np.int32)
        if d.shape != (cam.height, cam.width):
            raise ValueError("depth shape must be (height, width)")
        fid = C.c_uint32()
        self._check(self.L.qpso_frame_upload(self.h, d.ctypes.data,
                                             None if lab is None else lab.ctypes.data,
                                             C.byref(cam), C.byref(fid)))
        return fid.value

    def frame_release(self, fid: int):
        self._check(self.L.qpso_frame_release(self.h, fid))

    def set_launch_config(self, plain=None, batch=None):
        p = None if plain is None else C.byref(LaunchConfig(*plain))
        b = None if batch is None else C.byref(LaunchConfig(*batch))
        self._check(self.L.qpso_set_launch_config(self.h, p, b))

    def get_launch_config(self):
        p, b = LaunchConfig(), LaunchConfig()
        self._check(self.L.qpso_get_launch_config(self.h, C.byref(p), C.byref(b)))
        return (p.threads, p.tile_px, p.ppb), (b.threads, b.tile_px, b.ppb)

    def autotune(self, descs, batched: bool, tune_iters: int = 3):
        """Pick the fastest launch shape for these solves (installed in the
        context); returns ((threads, tile_px, ppb), ms of the tuning run)."""
        n = len(descs)
        arr = (SolveDesc * n)(*descs)
        best = LaunchConfig()
        ms = C.c_float()
        self._check(self.L.qpso_autotune(self.h, arr, n, 1 if batched else 0, tune_iters,
                                         C.byref(best), C.byref(ms)))
        return (best.threads, best.tile_px, best.ppb), ms.value

    def solve(self, desc: SolveDesc) -> Result:
        r = Result()
        self._check(self.L.qpso_solve(self.h, C.byref(desc), C.byref(r)))
        return r

    def solve_traced(self, desc: SolveDesc):
        P, it = desc.num_particles, desc.iterations
        trace = np.zeros((it, 8), np.float32)
        pos = np.zeros((7, P), np.float32)
        vel = np.zeros((7, P), np.float32)
        pb = np.zeros((7, P), np.float32)
        pbf = np.zeros(P, np.float32)
        r = Result()
        self._check(self.L.qpso_solve_traced(self.h, C.byref(desc), C.byref(r), trace.ctypes.data,
                                             pos.ctypes.data, vel.ctypes.data, pb.ctypes.data,
                                             pbf.ctypes.data))
        return r, {"trace_gbest": trace, "pos": pos, "vel": vel, "pbest": pb, "pbest_fit": pbf}

    def solve_batch(self, descs) -> list:
        n = len(descs)
        arr = (SolveDesc * n)(*descs)
        res = (Result * n)()
        self._check(self.L.qpso_solve_batch(self.h, arr, n, res))
        return list(res)

    def score_poses(self, desc: SolveDesc, poses: np.ndarray) -> np.ndarray:
        p = _f32(poses).reshape(-1, 7)
        out = np.zeros(p.shape[0], np.float32)
        self._check(self.L.qpso_score_poses(self.h, C.byref(desc), p.ctypes.data, p.shape[0],
                                            out.ctypes.data))
        return out

    def refine(self, desc: SolveDesc, pose, params: "RefineParams | None" = None):
        """Local refinement of a pose (qpso_refine): (pose float32[7], fitness)."""
        prm = params if params is not None else refine_params()
        p = _f32(pose)
        out = np.zeros(7, np.float32)
        fit = C.c_float()
        self._check(self.L.qpso_refine(self.h, C.byref(desc), C.byref(prm), p.ctypes.data, out.ctypes.data,
                                       C.byref(fit)))
        return out, fit.value

    def render(self, mesh_id: int, cam: Camera, pose, x0: int, y0: int, w: int, h: int):
        out = np.zeros((h, w), np.int32)
        box = np.zeros(4, np.int32)
        p = _f32(pose)
        self._check(self.L.qpso_render(self.h, mesh_id, C.byref(cam), p.ctypes.data, x0, y0, w, h,
                                       out.ctypes.data, box.ctypes.data))
        return out, box

    def frame_clusters(self, fid: int) -> list:
        """Cluster records of the frame's label map (SegResults fields)."""
        n = C.c_uint32()
        self._check(self.L.qpso_frame_clusters(self.h, fid, None, 0, C.byref(n)))
        arr = (Cluster * max(1, n.value))()
        self._check(self.L.qpso_frame_clusters(self.h, fid, arr, n.value, C.byref(n)))
        return [{"label": c.label, "num_points": c.num_points,
                 "aabb": (c.min_x, c.max_x, c.min_y, c.max_y), "depth_points": c.depth_points,
                 "centroid_mm": list(c.centroid_mm)} for c in arr[:n.value]]

    def segment_rgbd(self, bgr, depth_mm, params: "SegParams | None" = None,
                     front: "SegFrontParams | None" = None, planes: bool = False):
        """GraphCannySeg<hsv>::run on the GPU (qpso_segment_rgbd) from a
        BGR image (uint8 (height, width, 3)) and raw depth (uint16 mm).
        Returns {"labels", "n_sets", "clusters"} (the kept sets in the
        reference's order) and, with planes=True, the intermediate planes
        h, s, v, gray, smoothed, inpainted, saliency, edges."""
        b = np.ascontiguousarray(bgr, np.uint8)
        d = np.ascontiguousarray(depth_mm, np.uint16)
        H, W = d.shape
        if b.shape != (H, W, 3):
            raise ValueError("bgr must be (height, width, 3) like the depth")
        prm = params if params is not None else seg_params()
        fp = front if front is not None else seg_front_params()
        labels = np.empty((H, W), np.int32)
        ns, nc = C.c_uint32(), C.c_uint32()
        out = {}
        po = None
        if planes:
            out = {k: np.empty((H, W), t) for k, t in (("h", np.uint8), ("s", np.uint8), ("v", np.uint8),
                                                        ("gray", np.uint8), ("smoothed", np.uint16),
                                                        ("inpainted", np.uint16), ("saliency", np.float32),
                                                        ("edges", np.uint8))}
            po = SegFrameOut(*(out[k].ctypes.data for k, _ in SegFrameOut._fields_))
        cap = W * H // 16 + 16
        arr = (SegCluster * cap)()
        self._check(self.L.qpso_segment_rgbd(self.h, b.ctypes.data, d.ctypes.data, W, H, C.byref(prm),
                                             C.byref(fp), labels.ctypes.data, C.byref(ns), arr, cap,
                                             C.byref(nc), C.byref(po) if po is not None else None))
        out.update(labels=labels, n_sets=ns.value, clusters=list(arr[:min(nc.value, cap)]))
        return out

    def segment_clusters(self, labels, n_sets: int, inpainted_mm, v_plane,
                         front: "SegFrontParams | None" = None, keep_all: bool = False) -> list:
        """PostSegmFilter over a label map (qpso_segment_clusters)."""
        lab = np.ascontiguousarray(labels, np.int32)
        z = np.ascontiguousarray(inpainted_mm, np.uint16)
        v = np.ascontiguousarray(v_plane, np.uint8)
        H, W = lab.shape
        fp = front if front is not None else seg_front_params()
        arr = (SegCluster * max(1, n_sets))()
        n = C.c_uint32()
        self._check(self.L.qpso_segment_clusters(self.h, lab.ctypes.data, n_sets, z.ctypes.data, v.ctypes.data,
                                                 W, H, C.byref(fp), int(keep_all), arr, max(1, n_sets),
                                                 C.byref(n)))
        return list(arr[:n.value])

    def segment_planes(self, h8, s8, v8, depth_mm, saliency, params: "SegParams | None" = None,
                       weights: bool = False):
        """The segmentation's graph stage on the GPU (qpso_segment_planes):
        HSV planes (uint8, H in 0..180), depth (uint16 mm) and saliency
        (float32), all (height, width).  Returns (labels int32 (height,
        width), n_clusters) and, with weights=True, the edge weights in
        the reference's edge order."""
        h8, s8, v8 = (np.ascontiguousarray(x, np.uint8) for x in (h8, s8, v8))
        d = np.ascontiguousarray(depth_mm, np.uint16)
        sal = _f32(saliency)
        H, W = h8.shape
        if not all(x.shape == (H, W) for x in (s8, v8, d, sal)):
            raise ValueError("planes differ in shape")
        prm = params if params is not None else seg_params()
        labels = np.empty((H, W), np.int32)
        w = np.empty(max(1, segment_num_edges(W, H)), np.float32) if weights else None
        n = C.c_uint32()
        self._check(self.L.qpso_segment_planes(self.h, h8.ctypes.data, s8.ctypes.data, v8.ctypes.data,
                                               d.ctypes.data, sal.ctypes.data, W, H, C.byref(prm),
                                               labels.ctypes.data, None if w is None else w.ctypes.data,
                                               C.byref(n)))
        if weights:
            return labels, n.value, w[:segment_num_edges(W, H)]
        return labels, n.value

    def render_depth_f32(self, mesh_id: int, cam: Camera, pose) -> np.ndarray:
        """The reference's best-pose depth image (RenderCPU arithmetic)."""
        out = np.empty((cam.height, cam.width), np.float32)
        p = _f32(pose)
        self._check(self.L.qpso_render_depth_f32(self.h, mesh_id, C.byref(cam), p.ctypes.data,
                                                 out.ctypes.data))
        return out

    def frame_update(self, fid: int, depth_mm: np.ndarray, labels: np.ndarray | None = None):
        self._check(self.L.qpso_frame_update(self.h, fid, depth_mm.ctypes.data,
                                             None if labels is None else labels.ctypes.data))

    def stream_handle(self) -> int:
        return self.L.qpso_get_stream(self.h) or 0

    def set_profiling(self, on: bool):
        self._check(self.L.qpso_set_profiling(self.h, 1 if on else 0))

    def profile(self, reset: bool = False) -> dict:
        p = Profile()
        self._check(self.L.qpso_get_profile(self.h, C.byref(p), 1 if reset else 0))
        return {k: getattr(p, k) for k, _ in Profile._fields_}

    def timer_record(self, slot: int):
        self._check(self.L.qpso_timer_record(self.h, slot))

    def timer_elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        self._check(self.L.qpso_timer_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value

    def scrub_l2(self, nbytes: int = 256 << 20):
        self._check(self.L.qpso_scrub_l2(self.h, nbytes))

    def barrier_selftest(self, timeout_ns: int):
        bits = C.c_uint32()
        st = self.L.qpso_barrier_selftest(self.h, timeout_ns, C.byref(bits))
        return st, bits.value


class Server:
    """Continuous-batching request loop on a context (qpso_server_*)."""

    def __init__(self, ctx: Context, max_slots: int = 64, hbm_budget_bytes: int = 0,
                 iters_per_epoch: int = 4):
        self.L = ctx.L
        self.h = C.c_void_p()
        cfg = ServerConfig(max_slots, hbm_budget_bytes, iters_per_epoch)
        st = self.L.qpso_server_start(ctx.h, C.byref(cfg), C.byref(self.h))
        if st != OK:
            raise QpsoError(st, ctx.L.qpso_last_error(ctx.h).decode())

    def submit(self, desc: SolveDesc) -> int:
        rid = C.c_uint64()
        st = self.L.qpso_server_submit(self.h, C.byref(desc), C.byref(rid))
        if st != OK:
            raise QpsoError(st, "submit refused")
        return rid.value

    def poll(self, rid: int):
        done = C.c_int()
        r = Result()
        lat = C.c_double()
        st = self.L.qpso_server_poll(self.h, rid, C.byref(done), C.byref(r), C.byref(lat))
        if st != OK:
            raise QpsoError(st, "request %d failed" % rid)
        return (r, lat.value) if done.value else None

    def wait(self, rid: int, timeout_ms: int = 600000):
        r = Result()
        lat = C.c_double()
        st = self.L.qpso_server_wait(self.h, rid, timeout_ms, C.byref(r), C.byref(lat))
        if st != OK:
            raise QpsoError(st, "request %d" % rid)
        return r, lat.value

    def stats(self) -> dict:
        s = ServerStats()
        self.L.qpso_server_stats_get(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def stop(self):
        if self.h:
            self.L.qpso_server_stop(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop()


class PinnedArray:
    """numpy view of a page-locked host buffer (qpso_host_alloc)."""

    def __init__(self, shape, dtype):
        L = load_library()
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = L.qpso_host_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError("qpso_host_alloc(%d) failed" % self.nbytes)
        buf = (C.c_char * self.nbytes).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def close(self):
        if self.ptr:
            self.array = None
            load_library().qpso_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _status(st: int, what: str):
    if st != OK:
        raise QpsoError(st, what)


def obj_load(path: str):
    """OBJ text -> (loadOBJ3 SoA float32 array of 9*F, F).  Host only."""
    L = load_library()
    F = C.c_uint32()
    _status(L.qpso_obj_load(path.encode(), None, 0, C.byref(F)), path)
    soa = np.empty(9 * F.value, np.float32)
    _status(L.qpso_obj_load(path.encode(), soa.ctypes.data, F.value, C.byref(F)), path)
    return soa, F.value


def image_u16_load(path: str) -> np.ndarray:
    """ACCV binary depth or greyscale PNG -> uint16 (height, width).  Host only."""
    L = load_library()
    w, h = C.c_uint32(), C.c_uint32()
    _status(L.qpso_image_u16_load(path.encode(), None, 0, C.byref(w), C.byref(h)), path)
    out = np.empty((h.value, w.value), np.uint16)
    _status(L.qpso_image_u16_load(path.encode(), out.ctypes.data, out.size, C.byref(w), C.byref(h)), path)
    return out


def image_bgr8_load(path: str) -> np.ndarray:
    """Colour PNG or binary PPM -> uint8 (height, width, 3), B G R.  Host only."""
    L = load_library()
    w, h = C.c_uint32(), C.c_uint32()
    _status(L.qpso_image_bgr8_load(path.encode(), None, 0, C.byref(w), C.byref(h)), path)
    out = np.empty((h.value, w.value, 3), np.uint8)
    _status(L.qpso_image_bgr8_load(path.encode(), out.ctypes.data, h.value * w.value, C.byref(w), C.byref(h)),
            path)
    return out


def image_jpeg_write(path: str, bgr, quality: int = 95) -> None:
    """uint8 (height, width, 3) B G R -> baseline JPEG file.  Host only."""
    L = load_library()
    a = np.ascontiguousarray(bgr, np.uint8)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError("expected (height, width, 3) uint8")
    _status(L.qpso_image_jpeg_write(path.encode(), a.ctypes.data, a.shape[1], a.shape[0], int(quality)), path)


def result_dict(r: Result) -> dict:
    return {"fit": r.fit, "pose": np.array(r.pose[:], np.float32), "flags": r.flags,
            "raster_writes": r.raster_writes, "tile_passes": r.tile_passes}


def seg_params(**kw) -> SegParams:
    """The reference main's segmentation constants, fields overridden by kw."""
    p = SegParams()
    load_library().qpso_seg_params_init(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def refine_params(**kw) -> RefineParams:
    """The refinement's defaults (qpso_refine_params_init), overridden by kw."""
    p = RefineParams()
    load_library().qpso_refine_params_init(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def seg_front_params(**kw) -> SegFrontParams:
    """The reference main's constants for the stages around the graph stage
    (main.h:51-77), fields overridden by kw."""
    p = SegFrontParams()
    load_library().qpso_seg_front_params_init(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def segment_num_edges(width: int, height: int) -> int:
    return int(load_library().qpso_segment_num_edges(width, height))


def segment_edge_ends(width: int, height: int):
    """(a, b): every edge's ends in the reference's edge order.  Host only."""
    n = segment_num_edges(width, height)
    a, b = np.empty(max(1, n), np.int32), np.empty(max(1, n), np.int32)
    _status(load_library().qpso_segment_edge_ends(width, height, a.ctypes.data, b.ctypes.data),
            "qpso_segment_edge_ends")
    return a[:n], b[:n]


def segment_gauss_mask(sigma: float) -> np.ndarray:
    m = np.empty(64, np.float32)
    n = load_library().qpso_segment_gauss_mask(C.c_float(sigma), m.ctypes.data, 64)
    if n < 0:
        raise QpsoError(ERR_ARG, "qpso_segment_gauss_mask")
    return m[:n].copy()


def segment_edges(width: int, height: int, weights, params: "SegParams | None" = None):
    """The merge passes over given edge weights.  Host only.  Returns
    (labels int32 (height, width), n_clusters)."""
    w = _f32(weights)
    if w.size != segment_num_edges(width, height):
        raise ValueError("one weight per edge")
    prm = params if params is not None else seg_params()
    labels = np.empty((height, width), np.int32)
    n = C.c_uint32()
    wbuf = w if w.size else np.zeros(1, np.float32)
    _status(load_library().qpso_segment_edges(width, height, wbuf.ctypes.data, C.byref(prm), labels.ctypes.data,
                                              C.byref(n)), "qpso_segment_edges")
    return labels, n.value
