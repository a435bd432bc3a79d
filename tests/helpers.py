"""Shared test helpers: turn a workload solve entry into oracle parameters
and into a GPU solve descriptor with the same meaning."""
import numpy as np

import scene  # noqa: E402
from oracle import pyoracle as po


def oracle_params(s, **over):
    f = scene.solve_fields(s)
    f.update(over)
    prm = po.default_params()
    prm.t_lo[:] = f["t_lo"]
    prm.t_hi[:] = f["t_hi"]
    prm.cl_min_x, prm.cl_max_x = f["cl_min_x"], f["cl_max_x"]
    prm.cl_min_y, prm.cl_max_y = f["cl_min_y"], f["cl_max_y"]
    prm.num_points = f["num_points"]
    prm.num_particles = f["num_particles"]
    prm.iterations = f["iterations"]
    prm.seed = f["seed"]
    prm.stream = f["stream"]
    prm.raster_mode = f.get("raster_mode", 0)
    return prm


def gpu_desc(s, mesh_id, frame_id, **over):
    import qpso

    f = scene.solve_fields(s)
    f.update(over)
    return qpso.solve_desc(mesh_id=mesh_id, frame_id=frame_id, **f)


def gpu_camera():
    import qpso

    return qpso.Camera(*scene.camera_tuple())


def upload_workload(ctx, w):
    """Upload every mesh and frame of a workload; returns (mesh ids, frame ids)."""
    cam = gpu_camera()
    mids = [ctx.mesh_upload(soa, F) for soa, F in w["meshes"]]
    fids = [ctx.frame_upload(d, cam, labels=lab) for d, lab, _ in w["frames"]]
    return mids, fids


def oracle_obs(w, s):
    depth, labels, _ = w["frames"][s["frame"]]
    return scene.masked_depth(depth, labels, s["cluster"]["label"])


def rot_err_deg(q1, q2):
    d = abs(float(np.dot(np.asarray(q1, np.float64), np.asarray(q2, np.float64))))
    return 2.0 * np.degrees(np.arccos(min(1.0, d)))
