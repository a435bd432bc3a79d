"""Generate the committed golden fixtures of tests/golden/.

ref_pin_cpu_render.npz -- the reference's host render of a pose (RenderCPU:
projectModelPointsToPixelsCPU + CPUfixedPointRender, main.h:1823-1991):
the single triangles above that write at most 2000 pixels, and whole
C1-mesh renders at four poses.

ref_pin.npz -- outputs of the reference's own main.h helpers, compiled for
the host CPU from the reference sources by oracle/build.py (ref_pin): the
fixed-point rasteriser renderFixedPointAABB with its AABB reduction, the
quaternion products, normalisation, hemisphere cast, vertex rotation, the
exponential-map step and the projection with the reference's compiled-in
intrinsics.  Needs the directory of the reference sources in the
environment variable QPSO_REFERENCE_SRC; run once, commit the .npz.

oracle_c1.npz -- the oracle's own C1 solve (per-iteration global best and
final state), frozen so that later changes to the oracle are caught.

ref_seg.npz -- the reference's segmentation core (disjoint-set forest,
segment_graph, small-component merge, collectSets; GraphCannySeg.cpp) run
by oracle/build.py's build_seg_pin on the pixel graphs of
tests/test_segmentation_core.py: per case the edges, and the collectSets
lists with the set count.  The tie case stores the edges in the order the
reference's std::sort left them (presorted).

ref_seg_graph.npz -- the reference's pixel graph (Gaussian smoothing, depth
normalisation, edge loop and edge weight of GraphCannySeg) run by the same
library on the frames of tests/test_segmentation_graph.py: per frame the
HSV planes, depth and saliency, and the edges with their weights.

Usage:  python tests/golden/make_golden.py            (every fixture)
        python tests/golden/make_golden.py --only seg (ref_seg.npz alone)
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "q-pso_gb300"))

from oracle import pyoracle as po  # noqa: E402
from tests.helpers import oracle_params  # noqa: E402

f_p = C.POINTER(C.c_float)
i_p = C.POINTER(C.c_int32)


def raster_cases(rng, n):
    """Single triangles whose bounding rectangles stay inside 640x480 (the
    reference does not clip): random sizes and windings plus hand-made edge
    cases (axis-aligned edges on pixel boundaries, slivers, sub-pixel,
    degenerate)."""
    tris = []
    special = [
        [[100.0, 100.0, 800.0], [110.0, 100.0, 800.0], [100.0, 110.0, 800.0]],
        [[100.0, 100.0, 800.0], [100.0, 110.0, 800.0], [110.0, 100.0, 800.0]],
        [[50.5, 60.5, 900.0], [70.5, 60.5, 950.0], [60.5, 80.5, 1000.0]],
        [[200.0, 200.0, 700.0], [200.3, 200.2, 700.0], [200.1, 200.4, 700.0]],
        [[300.0, 300.0, 700.0], [340.0, 300.0, 720.0], [380.0, 300.0, 740.0]],
        [[10.0, 10.0, 1200.0], [60.0, 11.0, 1100.0], [10.5, 12.0, 1000.0]],
        [[400.25, 100.75, 650.0], [430.125, 140.5, 690.0], [390.0, 160.0, 610.0]],
        [[620.0, 460.0, 500.0], [635.0, 470.0, 520.0], [625.0, 475.0, 540.0]],
        [[320.0, 240.0, 60010.0], [330.0, 240.0, 60020.0], [320.0, 250.0, 59990.0]],
        [[320.0, 100.0, -50.0], [330.0, 100.0, 20.0], [320.0, 110.0, 10.0]],
    ]
    for t in special:
        tris.append(np.array(t, np.float32))
    while len(tris) < n:
        size = rng.choice([0.4, 1.5, 4.0, 12.0, 40.0, 120.0])
        c = rng.uniform([30, 30], [610, 450])
        v = np.zeros((3, 3), np.float32)
        v[:, :2] = c + rng.normal(0, size, (3, 2))
        v[:, 2] = rng.uniform(300, 1500, 3)
        if v[:, 0].min() < 2 or v[:, 0].max() > 636 or v[:, 1].min() < 2 or v[:, 1].max() > 476:
            continue
        tris.append(v)
    return np.stack(tris)


def make_seg_golden():
    import test_segmentation_core as T

    cases = [T.CASES[i] for i in (0, 1, 2, 4, 7, 8)]
    runs = []
    for case in cases:
        H, W, _, k, min_size, merge, _ = case
        edges = T._case_edges(case)
        res = po.segment_graph_reference(H, W, edges, k, min_size, merge)
        if res is None:
            raise SystemExit("reference sources not found; set QPSO_REFERENCE_SRC")
        runs.append((H, W, k, min_size, merge, 0, edges, res))
    H, W = 24, 32
    tied = T.region_weights(H, W, 6, np.random.default_rng(11), tie_levels=16)
    res = po.segment_graph_reference(H, W, tied, 0.05, 20.0, True)
    runs.append((H, W, 0.05, 20.0, True, 1, res[2], res))

    e_off, l_off, bounds, pts = [0], [0], [], []
    ea, eb, ew = [], [], []
    for H, W, k, min_size, merge, presorted, edges, (lists, ns, _) in runs:
        ea.append(edges["a"]); eb.append(edges["b"]); ew.append(edges["w"])
        e_off.append(e_off[-1] + len(edges))
        base = sum(len(p) for p in pts)
        b = [base]
        for L in lists:
            pts.append(L.astype(np.int32))
            b.append(b[-1] + len(L))
        l_off.append(l_off[-1] + len(b))
        bounds.extend(b)
    # list_bounds holds, per case, n_lists + 1 absolute offsets into points;
    # case c's block is list_bounds[list_off[c] : list_off[c+1]]
    np.savez_compressed(
        os.path.join(HERE, "ref_seg.npz"),
        case_hw=np.array([(r[0], r[1]) for r in runs], np.int32),
        case_k_min=np.array([(r[2], r[3]) for r in runs], np.float32),
        case_merge=np.array([r[4] for r in runs], np.int32),
        presorted=np.array([r[5] for r in runs], np.int32),
        num_sets=np.array([r[7][1] for r in runs], np.int32),
        edge_a=np.concatenate(ea).astype(np.int32), edge_b=np.concatenate(eb).astype(np.int32),
        edge_w=np.concatenate(ew).astype(np.float32), edge_off=np.array(e_off, np.int64),
        list_off=np.array(l_off, np.int64), list_bounds=np.array(bounds, np.int64),
        points=np.concatenate(pts))

    import test_segmentation_graph as G

    sp = po.seg_params()
    hw, pix_off, planes = [], [0], {k: [] for k in ("h8", "s8", "v8", "depth", "sal")}
    e_off, ea, eb, ew = [0], [], [], []
    for fr in G.FRAMES:
        h8, s8, v8, d, sal = G.frame(*fr)
        edges, _, _ = po.graph_reference(h8, s8, v8, d, sal, sp)
        hw.append(h8.shape)
        pix_off.append(pix_off[-1] + h8.size)
        for k, v in zip(planes, (h8, s8, v8, d, sal)):
            planes[k].append(v.ravel())
        ea.append(edges["a"]); eb.append(edges["b"]); ew.append(edges["w"])
        e_off.append(e_off[-1] + len(edges))
    np.savez_compressed(
        os.path.join(HERE, "ref_seg_graph.npz"), hw=np.array(hw, np.int32),
        pix_off=np.array(pix_off, np.int64), **{k: np.concatenate(v) for k, v in planes.items()},
        edge_off=np.array(e_off, np.int64), edge_a=np.concatenate(ea).astype(np.int32),
        edge_b=np.concatenate(eb).astype(np.int32), edge_w=np.concatenate(ew).astype(np.float32))


def main():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    if sys.argv[1:] == ["--only", "seg"]:
        make_seg_golden()
        print("wrote ref_seg.npz, ref_seg_graph.npz")
        return
    make_seg_golden()
    pin = po.pin()
    if pin is None:
        raise SystemExit("reference sources not found; set QPSO_REFERENCE_SRC")
    rng = np.random.default_rng(20260101)

    # ---- raster ----
    tris = raster_cases(rng, 300)
    boxes, crops, offs = [], [], [0]
    for v in tris:
        buf = np.full(480 * 640, 60000, np.int32)
        box = np.zeros(4, np.int32)
        a, b, c = (np.ascontiguousarray(v[i]) for i in range(3))
        pin.pin_raster_face(a.ctypes.data_as(f_p), b.ctypes.data_as(f_p), c.ctypes.data_as(f_p),
                            buf.ctypes.data_as(i_p), box.ctypes.data_as(i_p))
        img = buf.reshape(480, 640)
        x0, x1, y0, y1 = box
        assert 0 <= x0 <= x1 <= 640 and 0 <= y0 <= y1 <= 480
        crop = img[y0:y1, x0:x1].copy()
        outside = img.copy()
        outside[y0:y1, x0:x1] = 60000
        assert (outside == 60000).all()
        boxes.append(box)
        crops.append(crop.ravel())
        offs.append(offs[-1] + crop.size)
    raster_depth = np.concatenate(crops).astype(np.int32)

    # ---- quaternion / rotation / projection ----
    n = 400
    S = rng.normal(size=(n, 7)).astype(np.float32)
    Q = rng.normal(size=(n, 7)).astype(np.float32)
    Vv = rng.normal(size=(n, 3)).astype(np.float32)
    Wv = rng.normal(0, 6, size=(n, 7)).astype(np.float32)
    rot = np.zeros((n, 3), np.float32)
    prod = np.zeros((n, 4), np.float32)
    prodc = np.zeros((n, 4), np.float32)
    norm = S.copy()
    cast = Q[:, 3:7].copy()
    kin = np.zeros((n, 7), np.float32)
    kin_init = np.zeros((n, 7), np.float32)
    proj = np.zeros((n, 3), np.float32)
    proj_pose = np.zeros((n, 7), np.float32)
    proj_pt = np.zeros((n, 3), np.float32)
    for i in range(n):
        s, q, v, w = (np.ascontiguousarray(x[i]) for x in (S, Q, Vv, Wv))
        pin.pin_rotate(s.ctypes.data_as(f_p), v.ctypes.data_as(f_p), rot[i].ctypes.data_as(f_p))
        pin.pin_quat_prod(s.ctypes.data_as(f_p), q.ctypes.data_as(f_p), prod[i].ctypes.data_as(f_p))
        pin.pin_quat_prod_conj(s.ctypes.data_as(f_p), q.ctypes.data_as(f_p),
                               prodc[i].ctypes.data_as(f_p))
        row = np.ascontiguousarray(norm[i])
        pin.pin_normalize(row.ctypes.data_as(f_p))
        norm[i] = row
        c4 = np.ascontiguousarray(cast[i])
        pin.pin_cast_top(c4.ctypes.data_as(f_p))
        cast[i] = c4
        sk = s.copy()
        sk[3:] /= np.linalg.norm(sk[3:])
        k = sk.copy()
        pin.pin_kinematics(k.ctypes.data_as(f_p), w.ctypes.data_as(f_p))
        kin[i] = k
        qi = np.array([0, 0, 0, 0.7071, 0.7071, 0, 0], np.float32)
        ki = np.zeros(7, np.float32)
        pin.pin_kinematics_init(qi.ctypes.data_as(f_p), ki.ctypes.data_as(f_p), w.ctypes.data_as(f_p))
        kin_init[i] = ki
        pose = np.array([rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2), rng.uniform(0.5, 1.2),
                         *sk[3:]], np.float32)
        pt = (rng.normal(size=3) * 0.05).astype(np.float32)
        o = np.zeros(3, np.float32)
        pin.pin_project(pose.ctypes.data_as(f_p), pt.ctypes.data_as(f_p), o.ctypes.data_as(f_p))
        proj[i], proj_pose[i], proj_pt[i] = o, pose, pt
    K = np.zeros(4, np.float64)
    pin.pin_intrinsics(K.ctypes.data_as(C.POINTER(C.c_double)))

    # ---- the host render of the best pose (RenderCPU, main.h:1823-2043):
    # its own rasteriser on the same triangles, then whole C1-mesh renders
    # through its own projection (every face inside the image) ----
    cpu_idx, cpu_val, cpu_off, cpu_sel = [], [], [0], []
    for i, v in enumerate(tris):
        buf = np.full(480 * 640, 60000.0, np.float32)
        a, b, c = (np.ascontiguousarray(v[i]) for i in range(3))
        pin.pin_cpu_raster_face(a.ctypes.data_as(f_p), b.ctypes.data_as(f_p), c.ctypes.data_as(f_p),
                                buf.ctypes.data_as(f_p))
        idx = np.nonzero(buf != 60000.0)[0]
        if idx.size > 2000:  # keeps the fixture small
            continue
        cpu_sel.append(i)
        cpu_idx.append(idx.astype(np.int32))
        cpu_val.append(buf[idx])
        cpu_off.append(cpu_off[-1] + idx.size)
    import scene
    w1 = scene.workload_c1()
    soa1, F1 = w1["meshes"][0]
    gt = np.asarray(w1["solves"][0]["gt_pose"], np.float32)
    r_poses = [gt]
    for _ in range(3):
        p = gt.copy()
        p[:3] += rng.uniform(-0.05, 0.05, 3).astype(np.float32)
        q = rng.normal(size=4)
        p[3:] = (q / np.linalg.norm(q) * np.sign(q[0])).astype(np.float32)
        r_poses.append(p)
    r_idx, r_val, r_off = [], [], [0]
    for pose in r_poses:
        buf = np.full(480 * 640, 60000.0, np.float32)
        for f in range(F1):
            uvz = []
            for j in range(3):
                vtx = np.array([soa1[f + j * F1], soa1[3 * F1 + f + j * F1], soa1[6 * F1 + f + j * F1]],
                               np.float32)
                o = np.zeros(3, np.float32)
                pin.pin_project_cpu(pose.ctypes.data_as(f_p), vtx.ctypes.data_as(f_p), o.ctypes.data_as(f_p))
                assert 2.0 < o[0] < 636.0 and 2.0 < o[1] < 476.0
                uvz.append(o)
            pin.pin_cpu_raster_face(uvz[0].ctypes.data_as(f_p), uvz[1].ctypes.data_as(f_p),
                                    uvz[2].ctypes.data_as(f_p), buf.ctypes.data_as(f_p))
        idx = np.nonzero(buf != 60000.0)[0]
        r_idx.append(idx.astype(np.int32))
        r_val.append(buf[idx])
        r_off.append(r_off[-1] + idx.size)
    np.savez_compressed(
        os.path.join(HERE, "ref_pin_cpu_render.npz"), tri_sel=np.array(cpu_sel, np.int32),
        tri_idx=np.concatenate(cpu_idx),
        tri_val=np.concatenate(cpu_val), tri_off=np.array(cpu_off, np.int64), poses=np.stack(r_poses),
        render_idx=np.concatenate(r_idx), render_val=np.concatenate(r_val),
        render_off=np.array(r_off, np.int64))

    np.savez_compressed(
        os.path.join(HERE, "ref_pin.npz"), tris=tris, boxes=np.array(boxes, np.int32),
        raster_depth=raster_depth, raster_off=np.array(offs, np.int64), S=S, Q=Q, V=Vv, W=Wv,
        rot=rot, prod=prod, prodc=prodc, norm=norm, cast=cast, kin=kin, kin_init=kin_init,
        proj=proj, proj_pose=proj_pose, proj_pt=proj_pt, intrinsics=K)

    # ---- oracle C1 solve, frozen ----
    w = scene.workload_c1()
    soa, F = w["meshes"][0]
    depth, labels, _ = w["frames"][0]
    s = w["solves"][0]
    prm = oracle_params(s)
    out = po.solve(soa, F, scene.masked_depth(depth, labels, 0), po.camera(), prm, trace=True)
    np.savez_compressed(os.path.join(HERE, "oracle_c1.npz"), trace_gbest=out["trace_gbest"],
                        pos=out["pos"], pbest_fit=out["pbest_fit"], fit=np.float32(out["fit"]),
                        pose=out["pose"])
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
