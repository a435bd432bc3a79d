"""The command-line drop-in end to end on the GPU: OBJ model, ACCV binary
and PNG depth, a PNG label map in place of the segmentation, and the two
result files the reference writes (main.cu:1752-1762):
results/<rgb>-<N>-bestpose.csv equals the library's solve of the same
cluster printed as the reference prints it (with the reference's cluster
size, pixels + 1: its collectSets lists repeat one pixel), and
results/<rgb>-<N>-best.csv
equals the oracle's restatement of the reference's host render of that pose.
The cluster records equal the label map's own pixel statistics."""
import os
import subprocess

import numpy as np
import pytest

import qpso
import scene
from oracle import pyoracle as po
from tests.test_ingest import CLI, _jpeg_decode, write_accv, write_obj, write_png_gray

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    w = scene.workload_c2(frames=1, particles=32, iterations=6)
    depth, labels, _ = w["frames"][0]
    s = w["solves"][3]
    soa, F = w["meshes"][s["mesh"]]
    obj = str(d / "model.obj")
    write_obj(obj, soa, F)
    write_accv(str(d / "depth.bin"), depth)
    write_png_gray(str(d / "depth.png"), depth, 16, 6, (0, 1, 2, 3, 4))
    write_png_gray(str(d / "labels.png"), (labels + 1).astype(np.uint16), 16, 9, (4,))
    return d, w, s, obj


def run_cli(d, obj, depth_name, k, extra=(), camera=("--camera", "525,525,319.5,239.5")):
    cmd = [CLI, obj, "img_0042.png", str(d / depth_name), str(k), "--labels", str(d / "labels.png"),
           *camera, "--particles", "32", "--iterations", "6", "--seed", "7",
           "--results", str(d / "results"), *extra]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=300)


def test_cluster_records_match_label_map(gpu_ctx, files):
    d, w, s, _ = files
    depth, labels, _ = w["frames"][0]
    cam = qpso.Camera(*scene.camera_tuple())
    fid = gpu_ctx.frame_upload(depth, cam, labels=labels)
    got = gpu_ctx.frame_clusters(fid)
    want = [scene.cluster_info(depth, labels, k) for k in range(int(labels.max()) + 1)]
    want = [x for x in want if x is not None]
    assert [g["label"] for g in got] == [x["label"] for x in want]
    for g, x in zip(got, want):
        assert g["num_points"] == x["num_points"] and tuple(g["aabb"]) == tuple(x["aabb"])
        np.testing.assert_allclose(g["centroid_mm"], x["centroid_mm"], rtol=1e-5, atol=1e-3)
    gpu_ctx.frame_release(fid)


@pytest.mark.parametrize("depth_name", ["depth.bin", "depth.png"])
def test_cli_outputs_equal_library_and_oracle(gpu_ctx, files, depth_name):
    d, w, s, obj = files
    k = s["cluster"]["label"]
    r = run_cli(d, obj, depth_name, k)
    assert r.returncode == 0, r.stderr
    assert "Solution Best Pose:" in r.stdout

    # the same solve through the library
    soa, F = qpso.obj_load(obj)
    depth, labels, _ = w["frames"][0]
    cam = qpso.Camera(*scene.camera_tuple())
    mid = gpu_ctx.mesh_upload(soa, F)
    fid = gpu_ctx.frame_upload(depth, cam, labels=labels)
    c = [x for x in gpu_ctx.frame_clusters(fid) if x["label"] == k][0]
    lo, hi = qpso.box_from_centroid(c["centroid_mm"])
    x0, x1, y0, y1 = c["aabb"]
    desc = qpso.solve_desc(mesh_id=mid, frame_id=fid, cluster_label=k, cl_min_x=x0, cl_max_x=x1,
                           cl_min_y=y0, cl_max_y=y1, num_points=c["num_points"] + 1, t_lo=lo, t_hi=hi,
                           num_particles=32, iterations=6, seed=7, stream=0)
    res = gpu_ctx.solve(desc)
    stem = d / "results" / ("img_0042.png-%d" % k)
    want = "%f,%f,%f,%f,%f,%f,%f,%f" % (res.fit, *res.pose)
    assert (str(stem) + "-bestpose.csv") and open(str(stem) + "-bestpose.csv").read() == want

    img = po.render_cpu(soa, F, np.array(res.pose[:], np.float32), po.camera())
    text = "".join(", ".join("%g" % float(v) for v in row) + "\n" for row in img)
    assert open(str(stem) + "-best.csv").read() == text
    assert (img < 60000).sum() > 100
    gpu_ctx.frame_release(fid)
    gpu_ctx.mesh_release(mid)


def test_cli_edge_raster_mode(gpu_ctx, files):
    """--raster-mode edge solves with QPSO_RASTER_EDGE: the pose file equals
    the library's EDGE solve of the same cluster."""
    d, w, s, obj = files
    k = s["cluster"]["label"]
    r = run_cli(d, obj, "depth.bin", k, ("--raster-mode", "edge", "--results", str(d / "res_edge")))
    assert r.returncode == 0, r.stderr
    soa, F = qpso.obj_load(obj)
    depth, labels, _ = w["frames"][0]
    cam = qpso.Camera(*scene.camera_tuple())
    mid = gpu_ctx.mesh_upload(soa, F)
    fid = gpu_ctx.frame_upload(depth, cam, labels=labels)
    c = [x for x in gpu_ctx.frame_clusters(fid) if x["label"] == k][0]
    lo, hi = qpso.box_from_centroid(c["centroid_mm"])
    x0, x1, y0, y1 = c["aabb"]
    desc = qpso.solve_desc(mesh_id=mid, frame_id=fid, cluster_label=k, cl_min_x=x0, cl_max_x=x1,
                           cl_min_y=y0, cl_max_y=y1, num_points=c["num_points"] + 1, t_lo=lo, t_hi=hi,
                           num_particles=32, iterations=6, seed=7, stream=0, raster_mode=qpso.RASTER_EDGE)
    res = gpu_ctx.solve(desc)
    got = open(str(d / "res_edge" / ("img_0042.png-%d-bestpose.csv" % k))).read()
    assert got == "%f,%f,%f,%f,%f,%f,%f,%f" % (res.fit, *res.pose)
    gpu_ctx.frame_release(fid)
    gpu_ctx.mesh_release(mid)


def test_cli_default_reference_projection(gpu_ctx, files):
    """Without --camera the command line projects as the reference does (its
    ACCV intrinsics in double): the pose file equals the library's solve
    with QPSO_PROJ_REF_ACCV, and the best-pose depth image equals the
    oracle's restatement of the reference's host render in that
    projection."""
    d, w, s, obj = files
    k = s["cluster"]["label"]
    r = run_cli(d, obj, "depth.bin", k, ("--results", str(d / "res_ref")), camera=())
    assert r.returncode == 0, r.stderr
    soa, F = qpso.obj_load(obj)
    depth, labels, _ = w["frames"][0]
    cam = qpso.Camera(0, 0, 0, 0, 640, 480, qpso.PROJ_REF_ACCV)
    mid = gpu_ctx.mesh_upload(soa, F)
    fid = gpu_ctx.frame_upload(depth, cam, labels=labels)
    c = [x for x in gpu_ctx.frame_clusters(fid) if x["label"] == k][0]
    lo, hi = qpso.box_from_centroid(c["centroid_mm"])
    x0, x1, y0, y1 = c["aabb"]
    desc = qpso.solve_desc(mesh_id=mid, frame_id=fid, cluster_label=k, cl_min_x=x0, cl_max_x=x1,
                           cl_min_y=y0, cl_max_y=y1, num_points=c["num_points"] + 1, t_lo=lo, t_hi=hi,
                           num_particles=32, iterations=6, seed=7, stream=0)
    res = gpu_ctx.solve(desc)
    stem = d / "res_ref" / ("img_0042.png-%d" % k)
    assert open(str(stem) + "-bestpose.csv").read() == "%f,%f,%f,%f,%f,%f,%f,%f" % (res.fit, *res.pose)
    img = po.render_cpu(soa, F, np.array(res.pose[:], np.float32), po.camera_ref_accv())
    text = "".join(", ".join("%g" % float(v) for v in row) + "\n" for row in img)
    assert open(str(stem) + "-best.csv").read() == text
    gpu_ctx.frame_release(fid)
    gpu_ctx.mesh_release(mid)


def test_cli_unknown_cluster(files):
    d, w, s, obj = files
    r = run_cli(d, obj, "depth.bin", 999)
    assert r.returncode == 1 and "not in the label map" in r.stderr


# ---- from the colour image and the depth alone (no label map) ----

@pytest.fixture(scope="module")
def rgbd_files(tmp_path_factory, gpu_ctx):
    from tests.test_ingest import write_png_color, write_ppm

    d = tmp_path_factory.mktemp("cli_rgbd")
    w = scene.workload_c2(frames=1, particles=32, iterations=6)
    depth, gt, bgr = w["frames"][0]
    write_png_color(str(d / "img_0007.png"), bgr[..., ::-1])  # RGB order in the file
    write_ppm(str(d / "img_0007.ppm"), bgr[..., ::-1])
    write_png_gray(str(d / "depth.png"), depth, 16, 6, (0, 1, 2, 3, 4))
    # the kept cluster that covers solve 2's object, and that object's mesh
    s = w["solves"][2]
    seg = gpu_ctx.segment_rgbd(bgr, depth)
    m = gt == s["cluster"]["label"]
    ious = [((seg["labels"] == c.label) & m).sum() / ((seg["labels"] == c.label) | m).sum() for c in seg["clusters"]]
    n = int(np.argmax(ious))
    assert ious[n] > 0.5
    soa, F = w["meshes"][s["mesh"]]
    obj = str(d / "model.obj")
    write_obj(obj, soa, F)
    return d, bgr, depth, obj, n


@pytest.mark.parametrize("colour", ["img_0007.png", "img_0007.ppm"])
def test_cli_segments_the_frame_itself(gpu_ctx, rgbd_files, colour):
    """qpso_main obj rgb depth N with no label map: the frame is segmented on
    the GPU (qpso_segment_rgbd), cluster N of the kept clusters is solved
    against its inpainted depth, and the pose file equals the library's
    solve of that cluster and the oracle's solve of the same inputs."""
    d, bgr, depth, obj, n = rgbd_files
    res_dir = d / ("res_" + colour.split(".")[1])
    cmd = [CLI, obj, str(d / colour), str(d / "depth.png"), str(n), "--particles", "32", "--iterations", "6",
           "--seed", "7", "--results", str(res_dir)]
    run_dir = d / ("cwd_" + colour.split(".")[1])
    run_dir.mkdir(exist_ok=True)
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=str(run_dir))
    assert r.returncode == 0, r.stderr
    assert "clusters kept" in r.stdout

    seg = gpu_ctx.segment_rgbd(bgr, depth, planes=True)
    c = seg["clusters"][n]
    # one image per kept cluster (main.cu:1257-1263): the colour image inside
    # the cluster, black elsewhere; cluster N again as ./cluster.jpg (main.cu:1272)
    for i, ci in enumerate(seg["clusters"]):
        got, _ = _jpeg_decode(open(str(res_dir / ("%s-cluster%d.jpg" % (colour, i))), "rb").read())
        inside = seg["labels"] == ci.label
        want = np.where(inside[..., None], bgr, 0).astype(np.float64)
        assert got.shape == bgr.shape
        mse = np.mean((got.astype(np.float64) - want) ** 2)
        assert 10 * np.log10(255.0 ** 2 / max(mse, 1e-12)) > 30, (i, mse)
    assert not (res_dir / ("%s-cluster%d.jpg" % (colour, len(seg["clusters"])))).exists()
    assert open(str(run_dir / "cluster.jpg"), "rb").read() == \
        open(str(res_dir / ("%s-cluster%d.jpg" % (colour, n))), "rb").read()
    soa, F = qpso.obj_load(obj)
    cam = qpso.Camera(0, 0, 0, 0, 640, 480, qpso.PROJ_REF_ACCV)
    mid = gpu_ctx.mesh_upload(soa, F)
    fid = gpu_ctx.frame_upload(seg["inpainted"], cam, labels=seg["labels"])
    lo, hi = qpso.box_from_centroid(list(c.centroid_mm))
    desc = qpso.solve_desc(mesh_id=mid, frame_id=fid, cluster_label=c.label, cl_min_x=c.min_x, cl_max_x=c.max_x,
                           cl_min_y=c.min_y, cl_max_y=c.max_y, num_points=c.num_points, t_lo=lo, t_hi=hi,
                           num_particles=32, iterations=6, seed=7, stream=0)
    res = gpu_ctx.solve(desc)
    stem = res_dir / ("%s-%d" % (colour, n))
    assert open(str(stem) + "-bestpose.csv").read() == "%f,%f,%f,%f,%f,%f,%f,%f" % (res.fit, *res.pose)
    # the oracle on the same masked inpainted depth
    prm = po.default_params()
    prm.t_lo[:] = lo
    prm.t_hi[:] = hi
    prm.cl_min_x, prm.cl_max_x, prm.cl_min_y, prm.cl_max_y = c.min_x, c.max_x, c.min_y, c.max_y
    prm.num_points = c.num_points
    prm.num_particles, prm.iterations, prm.seed, prm.stream = 32, 6, 7, 0
    obs = np.where(seg["labels"] == c.label, seg["inpainted"], 0).astype(np.uint16)
    want = po.solve(soa, F, obs, po.camera_ref_accv(), prm)
    assert res.fit == want["fit"]
    np.testing.assert_array_equal(np.array(res.pose[:], np.float32), want["pose"])
    gpu_ctx.frame_release(fid)
    gpu_ctx.mesh_release(mid)


def test_cli_cluster_beyond_the_kept_ones(rgbd_files):
    d, _, _, obj, _ = rgbd_files
    run_dir = d / "cwd_beyond"
    run_dir.mkdir(exist_ok=True)
    r = subprocess.run([CLI, obj, str(d / "img_0007.png"), str(d / "depth.png"), "999", "--particles", "8",
                        "--iterations", "1"], capture_output=True, text=True, timeout=300, cwd=str(run_dir))
    assert r.returncode == 1 and "beyond" in r.stderr
