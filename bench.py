"""Benchmark of the Q-PSO pose solve on one GB300 (or N replicas).

Default workload: the plain method at production size -- one synthetic
640x480 RGB-D frame with 8 non-overlapping objects drawn from 4 procedural
meshes (~5k faces, 50-200 mm), each cluster solved by its own plain solve
(one fused launch per iteration), 256 particles x 100 iterations, fp32.  A
step is one frame: 8 pose solves.  `value` is pose solves/s with meshes and
frame resident in HBM; `e2e` re-uploads the frame (depth + labels) from
page-locked host memory every step and reads every result back.  The same
workload through the batched persistent kernel is reported under
`batched`.  Inputs are far smaller than L2, so L2 is scrubbed (256 MB
written) before every timed step.

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                        [--workload c2|c1|c3|c4|c5|seg]

--workload seg times the segmentation's graph stage instead (frames/s).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "q-pso_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "pose solves/sec (particle-renders/sec alongside), plain vs batched"
L2_SCRUB_BYTES = 256 << 20


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-over-ranks for N replicas (gloo, host scalars)."""

    def __init__(self, ws):
        self.ws = ws
        self.dist = None
        if ws > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "qpso_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device),
                                          "--query-gpu=" + self.FIELDS, "--format=csv,noheader",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # nvidia-smi's start-up competes with the launching thread for the
        # host and the driver: begin timing once it is sampling
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            self.f.flush()
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.05)
        time.sleep(0.3)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax.append(float(parts[2].split()[0]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.remove(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_workload(name: str):
    import scene

    if name == "c1":
        return scene.workload_c1(), "c1: plain single solve, 1280-face ellipsoid, 64 particles x 50 iterations"
    if name == "c2":
        return scene.workload_c2(), ("c2: plain method at production size, 8 clusters per frame, "
                                     "4 meshes ~5k faces (50-200 mm), 256 particles x 100 iterations")
    if name == "c3":
        return scene.workload_c3(), ("c3: 64 clusters from 8 frames, meshes log-uniform 1k-50k faces, "
                                     "windows 40-300 px, particles in {128..1024} x 100 iterations")
    if name == "c4":
        return scene.workload_c4(), ("c4: serving, Poisson arrivals over 16 resident meshes "
                                     "(2k-100k faces) and 32 resident 640x480 frames, 256 or 1024 "
                                     "particles x 100 iterations")
    if name == "c5":
        return scene.workload_c5(), ("c5: one level-7 icosphere (327,680 faces, 250 mm), "
                                     "4096 particles x 200 iterations, full 640x480 window")
    raise SystemExit("unknown workload " + name)


def algorithmic_bytes(w) -> tuple[float, float]:
    """Per particle-render: 36 F (mesh, loadOBJ3 layout) + 2 A (uint16
    observed window, A = cluster AABB area) + 96 (pose/velocity/best state
    read and written).  Returns (bytes summed over all renders of one pass of
    every solve, renders of that pass)."""
    tot, n = 0.0, 0
    for s in w["solves"]:
        F = w["meshes"][s["mesh"]][1]
        x0, x1, y0, y1 = s["cluster"]["aabb"]
        per = 36.0 * F + 2.0 * (x1 - x0) * (y1 - y0) + 96.0
        tot += per * s["particles"]
        n += s["particles"]
    return tot, n


def profile_figure(workload: str, kernel: str, key: str):
    """A per-launch figure of the dominant kernel from the committed ncu
    summary (profiles/<kernel>_kernel_<workload>.md, line '<key>: value')."""
    p = os.path.join(ROOT, "profiles", "%s_kernel_%s.md" % (kernel, workload))
    try:
        for line in open(p):
            if line.strip().startswith(key + ":"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def traffic_per_launch(workload: str, kernel: str = "step"):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)."""
    return profile_figure(workload, kernel, "dram_bytes_per_launch")


def sm_count(local: int) -> int:
    try:
        import torch

        return int(torch.cuda.get_device_properties(local).multi_processor_count)
    except Exception:
        return 152  # GB300


def _oracle_sample(w, budget_s: float, threads: int):
    """Run every solve of the workload through the oracle for the same number
    of iterations, chosen so that the whole sample takes about budget_s, and
    return (solve-equivalents done, particle-renders, seconds).  A solve
    run for k of its n iterations counts as k/n of a solve (iteration costs
    are flat within a solve), so the mix of the workload is preserved."""
    from oracle import pyoracle as po
    from tests.helpers import oracle_obs, oracle_params

    # probe: one iteration of the first solve, timed warm (the first call
    # also starts the library and its thread pool)
    s0 = w["solves"][0]
    soa, F = w["meshes"][s0["mesh"]]
    probe = 1e30
    for _ in range(2):
        t = time.perf_counter()
        po.solve(soa, F, oracle_obs(w, s0), po.camera(), oracle_params(s0, iterations=1),
                 threads=threads)
        probe = min(probe, time.perf_counter() - t)
    cost0 = s0["particles"] * F
    total = sum(s["particles"] * w["meshes"][s["mesh"]][1] for s in w["solves"])
    per_iter_all = probe * total / max(cost0, 1)
    iters = max(1, min(min(s["iterations"] for s in w["solves"]),
                       int(budget_s / max(per_iter_all, 1e-9))))
    done, renders = 0.0, 0
    t0 = time.perf_counter()
    for s in w["solves"]:
        soa, F = w["meshes"][s["mesh"]]
        k = min(iters, s["iterations"])
        po.solve(soa, F, oracle_obs(w, s), po.camera(), oracle_params(s, iterations=k),
                 threads=threads)
        done += k / s["iterations"]
        renders += s["particles"] * k
    return done, renders, time.perf_counter() - t0, iters


def cpu_baseline(w, budget_s: float = 12.0, single_budget_s: float = 6.0):
    """The oracle (scalar C restatement) with every host thread on a bounded
    sample of the workload (see _oracle_sample), and on one thread where one
    iteration of the workload is small enough for a few seconds of one core."""
    threads = os.cpu_count() or 1
    done, renders, dt, iters = _oracle_sample(w, budget_s, threads)
    out = {"value": done / dt, "unit": "solves/s", "cores": threads, "kind": "port",
           "sample": "every solve of the workload for %d iteration(s) (%.2f solve-equivalents, "
                     "%d particle-renders) in %.1f s" % (iters, done, renders, dt),
           "particle_renders_per_s": renders / dt}
    face_renders = sum(s["particles"] * w["meshes"][s["mesh"]][1] for s in w["solves"])
    if face_renders <= 5e7:
        d1, r1, t1, i1 = _oracle_sample(w, single_budget_s, 1)
        out["single_thread"] = {"value": d1 / t1, "unit": "solves/s", "cores": 1,
                                "particle_renders_per_s": r1 / t1,
                                "sample": "every solve for %d iteration(s) in %.1f s" % (i1, t1)}
    return out


# the ACCV intrinsics compiled into the reference's kernels (main.h:30-33)
ACCV = (572.41140, 573.57043, 325.26110, 242.04899)
REF_PARTICLES, REF_ITERATIONS = 1024, 20  # Nparticle_ and max_steps_, main.h:84, 97


def reference_shape(w, si: int = 0):
    """The reference's own solve shape (1024 particles x 20 iterations, ACCV
    camera) on solve si of the workload: its mesh and cluster, with a
    translation box around (0, 0, 0.9 m) that keeps every particle's mesh
    8 px inside the image at any rotation (the reference's raster does not
    clip): a vertex lies within r of the translation, r the largest
    object-space corner norm, so (b + r) / (z_lo - r) bounds x/z."""
    s = w["solves"][si]
    soa, F = w["meshes"][s["mesh"]]
    m = np.asarray(soa, np.float64).reshape(3, 3 * F)
    r = float(np.linalg.norm(np.maximum(np.abs(m.min(axis=1)), np.abs(m.max(axis=1)))))
    fx, fy, cx, cy = ACCV
    zc = 0.9
    zmin = zc - 0.1 - r
    bx = 0.9 * (min(cx, 640 - cx) - 8) / fx * zmin - r
    by = 0.9 * (min(cy, 480 - cy) - 8) / fy * zmin - r
    if F > 64 * 512 or min(bx, by) < 0.02:
        return None  # beyond the render's 64 block slots, or too large to stay in frame
    c = s["cluster"]
    x0, x1, y0, y1 = c["aabb"]
    return {"mesh": s["mesh"], "faces": F, "frame": s["frame"], "label": c["label"],
            "t_lo": (-bx, -by, zc - 0.1), "t_hi": (bx, by, zc + 0.1), "num_points": c["num_points"],
            "aabb": (x0, min(x1, 639), y0, min(y1, 479)), "seed": s["seed"], "stream": s["stream"],
            "desc": "mesh of %d faces, its cluster, %d particles x %d iterations, ACCV camera, "
                    "translation box +-(%.3f, %.3f) m around (0, 0, 0.9) m, +-0.1 m in z"
                    % (F, REF_PARTICLES, REF_ITERATIONS, bx, by)}


def reference_shapes(w):
    """reference_shape of every solve of the workload that the reference's
    kernels can render (all 8 clusters of the production-size frame)."""
    out = []
    for si in range(len(w["solves"])):
        sh = reference_shape(w, si)
        if sh is not None:
            out.append(sh)
    return out


REF_SHAPE_ALL = ("every cluster of the workload whose mesh the reference's kernels can render, "
                 "each at the reference's solve shape: 1024 particles x 20 iterations, ACCV camera, "
                 "its own mesh, cluster and a translation box around (0, 0, 0.9 m) that keeps every "
                 "particle in frame")


def reference_kernels_gb300(w):
    """The reference's own CUDA kernels (main.h + main.cu:72-1195 built with
    its Makefile's -use_fast_math -O3 for sm_103a) running its host loop
    (main.cu:1601-1727) on this GPU, the oracle's Philox draws in its
    uniform table: the reference-shaped solve of the workload's first
    cluster, and every cluster solved one after another, as the reference
    solves one cluster per run (its plain per-cluster path)."""
    from oracle import refgpu

    if not refgpu.available("fast"):
        return {"unavailable": "reference kernels not built: the reference sources were absent "
                               "where the repository was built"}
    shapes = reference_shapes(w)
    if not shapes:
        return {"unavailable": "does not apply: the reference's render grid holds at most 32768 "
                               "faces (64 block slots of 512 per particle, main.h:1290-1293)"}
    runs = []
    try:
        with refgpu.RefKernels("fast") as rk:
            for k, sh in enumerate(shapes):
                soa, F = w["meshes"][sh["mesh"]]
                dep, lab, _ = w["frames"][sh["frame"]]
                obs = np.where(lab == sh["label"], dep, 0).astype(np.int32)
                rk.set_scene(soa, F, obs, sh["t_lo"], sh["t_hi"], sh["num_points"], sh["aabb"])
                rk.set_rand_table(refgpu.uniform_table(sh["seed"], sh["stream"]))
                if k == 0:
                    rk.solve(2)  # warm-up
                runs.append((sh, rk.solve(REF_ITERATIONS)))
    except Exception as e:  # a baseline, not the product: report, do not fail the arm
        return {"unavailable": "reference kernels failed: %s" % e}
    sh, out = runs[0]
    done, ms = out["done"], out["ms"]
    F = sh["faces"]
    res = {"build": "reference main.h + main.cu:72-1195, -use_fast_math -O3, sm_103a; host loop "
                    "main.cu:1601-1727 (1024 render + 1024 fitness launches per iteration on 16 "
                    "streams, thrust::min_element, best and particle updates)",
           "config": "first cluster: " + sh["desc"], "render_grid": [max(6, -(-F // 512)), 512],
           "iterations_done": done, "ms_per_iteration": ms / max(done, 1),
           "particle_renders_per_s": REF_PARTICLES * done / (ms / 1000.0) if ms > 0 else None,
           "best_fit": float(out["trace"][-1]) if done else None}
    if done == REF_ITERATIONS:
        res.update(value=1000.0 / ms, unit="solves/s", ms_per_solve=ms)
    else:
        res["stopped"] = out["error"]
    per = [{"faces": sh["faces"], "iterations_done": o["done"], "ms": o["ms"],
            "best_fit": float(o["trace"][-1]) if o["done"] else None,
            "stopped": o["error"] or None} for sh, o in runs]
    full = [(sh, o) for sh, o in runs if o["done"] == REF_ITERATIONS]
    tot = sum(o["ms"] for _, o in full)
    res["all_clusters"] = {"config": REF_SHAPE_ALL, "solves": len(runs), "completed": len(full),
                           "ms": tot, "value": 1000.0 * len(full) / tot if tot > 0 else None,
                           "unit": "solves/s", "per_cluster": per}
    return res


def reference_shape_ours(ctx, w, repeats: int = 3):
    """The reference-shaped solves through this library: the first cluster
    on the plain path (the solve the reference's kernels are timed on), and
    every cluster one after another on the plain path and together in one
    batched launch (qpso_solve_batch), L2 scrubbed before each timed run."""
    import qpso

    shapes = reference_shapes(w)
    if not shapes:
        return {"unavailable": "does not apply: mesh above the reference kernels' 32768 faces"}
    mids = {}
    fids = {}
    descs = []
    for sh in shapes:
        if sh["mesh"] not in mids:
            soa, F = w["meshes"][sh["mesh"]]
            mids[sh["mesh"]] = ctx.mesh_upload(soa, F)
        if sh["frame"] not in fids:
            dep, lab, _ = w["frames"][sh["frame"]]
            fids[sh["frame"]] = ctx.frame_upload(dep, qpso.Camera(*ACCV, 640, 480), labels=lab)
        x0, x1, y0, y1 = sh["aabb"]
        descs.append(qpso.solve_desc(mesh_id=mids[sh["mesh"]], frame_id=fids[sh["frame"]],
                                     cluster_label=sh["label"], cl_min_x=x0, cl_max_x=x1, cl_min_y=y0,
                                     cl_max_y=y1, num_points=sh["num_points"], t_lo=sh["t_lo"],
                                     t_hi=sh["t_hi"], num_particles=REF_PARTICLES,
                                     iterations=REF_ITERATIONS, seed=sh["seed"], stream=sh["stream"]))

    def timed(fn):
        fn()  # warm-up (and graph capture for the batched launch)
        tot = 0.0
        for _ in range(repeats):
            ctx.scrub_l2(L2_SCRUB_BYTES)
            ctx.timer_record(0)
            out = fn()
            ctx.timer_record(1)
            tot += ctx.timer_elapsed_ms(0, 1)
        return tot / repeats, out

    ms1, r1 = timed(lambda: [ctx.solve(descs[0])])
    ms_plain, rp = timed(lambda: [ctx.solve(d) for d in descs])
    ms_batch, rb = timed(lambda: ctx.solve_batch(descs))
    same = all(a.fit == b.fit and list(a.pose) == list(b.pose) for a, b in zip(rp, rb))
    for f in fids.values():
        ctx.frame_release(f)
    for m in mids.values():
        ctx.mesh_release(m)
    n = len(descs)
    return {"config": "first cluster: " + shapes[0]["desc"], "value": 1000.0 / ms1, "unit": "solves/s",
            "ms_per_solve": ms1,
            "particle_renders_per_s": REF_PARTICLES * REF_ITERATIONS / (ms1 / 1000.0),
            "best_fit": float(r1[0].fit),
            "all_clusters": {"config": REF_SHAPE_ALL, "solves": n,
                             "plain": {"value": 1000.0 * n / ms_plain, "unit": "solves/s", "ms": ms_plain},
                             "batched": {"value": 1000.0 * n / ms_batch, "unit": "solves/s",
                                         "ms": ms_batch},
                             "plain_batched_bit_identical": bool(same),
                             "best_fits": [float(r.fit) for r in rb]}}


def accuracy_vs_ground_truth(ctx, w, descs, results, refine: bool = True):
    """How close the solved poses are to the synthetic scenes' true poses:
    median translation error (mm) and rotation error (degrees; symmetric
    procedural shapes make this an upper bound), and the fraction of solves
    whose best fitness is at most the true pose's own fitness (the swarm
    found a pose the objective ranks at least as well as the truth).  With
    refine, the same after qpso_refine (EDGE raster, default search) of
    every solved pose, beside the unchanged solve."""
    import qpso

    def errs(poses):
        t_err, r_err = [], []
        for s, pose in zip(w["solves"], poses):
            gt = np.asarray(s["gt_pose"], np.float64)
            pose = np.asarray(pose, np.float64)
            t_err.append(1000.0 * float(np.linalg.norm(pose[:3] - gt[:3])))
            dq = abs(float(np.dot(pose[3:], gt[3:])))
            r_err.append(2.0 * float(np.degrees(np.arccos(min(1.0, dq)))))
        return float(np.median(t_err)), float(np.median(r_err))

    le = 0
    for s, d, r in zip(w["solves"], descs, results):
        le += int(r.fit <= float(ctx.score_poses(d, np.asarray(s["gt_pose"], np.float32)[None])[0]))
    t_med, r_med = errs([r.pose[:] for r in results])
    out = {"trans_mm_median": t_med, "rot_deg_median": r_med,
           "fit_at_most_true_pose_fraction": le / len(results), "solves": len(results)}
    if refine:
        prm = qpso.refine_params()
        poses, le_r = [], 0
        t0 = time.perf_counter()
        for s, d, r in zip(w["solves"], descs, results):
            pose, fit = ctx.refine(d, np.array(r.pose[:], np.float32), prm)
            poses.append(pose)
            d_edge = qpso.SolveDesc.from_buffer_copy(d)
            d_edge.raster_mode = qpso.RASTER_EDGE
            le_r += int(fit <= float(ctx.score_poses(d_edge, np.asarray(s["gt_pose"], np.float32)[None])[0]))
        dt = time.perf_counter() - t0
        t_ref, r_ref = errs(poses)
        out["refined"] = {"trans_mm_median": t_ref, "rot_deg_median": r_ref,
                          "fit_at_most_true_pose_fraction": le_r / len(results),
                          "ms_per_solve": 1000.0 * dt / len(results),
                          "search": "qpso_refine: %d rounds x %d candidates, EDGE raster, steps %.3f m / %.2f rad"
                                    % (prm.rounds, prm.candidates, prm.step_t, prm.step_rot)}
    return out


def run_reference(args, ws, rank):
    """Reference arm: the oracle port on the host cores (the reference's own
    program needs OpenCV 2.4, assimp, GSL and a missing header and cannot be
    built); each step is a bounded sample of the workload (_oracle_sample)."""
    if rank != 0:
        return
    w, desc = load_workload(args.workload)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        _oracle_sample(w, 2.0, threads)
    tot_done, tot_renders, tot_dt, iters = 0.0, 0, 0.0, 0
    for _ in range(args.steps):
        d_, r_, t_, iters = _oracle_sample(w, 6.0, threads)
        tot_done += d_
        tot_renders += r_
        tot_dt += t_
    v = tot_done / tot_dt
    sample = ("per step every solve of the workload for %d iteration(s), counted as "
              "solve-equivalents" % iters)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tot_dt * 1000 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "sample": sample},
            "particle_renders_per_s": tot_renders / tot_dt,
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if not args.no_ref_kernels:
        line["reference_kernels_gb300"] = reference_kernels_gb300(w)
    print(json.dumps(line))


def extra_c3(ctx, local, hbm: float, mhz: float):
    """The batching config (C3: 64 clusters, 1k-50k faces, 128-1024
    particles x 100 iterations) in the default run: one batched step (all
    64 solves in one persistent launch) and one plain step (the same solves
    one plain solve after another), both L2-scrubbed, with the batched
    kernel's HBM and issue rooflines."""
    import qpso
    import scene

    w = scene.workload_c3()
    cam = qpso.Camera(*scene.camera_tuple())
    mids = [ctx.mesh_upload(soa, F) for soa, F in w["meshes"]]
    fids = [ctx.frame_upload(dep, cam, labels=lab) for dep, lab, _ in w["frames"]]
    descs = [qpso.solve_desc(mesh_id=mids[s["mesh"]], frame_id=fids[s["frame"]], **scene.solve_fields(s))
             for s in w["solves"]]
    tune = descs[::max(1, len(descs) // 16)][:16]
    plain_cfg, _ = ctx.autotune(tune[::4][:4], batched=False, tune_iters=30)
    batch_cfg, _ = ctx.autotune(tune, batched=True, tune_iters=30)
    rb = ctx.solve_batch(descs)  # warm-up (graph capture)
    rp = [ctx.solve(d) for d in descs]
    same = all(a.fit == b.fit and list(a.pose) == list(b.pose) for a, b in zip(rb, rp))

    def timed(fn, prof=False):
        ctx.set_profiling(prof)
        ctx.profile(reset=True)
        ctx.scrub_l2(L2_SCRUB_BYTES)
        ctx.timer_record(0)
        fn()
        ctx.timer_record(1)
        ms = ctx.timer_elapsed_ms(0, 1)
        ctx.set_profiling(False)
        return ms, ctx.profile(reset=True)

    ms_b, _ = timed(lambda: ctx.solve_batch(descs))
    ms_b2, prof = timed(lambda: ctx.solve_batch(descs), prof=True)
    ms_p, _ = timed(lambda: [ctx.solve(d) for d in descs])
    n = len(descs)
    renders = sum(s["particles"] * s["iterations"] for s in w["solves"])
    bytes_pass, _ = algorithmic_bytes(w)
    iters = sum(s["iterations"] for s in w["solves"])
    kern_ms = min(ms_b, prof["batch_ms"] / max(1, prof["batch_launches"]))
    bytes_launch = bytes_pass * iters / n
    achieved = bytes_launch / (kern_ms / 1000.0) / 1e9
    out = {"workload": "c3: 64 clusters from 8 frames, meshes log-uniform 1k-50k faces, windows "
                       "40-300 px, particles in {128..1024} x 100 iterations",
           "batched": {"value": 1000.0 * n / ms_b, "unit": "solves/s", "ms_per_step": ms_b,
                       "particle_renders_per_s": renders / (ms_b / 1000.0),
                       "launch": {"threads": batch_cfg[0], "tile_px": batch_cfg[1], "ppb": batch_cfg[2]}},
           "plain": {"value": 1000.0 * n / ms_p, "unit": "solves/s", "ms_per_step": ms_p,
                     "launch": {"threads": plain_cfg[0], "tile_px": plain_cfg[1], "ppb": plain_cfg[2]}},
           "speedup_batched_vs_plain": ms_p / ms_b, "plain_batched_bit_identical": bool(same),
           "accuracy_vs_ground_truth": accuracy_vs_ground_truth(ctx, w, descs, rb),
           "device_error_bits": int(max(r.flags for r in rb)),
           "roofline": {"kernel": "qpso_batch_kernel", "bound": "hbm", "achieved": achieved, "peak": hbm,
                        "unit": "GB/s", "frac": achieved / hbm, "bytes_per_launch": bytes_launch,
                        "avg_launch_ms": kern_ms, "model": "36F + 2A + 96 bytes per particle-render"}}
    inst = profile_figure("c3", "batch", "inst_per_launch")
    if inst:
        peak_issue = 4.0 * sm_count(local) * mhz * 1e6
        out["issue_roofline"] = {"kernel": "qpso_batch_kernel", "achieved": inst / (kern_ms / 1000.0),
                                 "peak": peak_issue, "unit": "warp-inst/s",
                                 "frac": inst / (kern_ms / 1000.0) / peak_issue, "inst_per_launch": inst,
                                 "sm_mhz": mhz}
    for f in fids:
        ctx.frame_release(f)
    for m in mids:
        ctx.mesh_release(m)
    return out


def extra_c4(ctx, slots: int = 64, epoch_iters: int = 10, rates=(25.0, 40.0, 50.0), duration_s: float = 5.0):
    """The serving config (C4) in the default run: Poisson arrivals at three
    rates for duration_s each (serving_sweep)."""
    import scene

    w = scene.workload_c4()
    pool, mids, fids = c4_pool(ctx, w)
    cfg, _ = ctx.autotune(pool[:16], batched=True, tune_iters=6)
    results, top, best = serving_sweep(ctx, pool, list(rates), duration_s, slots, epoch_iters,
                                       max_requests=400)
    batched = batched_same_mix(ctx, pool)
    for f in fids:
        ctx.frame_release(f)
    for m in mids:
        ctx.mesh_release(m)
    head = top or best
    return {"workload": "c4: Poisson arrivals over 16 resident meshes (2k-100k faces) and 32 resident "
                        "640x480 frames, 256 or 1024 particles x 100 iterations",
            "slots": slots, "iters_per_epoch": epoch_iters, "seconds_per_rate": duration_s,
            "launch_batched": {"threads": cfg[0], "tile_px": cfg[1], "ppb": cfg[2]},
            "sustained_rate_req_s": top["rate_req_s"] if top else None,
            "sustained_solves_per_s": top["solves_per_s"] if top else None,
            "p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"],
            "saturated_solves_per_s": best["solves_per_s"], "batched_same_mix": batched, "sweep": results}


def seg_throughput(local: int, bgr, depth, threads: int = 4, frames: int = 12) -> dict:
    """Frames/s of qpso_segment_rgbd with `threads` host threads, each with
    its own context (stream, workspaces, pinned buffers) on the same GPU,
    each segmenting `frames` frames: the host merge passes of different
    frames run on different cores while the GPUs' stages interleave.  The
    latency of one frame is unchanged."""
    import threading

    import qpso

    ctxs = [qpso.Context(local) for _ in range(threads)]
    for c in ctxs:  # size every context's buffers first
        for _ in range(2):
            c.segment_rgbd(bgr, depth)
    barrier = threading.Barrier(threads + 1)
    errors = []

    def work(c):
        try:
            barrier.wait()
            for _ in range(frames):
                c.segment_rgbd(bgr, depth)
        except Exception as e:  # reported below
            errors.append(e)
    ts = [threading.Thread(target=work, args=(c,)) for c in ctxs]
    for t in ts:
        t.start()
    barrier.wait()
    t0 = time.perf_counter()
    for t in ts:
        t.join()
    dt = time.perf_counter() - t0
    for c in ctxs:
        c.close()
    if errors:
        raise errors[0]
    return {"value": threads * frames / dt, "unit": "frames/s", "threads": threads, "contexts": threads,
            "frames_per_thread": frames}


def extra_seg(ctx, steps: int = 10, warmup: int = 3):
    """The segmentation in the default run: frames/s of qpso_segment_rgbd
    (GraphCannySeg<hsv>::run, colour image and raw depth on the host to the
    label map and the kept clusters on the host) on the stress
    configuration's 640x480 frame with 15 objects, and of the graph stage
    alone (qpso_segment_planes) on its own synthetic planes."""
    import qpso
    import scene

    depth, _, bgr = scene.segmentation_frame_c5()
    for _ in range(warmup):  # the first calls size the workspace and the pinned buffers
        ctx.segment_rgbd(bgr, depth)
    t0 = time.perf_counter()
    for _ in range(steps):
        out = ctx.segment_rgbd(bgr, depth)
    dt = time.perf_counter() - t0
    frame = segmentation_frame(seed=11)
    prm = qpso.seg_params()
    for _ in range(warmup):
        ctx.segment_planes(*frame, prm)
    t1 = time.perf_counter()
    for _ in range(steps):
        ctx.segment_planes(*frame, prm)
    dt_g = time.perf_counter() - t1
    return {"workload": "the stress configuration's 640x480 RGB-D frame with 15 objects, qpso_segment_rgbd "
                        "from host BGR and depth to host labels and kept clusters",
            "value": steps / dt, "unit": "frames/s", "ms_per_frame": dt * 1000.0 / steps,
            "sets": int(out["n_sets"]), "clusters_kept": len(out["clusters"]),
            "graph_stage_only": {"value": steps / dt_g, "unit": "frames/s", "ms_per_frame": dt_g * 1000.0 / steps},
            "four_contexts": seg_throughput(ctx.device, bgr, depth)}


def run_ours(args, ws, rank, local):
    import qpso
    import build as pkg_build
    import scene

    pkg_build.build()
    d = Dist(ws)
    w, desc = load_workload(args.workload)
    ctx = qpso.Context(local)
    cam = qpso.Camera(*scene.camera_tuple())
    mids = [ctx.mesh_upload(soa, F) for soa, F in w["meshes"]]
    fids = [ctx.frame_upload(dep, cam, labels=lab) for dep, lab, _ in w["frames"]]
    descs = []
    for s in w["solves"]:
        f = scene.solve_fields(s)
        descs.append(qpso.solve_desc(mesh_id=mids[s["mesh"]], frame_id=fids[s["frame"]], **f))
    n_solves = len(descs)
    renders_per_step = sum(s["particles"] * s["iterations"] for s in w["solves"])
    iters_per_step = sum(s["iterations"] for s in w["solves"])
    batched_default = args.workload == "c3"

    # pinned host copies of the frames for the end-to-end arm
    pinned = []
    for dep, lab, _ in w["frames"]:
        pd = qpso.PinnedArray(dep.shape, np.uint16)
        pl = qpso.PinnedArray(lab.shape, np.int32)
        pd.array[...] = dep
        pl.array[...] = lab
        pinned.append((pd, pl))
    h2d = sum(pd.nbytes + pl.nbytes for pd, pl in pinned) + n_solves * qpso.C.sizeof(qpso.SolveDesc)
    d2h = n_solves * qpso.C.sizeof(qpso.Result)

    def step_plain(e2e=False):
        if e2e:
            for fid, (pd, pl) in zip(fids, pinned):
                ctx.frame_update(fid, pd.array, pl.array)
        return [ctx.solve(x) for x in descs]

    def step_batch(e2e=False):
        if e2e:
            for fid, (pd, pl) in zip(fids, pinned):
                ctx.frame_update(fid, pd.array, pl.array)
        return ctx.solve_batch(descs)

    def timed(fn, steps, e2e=False, prof=False):
        ctx.set_profiling(prof)
        ctx.profile(reset=True)
        total = 0.0
        for _ in range(steps):
            ctx.scrub_l2(L2_SCRUB_BYTES)
            ctx.timer_record(0)
            fn(e2e)
            ctx.timer_record(1)
            total += ctx.timer_elapsed_ms(0, 1)
        ctx.set_profiling(False)
        return total, ctx.profile(reset=True)

    # launch shapes chosen by the autotuner on 30-iteration runs of up to 16
    # solves spread over the workload (the first iterations, with the swarm
    # still spread out, render larger than the converged ones)
    # (--launch fixes both shapes instead, e.g. to profile one shape)
    if args.launch:
        plain_cfg = batch_cfg = tuple(int(x) for x in args.launch.split(","))
        ctx.set_launch_config(plain=plain_cfg, batch=batch_cfg)
    else:
        tune = descs[::max(1, len(descs) // 16)][:16]
        tune_iters = 20 if args.workload == "c5" else 30
        plain_cfg, _ = ctx.autotune(tune[::max(1, len(tune) // 4)][:4], batched=False, tune_iters=tune_iters)
        batch_cfg, _ = ctx.autotune(tune, batched=True, tune_iters=tune_iters)

    main_fn, alt_fn = (step_batch, step_plain) if batched_default else (step_plain, step_batch)
    for _ in range(args.warmup):
        main_fn()
        alt_fn()
    # correctness of what is timed: plain and batched agree bit for bit
    r_main, r_alt = main_fn(), alt_fn()
    writes_per_step = sum(r.raster_writes for r in r_main)
    accuracy = accuracy_vs_ground_truth(ctx, w, descs, r_main)
    agree = all(a.fit == b.fit and list(a.pose) == list(b.pose) for a, b in zip(r_main, r_alt))
    flags = max(r.flags for r in r_main)

    sampler = ClockSampler(local)
    d.barrier()
    sampler.start()
    ms_main, _ = timed(main_fn, args.steps)
    clocks = sampler.stop()
    ms_main = d.max(ms_main)
    d.barrier()
    # the same steps again with events around every kernel launch, for the
    # roofline's per-launch kernel time (the events themselves slow the
    # step by a few per cent, so the headline is timed without them)
    _, prof = timed(main_fn, args.steps, prof=True)
    ms_e2e, _ = timed(main_fn, args.steps, e2e=True)
    ms_e2e = d.max(ms_e2e)
    alt_steps = max(1, args.steps if not batched_default else min(args.steps, 2))
    ms_alt, prof_alt = timed(alt_fn, alt_steps, prof=True)
    ms_alt = d.max(ms_alt)

    value = ws * n_solves * args.steps / (ms_main / 1000.0)
    e2e = ws * n_solves * args.steps / (ms_e2e / 1000.0)
    alt = ws * n_solves * alt_steps / (ms_alt / 1000.0)
    plain_v, batch_v = (alt, value) if batched_default else (value, alt)

    # roofline of the dominant kernel (fused per-iteration kernel on the plain
    # path, the persistent kernel on the batched path)
    bytes_pass, renders_pass = algorithmic_bytes(w)
    hbm, peak_kind = peaks()
    if batched_default:
        launches = max(1, prof["batch_launches"])
        kern_ms = prof["batch_ms"] / launches
        bytes_launch = bytes_pass * (iters_per_step / n_solves)
        kname = "qpso_batch_kernel"
        gpu_launches = prof["batch_launches"] + prof["prep_launches"]
    else:
        launches = max(1, prof["step_launches"])
        kern_ms = prof["step_ms"] / launches
        bytes_launch = bytes_pass / n_solves
        kname = "qpso_step_kernel"
        gpu_launches = prof["step_launches"] + prof["prep_launches"]
    # events around every launch also time the gap before each kernel starts,
    # so their mean is an upper bound; so is the clean pass's step time per
    # launch (it adds the prep kernels and gaps): take the smaller one
    kern_ms_events = kern_ms
    kern_ms_clean = ms_main / launches
    kern_ms = min(kern_ms_events, kern_ms_clean)
    achieved = bytes_launch / (kern_ms / 1000.0) / 1e9 if kern_ms > 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_main / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "path": "batched" if batched_default else "plain",
                   "launch_plain": {"threads": plain_cfg[0], "tile_px": plain_cfg[1], "ppb": plain_cfg[2]},
                   "launch_batched": {"threads": batch_cfg[0], "tile_px": batch_cfg[1], "ppb": batch_cfg[2]},
                   "launch_source": "fixed (--launch)" if args.launch else "autotuned",
                   "solves_per_step": n_solves, "l2": "scrubbed (256 MB write) before every step",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "particle_renders_per_s": value * renders_per_step / n_solves,
        "face_renders_per_s": value * sum(s["particles"] * s["iterations"] * w["meshes"][s["mesh"]][1]
                                          for s in w["solves"]) / n_solves,
        "raster_atomics_per_s": value * writes_per_step / n_solves,
        "plain": {"value": plain_v, "unit": "solves/s"},
        "batched": {"value": batch_v, "unit": "solves/s", "speedup_vs_plain": batch_v / plain_v},
        "plain_batched_bit_identical": bool(agree), "device_error_bits": int(flags),
        "accuracy_vs_ground_truth": accuracy,
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(gpu_launches),
        "roofline": {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm if achieved else None,
                     "peak_source": peak_kind,
                     "traffic": traffic_per_launch(args.workload, "batch" if batched_default else "step"),
                     "bytes_per_launch": bytes_launch, "avg_launch_ms": kern_ms,
                     "avg_launch_ms_events": kern_ms_events, "avg_launch_ms_clean_pass": kern_ms_clean,
                     "avg_launch_source": "the smaller of the per-launch CUDA-event mean and the "
                                          "clean pass's time per launch; both are upper bounds",
                     "model": "36F + 2A + 96 bytes per particle-render"},
        "clocks": clocks,
    }
    # the bound this kernel does meet: instruction issue.  Warp-instructions
    # per launch (smsp__inst_executed.sum, mean over the launch list of a run
    # of this workload) over the live launch time, against four schedulers
    # per SM issuing one warp-instruction per cycle at the sampled SM clock
    kind = "batch" if batched_default else "step"
    inst = profile_figure(args.workload, kind, "inst_per_launch")
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    if inst and kern_ms > 0:
        peak_issue = 4.0 * sm_count(local) * mhz * 1e6
        line["issue_roofline"] = {"kernel": kname, "bound": "issue", "achieved": inst / (kern_ms / 1000.0),
                                  "peak": peak_issue, "unit": "warp-inst/s",
                                  "frac": inst / (kern_ms / 1000.0) / peak_issue, "inst_per_launch": inst,
                                  "sm_mhz": mhz, "sms": sm_count(local)}
    if rank == 0 and ws == 1 and not args.no_ref_kernels:
        line["reference_shape"] = reference_shape_ours(ctx, w)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w)
    if rank == 0 and ws == 1 and args.workload == "c2" and not args.no_extras:
        # the other configurations of the metric, measured in the same run
        for pd, pl in pinned:
            pd.close()
            pl.close()
        pinned = []
        for f in fids:
            ctx.frame_release(f)
        for m in mids:
            ctx.mesh_release(m)
        sampler = ClockSampler(local)
        sampler.start()
        line["c3"] = extra_c3(ctx, local, hbm, mhz)
        line["c4"] = extra_c4(ctx)
        line["seg"] = extra_seg(ctx)
        line["extras_clocks"] = sampler.stop()
    if rank == 0:
        print(json.dumps(line))
    for pd, pl in pinned:
        pd.close()
        pl.close()
    ctx.close()
    d.close()


def serving_sweep(ctx, pool, rates, duration_s: float, slots: int, epoch_iters: int, seed: int = 17,
                  max_requests: int = 400):
    """Poisson arrivals at each rate for duration_s seconds, requests drawn
    from the pool of descriptors; latency is submit -> completion on the
    host clock, throughput is completed requests / (last completion - first
    arrival).  A rate counts as sustained when the server completed at least
    90% of the offered rate.  At most max_requests arrive per rate, so a
    rate far above capacity is a burst whose arrival window is reported."""
    import qpso

    rng = np.random.default_rng(seed)
    # warm-up: the first epochs capture and load the kernels
    with qpso.Server(ctx, max_slots=slots, iters_per_epoch=epoch_iters) as srv:
        for rid in [srv.submit(pool[i]) for i in range(min(4, len(pool)))]:
            srv.wait(rid)
    results = []
    for rate in rates:
        n = max(1, min(max_requests, int(rng.poisson(rate * duration_s))))
        gaps = rng.exponential(1.0 / rate, n)
        picks = [pool[int(i)] for i in rng.integers(0, len(pool), n)]
        with qpso.Server(ctx, max_slots=slots, iters_per_epoch=epoch_iters) as srv:
            ids = []
            t0 = time.perf_counter()
            due = t0
            for d, g in zip(picks, gaps):
                due += g
                while time.perf_counter() < due:
                    pass
                ids.append(srv.submit(d))
            t_arr = time.perf_counter() - t0
            lats = [srv.wait(rid)[1] for rid in ids]
            span = time.perf_counter() - t0
            st = srv.stats()
        lats = np.array(lats)
        offered = n / max(t_arr, 1e-9)
        tput = n / span
        results.append({"rate_req_s": rate, "requests": n, "arrival_s": t_arr, "offered_req_s": offered,
                        "p50_ms": float(np.percentile(lats, 50)), "p99_ms": float(np.percentile(lats, 99)),
                        "solves_per_s": tput, "sustained": bool(tput >= 0.9 * offered),
                        "particle_renders_per_s": sum(d.num_particles * d.iterations for d in picks) / span,
                        "peak_active": st["peak_active"], "epochs": st["epochs"],
                        "launches": st["launches"]})
    sus = [r for r in results if r["sustained"]]
    top = max(sus, key=lambda r: r["solves_per_s"]) if sus else None
    best = max(results, key=lambda r: r["solves_per_s"])
    return results, top, best


def batched_same_mix(ctx, pool, n: int = 64, seed: int = 17):
    """The batched path (qpso_solve_batch, one persistent launch) over n
    requests drawn from the serving pool as the sweep draws them: the
    throughput the serving loop's epochs are measured against."""
    rng = np.random.default_rng(seed + 1)
    picks = [pool[int(i)] for i in rng.integers(0, len(pool), n)]
    ctx.solve_batch(picks)  # warm-up (graph capture)
    ctx.scrub_l2(L2_SCRUB_BYTES)
    ctx.timer_record(0)
    ctx.solve_batch(picks)
    ctx.timer_record(1)
    ms = ctx.timer_elapsed_ms(0, 1)
    return {"requests": n, "value": 1000.0 * n / ms, "unit": "solves/s", "ms": ms}


def c4_pool(ctx, w):
    import qpso
    import scene

    cam = qpso.Camera(*scene.camera_tuple())
    mids = [ctx.mesh_upload(soa, F) for soa, F in w["meshes"]]
    fids = [ctx.frame_upload(dep, cam, labels=lab) for dep, lab, _ in w["frames"]]
    pool = [qpso.solve_desc(mesh_id=mids[s["mesh"]], frame_id=fids[s["frame"]], **scene.solve_fields(s))
            for s in w["solves"]]
    return pool, mids, fids


def run_serving(args, ws, rank, local):
    """C4: continuous-batching server under Poisson arrivals (serving_sweep)."""
    import qpso
    import build as pkg_build

    pkg_build.build()
    w, desc = load_workload("c4")
    ctx = qpso.Context(local)
    pool, _, _ = c4_pool(ctx, w)
    if args.launch:  # a fixed shape instead of the autotuner's choice
        cfg = tuple(int(x) for x in args.launch.split(","))
        ctx.set_launch_config(batch=cfg)
    else:
        cfg, _ = ctx.autotune(pool[:16], batched=True, tune_iters=6)
    rates = [float(r) for r in args.rates.split(",")]
    sampler = ClockSampler(local)
    sampler.start()
    results, top, best = serving_sweep(ctx, pool, rates, args.duration, args.slots, args.epoch_iters,
                                       max_requests=args.max_requests)
    clocks = sampler.stop()
    batched = None if args.no_extras else batched_same_mix(ctx, pool)
    head = top or best
    line = {"metric": "pose solves/sec at sustained load with p50/p99 latency (serving)",
            "value": head["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": len(rates),
            "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": desc, "slots": args.slots, "iters_per_epoch": args.epoch_iters,
                       "seconds_per_rate": args.duration,
                       "launch_batched": {"threads": cfg[0], "tile_px": cfg[1], "ppb": cfg[2]}},
            "sustained_rate_req_s": top["rate_req_s"] if top else None,
            "p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"],
            "saturated_solves_per_s": best["solves_per_s"], "batched_same_mix": batched, "sweep": results,
            "clocks": clocks}
    print(json.dumps(line))
    ctx.close()


SEG_METRIC = "segmentation frames/sec (GraphCannySeg from RGB-D, 640x480)"


def segmentation_frame(H: int = 480, W: int = 640, seed: int = 11):
    """A synthetic frame for the segmentation's graph stage: 8-bit HSV planes
    (a background plus a dozen rectangles of other colours), depth in mm (a
    tilted plane with the rectangles 50-400 mm nearer, 0-2 mm noise, 3%
    dropout) and a saliency map (forward differences of V)."""
    rng = np.random.default_rng(seed)
    h8 = np.full((H, W), 20, np.uint8)
    s8 = np.full((H, W), 60, np.uint8)
    v8 = np.full((H, W), 120, np.uint8)
    d = (900 + np.arange(H)[:, None] * 2 + np.arange(W)[None, :] // 2).astype(np.int32)
    for _ in range(12):
        y0, x0 = int(rng.integers(0, H - 40)), int(rng.integers(0, W - 40))
        y1, x1 = y0 + int(rng.integers(30, 160)), x0 + int(rng.integers(30, 200))
        h8[y0:y1, x0:x1] = rng.integers(0, 181)
        s8[y0:y1, x0:x1] = rng.integers(40, 256)
        v8[y0:y1, x0:x1] = rng.integers(40, 256)
        d[y0:y1, x0:x1] -= int(rng.integers(50, 400))
    d = d + rng.integers(0, 3, (H, W))
    d[rng.random((H, W)) < 0.03] = 0
    vf = v8.astype(np.float32)
    gx, gy = np.zeros_like(vf), np.zeros_like(vf)
    gx[:, :-1] = np.abs(np.diff(vf, axis=1))
    gy[:-1, :] = np.abs(np.diff(vf, axis=0))
    return h8, s8, v8, d.astype(np.uint16), ((gx + gy) / 510.0).astype(np.float32)


def _oracle_segment_rate(frame, budget_s: float):
    """The oracle's segmentation (GraphCannySeg<hsv>::run restated: depth
    smoothing, inpainting, Canny saliency, graph, merge, cluster filter) of
    the frame on one host core, repeated for about budget_s: frames/s."""
    from oracle import pyoracle as po

    depth, bgr = frame
    n, t0 = 0, time.perf_counter()
    while True:
        po.segment_rgbd(bgr, depth)
        n += 1
        dt = time.perf_counter() - t0
        if dt >= budget_s:
            return n / dt, n


def run_segment(args, ws, rank, local):
    """The segmentation (qpso_segment_rgbd): a step is one 640x480 RGB-D
    frame with 15 objects from host colour image and depth to the host
    label map and kept clusters, so every step includes the uploads, the
    GPU stages, the copies back and the host merge passes; it is timed on
    the host clock around the call.  Replicas under torchrun segment their
    own frames."""
    import qpso
    import build as pkg_build
    import scene

    d = Dist(ws)
    depth, _, bgr = scene.segmentation_frame_c5(seed=rank)
    frame = (depth, bgr)
    H, W = depth.shape
    desc = ("seg: one 640x480 RGB-D frame with 15 objects per step (the stress configuration's "
            "segmentation), GraphCannySeg<hsv>::run from host BGR and depth to host labels and clusters")
    if args.impl == "reference":
        if rank == 0:
            for _ in range(args.warmup):
                _oracle_segment_rate(frame, 0.5)
            rates = [_oracle_segment_rate(frame, 3.0)[0] for _ in range(args.steps)]
            v = statistics.median(rates)
            base = {"value": v, "unit": "frames/s", "cores": 1, "kind": "port",
                    "sample": "the oracle's segmentation of the frame, repeated for 3 s per step"}
            print(json.dumps({"impl": "reference", "metric": SEG_METRIC, "value": v, "unit": "frames/s",
                              "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                              "config": {"workload": desc}, "cpu_baseline": base,
                              "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0,
                                      "d2h_bytes_per_step": 0}}))
        d.close()
        return
    pkg_build.build()
    ctx = qpso.Context(local)
    for _ in range(args.warmup):
        out = ctx.segment_rgbd(bgr, depth)
    sampler = ClockSampler(local)
    d.barrier()
    sampler.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = ctx.segment_rgbd(bgr, depth)
    dt = d.max(time.perf_counter() - t0)
    clocks = sampler.stop()
    if rank == 0:
        value = ws * args.steps / dt
        E = qpso.segment_num_edges(W, H)
        line = {"metric": SEG_METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1000.0 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": desc, "edges": int(E), "sets": int(out["n_sets"]),
                           "clusters_kept": len(out["clusters"]), "l2": "inputs uploaded every step"},
                # per frame: 22 front-stage kernels, 26 graph-stage kernels (5 + 7 sort passes of 3
                # for a 640x480 frame), 17 for the merge (the weight-0 forest and packing, the
                # small-component candidates, the labels), 2 for the per-set moments
                "edges_per_s": value * E, "clocks": clocks, "gpu_launches": args.steps * 67,
                "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": int(H * W * 5),
                        "d2h_bytes_per_step": int(20 * E + 4 * H * W)}}
        line["four_contexts"] = seg_throughput(local, bgr, depth)
        if not args.no_cpu_baseline:
            v, n = _oracle_segment_rate(frame, 10.0)
            line["cpu_baseline"] = {"value": v, "unit": "frames/s", "cores": 1, "kind": "port",
                                    "sample": "%d oracle segmentations of the frame" % n}
        print(json.dumps(line))
    ctx.close()
    d.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "seg"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-kernels", action="store_true",
                    help="skip the reference-shaped solve (1024 particles x 20 iterations)")
    ap.add_argument("--no-extras", action="store_true",
                    help="c2: skip the C3, C4 and segmentation measurements added to the line; "
                         "c4: skip the batched run of the same mix")
    ap.add_argument("--launch", default="", help="THREADS,TILE_PX,PPB for both paths instead of autotuning")
    ap.add_argument("--rates", default="25,40,50,100,1000,20000", help="c4: arrival rates (req/s)")
    ap.add_argument("--max-requests", type=int, default=400, help="c4: requests per rate at most")
    ap.add_argument("--duration", type=float, default=5.0, help="c4: seconds of arrivals per rate")
    ap.add_argument("--slots", type=int, default=64, help="c4: server slots")
    ap.add_argument("--epoch-iters", type=int, default=10, help="c4: iterations a request advances per epoch")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.workload == "seg":
        run_segment(args, ws, rank, local)
        return
    if args.workload == "c4" and args.impl != "reference":
        run_serving(args, ws, rank, local)
        return
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
