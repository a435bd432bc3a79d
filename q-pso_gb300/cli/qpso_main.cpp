// qpso_main -- command-line drop-in for the reference's executable
// (main.cu:1198-1780, README.md:24-29):
//
//   qpso_main path/to/.obj color_image depth_image cluster_idx [options]
//
// loads the object model (OBJ text), the colour image (PNG or binary PPM)
// and the depth image (the ACCV binary format of loadDepth, main.cu:35-64,
// or a 16-bit greyscale PNG), segments the frame on the GPU as the
// reference's GraphCannySeg does (qpso_segment_rgbd: depth smoothing,
// inpainting, Canny saliency, graph segmentation, PostSegmFilter), takes
// the kept cluster `cluster_idx` in the reference's order
// (vecSegResult[N], main.cu:1253-1269), solves its pose on the GPU against
// the cluster's inpainted depth and writes what the reference writes:
//
//   results/<color_image>-cluster<i>.jpg             each kept cluster's colours
//                                                    (segmenting runs; cluster N
//                                                    also as ./cluster.jpg)
//   results/<color_image>-<cluster_idx>-bestpose.csv  fit,tx,ty,tz,q0,q1,q2,q3
//                                                     (main.cu:1752-1757)
//   results/<color_image>-<cluster_idx>-best.csv      the best pose's depth
//                                                     image (RenderCPU,
//                                                     main.h:2012-2043)
//
// With a label map (--labels FILE: a uint16 image in either format, 0 = no
// cluster, k+1 = cluster k; or a file <depth_image>.labels.png beside the
// depth) the clusters come from it instead, the raw depth is solved
// against, and the colour image only names the outputs.  Uses only the C
// ABI of libqpso_gb300.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "qpso.h"

namespace {

int usage(const char* argv0) {
  std::printf(
      "Usage: %s path/to/.obj color_image depth_image cluster_idx\n"
      "       [--labels FILE] [--particles N] [--iterations N] [--seed N] [--stream N]\n"
      "       [--camera fx,fy,cx,cy] [--results DIR] [--device N] [--raster-mode ref|edge]\n"
      "Without --camera the reference's own projection is used (its ACCV intrinsics in double).\n"
      "Without a label map the frame is segmented from the colour image and the depth.\n",
      argv0);
  return 0;  // the reference returns 0 after its usage line too
}

int die(const char* what, const std::string& detail) {
  std::fprintf(stderr, "qpso_main: %s: %s\n", what, detail.c_str());
  return 1;
}

std::string base_name(const std::string& p) {
  const size_t s = p.find_last_of('/');
  return s == std::string::npos ? p : p.substr(s + 1);
}

bool file_exists(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0;
}

bool parse_u64(const char* s, unsigned long long* out) {
  char* e = nullptr;
  errno = 0;
  *out = std::strtoull(s, &e, 10);
  return e != s && *e == '\0' && !errno;
}

const char* status_name(qpso_status st) {
  switch (st) {
    case QPSO_OK: return "ok";
    case QPSO_ERR_ARG: return "invalid argument or malformed input";
    case QPSO_ERR_NOMEM: return "out of memory";
    case QPSO_ERR_CUDA: return "CUDA error";
    case QPSO_ERR_TIMEOUT: return "device wait timed out";
    case QPSO_ERR_BUSY: return "busy";
    case QPSO_ERR_NOT_FOUND: return "not found";
    default: return "internal error";
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) return usage(argv[0]);
  const std::string obj_path = argv[1], rgb_path = argv[2], depth_path = argv[3];
  unsigned long long idx_u;
  if (!parse_u64(argv[4], &idx_u) || idx_u > 65535) return die("cluster_idx", argv[4]);
  const int32_t idx = (int32_t)idx_u;

  std::string labels_path = depth_path + ".labels.png", results = "results";
  unsigned long long particles = 0, iterations = 0, seed = 0, stream = 0, device = 0;
  bool have_seed = false, have_stream = false, labels_given = false;
  int raster_mode = 0;
  // the reference's compiled-in ACCV intrinsics (main.h:30-33)
  // default: the reference's own projection (its compiled-in ACCV
  // intrinsics in double); --camera gives fp32 intrinsics instead
  qpso_camera cam = {572.41140f, 573.57043f, 325.26110f, 242.04899f, 0, 0, QPSO_PROJ_REF_ACCV};
  for (int i = 5; i < argc; ++i) {
    const std::string a = argv[i];
    if (i + 1 >= argc) return die("missing value for", a);
    const char* v = argv[++i];
    bool ok = true;
    if (a == "--labels") labels_path = v, labels_given = true;
    else if (a == "--results") results = v;
    else if (a == "--particles") ok = parse_u64(v, &particles) && particles > 0;
    else if (a == "--iterations") ok = parse_u64(v, &iterations) && iterations > 0;
    else if (a == "--seed") ok = have_seed = parse_u64(v, &seed);
    else if (a == "--stream") ok = have_stream = parse_u64(v, &stream);
    else if (a == "--device") ok = parse_u64(v, &device);
    else if (a == "--camera") {
      ok = std::sscanf(v, "%f,%f,%f,%f", &cam.fx, &cam.fy, &cam.cx, &cam.cy) == 4;
      cam.projection = QPSO_PROJ_FP32;
    }
    else if (a == "--raster-mode") ok = (raster_mode = std::string(v) == "edge" ? 1 : std::string(v) == "ref" ? 0 : -1) >= 0;
    else return die("unknown option", a);
    if (!ok) return die("bad value", a + " " + v);
  }

  // ---- inputs (host) ----
  uint32_t F = 0;
  qpso_status st = qpso_obj_load(obj_path.c_str(), nullptr, 0, &F);
  if (st != QPSO_OK) return die(obj_path.c_str(), status_name(st));
  std::vector<float> soa(9 * (size_t)F);
  if ((st = qpso_obj_load(obj_path.c_str(), soa.data(), F, &F)) != QPSO_OK)
    return die(obj_path.c_str(), status_name(st));
  std::printf("NumVerts: %u\nNumFaces: %u\n", 3 * F, F);

  uint32_t W = 0, H = 0;
  if ((st = qpso_image_u16_load(depth_path.c_str(), nullptr, 0, &W, &H)) != QPSO_OK)
    return die(depth_path.c_str(), status_name(st));
  std::vector<uint16_t> depth((size_t)W * H);
  if ((st = qpso_image_u16_load(depth_path.c_str(), depth.data(), depth.size(), &W, &H)) != QPSO_OK)
    return die(depth_path.c_str(), status_name(st));
  const bool use_labels = labels_given || file_exists(labels_path);
  std::vector<int32_t> labels((size_t)W * H);
  cam.width = (int32_t)W;
  cam.height = (int32_t)H;
  if (use_labels) {
    uint32_t lw = 0, lh = 0;
    std::vector<uint16_t> lab16((size_t)W * H);
    if ((st = qpso_image_u16_load(labels_path.c_str(), lab16.data(), lab16.size(), &lw, &lh)) != QPSO_OK)
      return die(labels_path.c_str(), status_name(st));
    if (lw != W || lh != H) return die(labels_path.c_str(), "size differs from the depth image");
    for (size_t i = 0; i < lab16.size(); ++i) labels[i] = (int32_t)lab16[i] - 1;
    std::printf("rgb_file: %s depth_file: %s labels: %s (%ux%u)\n", rgb_path.c_str(), depth_path.c_str(),
                labels_path.c_str(), W, H);
  }
  std::vector<uint8_t> bgr;
  if (!use_labels) {
    // GraphCannySeg<hsv> runs on the colour image and the depth (main.cu:1238-1256)
    uint32_t cw = 0, chh = 0;
    if ((st = qpso_image_bgr8_load(rgb_path.c_str(), nullptr, 0, &cw, &chh)) != QPSO_OK)
      return die(rgb_path.c_str(), status_name(st));
    if (cw != W || chh != H) return die(rgb_path.c_str(), "size differs from the depth image");
    bgr.resize(3 * (size_t)W * H);
    if ((st = qpso_image_bgr8_load(rgb_path.c_str(), bgr.data(), (uint64_t)W * H, &cw, &chh)) != QPSO_OK)
      return die(rgb_path.c_str(), status_name(st));
    std::printf("rgb_file: %s depth_file: %s (%ux%u)\n", rgb_path.c_str(), depth_path.c_str(), W, H);
  }

  // ---- segmentation and solve (GPU) ----
  qpso_context* ctx = nullptr;
  if ((st = qpso_create((int)device, &ctx)) != QPSO_OK) return die("qpso_create", status_name(st));
  auto fail = [&](const char* what) {
    const std::string msg = qpso_last_error(ctx);
    qpso_destroy(ctx);
    return die(what, msg);
  };
  uint32_t mesh_id = 0, frame_id = 0;
  if (qpso_mesh_upload(ctx, soa.data(), F, &mesh_id) != QPSO_OK) return fail("mesh upload");
  int32_t label = idx;
  int32_t box[4];
  uint32_t num_points = 0;
  float centroid[3];
  if (use_labels) {
    uint32_t ncl = 0;
    if (qpso_frame_upload(ctx, depth.data(), labels.data(), &cam, &frame_id) != QPSO_OK)
      return fail("frame upload");
    if (qpso_frame_clusters(ctx, frame_id, nullptr, 0, &ncl) != QPSO_OK) return fail("clusters");
    std::vector<qpso_cluster> cl(ncl);
    if (ncl && qpso_frame_clusters(ctx, frame_id, cl.data(), ncl, &ncl) != QPSO_OK) return fail("clusters");
    const qpso_cluster* c = nullptr;
    for (const auto& x : cl)
      if (x.label == idx) c = &x;
    if (!c) {
      qpso_destroy(ctx);
      return die("cluster_idx", std::to_string(idx) + " is not in the label map (" + std::to_string(ncl) +
                                    " clusters)");
    }
    box[0] = c->min_x, box[1] = c->max_x, box[2] = c->min_y, box[3] = c->max_y;
    // the reference's cluster size is its collectSets list length, which
    // repeats one pixel (GraphCannySeg.cpp:305-352): pixels + 1 reach the
    // fitness as num_point_SegmentedCluster (main.cu:1322)
    num_points = c->num_points + 1;
    std::memcpy(centroid, c->centroid_mm, sizeof(centroid));
  } else {
    qpso_seg_params prm;
    qpso_seg_params_init(&prm);
    qpso_seg_front_params fp;
    qpso_seg_front_params_init(&fp);
    std::vector<uint16_t> inpainted((size_t)W * H);
    qpso_seg_frame_out planes;
    std::memset(&planes, 0, sizeof(planes));
    planes.inpainted = inpainted.data();
    const uint32_t cap = W * H / 64 + 16;
    std::vector<qpso_seg_cluster> cl(cap);
    uint32_t n_sets = 0, n_cl = 0;
    if (qpso_segment_rgbd(ctx, bgr.data(), depth.data(), W, H, &prm, &fp, labels.data(), &n_sets, cl.data(), cap,
                          &n_cl, &planes) != QPSO_OK)
      return fail("segmentation");
    std::printf("disjoint sets %u\nclusters kept %u\n", n_sets, n_cl);
    // the reference's cluster images (main.cu:1257-1272): the colour image
    // inside each kept cluster, black elsewhere, as results/<rgb>-cluster<i>.jpg,
    // and cluster N once more as cluster.jpg in the working directory
    if (::mkdir(results.c_str(), 0755) != 0 && errno != EEXIST) {
      qpso_destroy(ctx);
      return die("mkdir", results);
    }
    std::vector<uint8_t> img((size_t)W * H * 3);
    for (uint32_t i = 0; i < n_cl && i < cap; ++i) {
      std::fill(img.begin(), img.end(), (uint8_t)0);
      for (size_t p = 0; p < (size_t)W * H; ++p)
        if (labels[p] == cl[i].label)
          for (int c = 0; c < 3; ++c) img[3 * p + c] = bgr[3 * p + c];
      const std::string name = results + "/" + base_name(rgb_path) + "-cluster" + std::to_string(i) + ".jpg";
      if (qpso_image_jpeg_write(name.c_str(), img.data(), W, H, 95) != QPSO_OK) {
        qpso_destroy(ctx);
        return die("cannot write", name);
      }
      if ((int32_t)i == idx && qpso_image_jpeg_write("cluster.jpg", img.data(), W, H, 95) != QPSO_OK) {
        qpso_destroy(ctx);
        return die("cannot write", "cluster.jpg");
      }
    }
    if ((uint32_t)idx >= n_cl || idx >= (int32_t)cap) {
      qpso_destroy(ctx);
      return die("cluster_idx", std::to_string(idx) + " is beyond the " + std::to_string(n_cl) +
                                    " clusters the segmentation kept");
    }
    const qpso_seg_cluster& c = cl[idx];
    label = c.label;
    box[0] = c.min_x, box[1] = c.max_x, box[2] = c.min_y, box[3] = c.max_y;
    num_points = c.num_points;  // already the list length (pixels + 1)
    std::memcpy(centroid, c.centroid_mm, sizeof(centroid));
    // the observed depth is the cluster-masked inpainted depth (SegResults.clusterDepth,
    // GraphCannySeg.h:1808-1809; main.cu:1548-1557)
    if (qpso_frame_upload(ctx, inpainted.data(), labels.data(), &cam, &frame_id) != QPSO_OK)
      return fail("frame upload");
  }
  std::printf("centroid IDX_cluster: %d [%g, %g, %g]\n------\n", idx, centroid[0], centroid[1], centroid[2]);

  qpso_solve_desc d;
  qpso_solve_desc_init(&d);
  d.mesh_id = mesh_id;
  d.frame_id = frame_id;
  d.cluster_label = label;
  d.cl_min_x = box[0];
  d.cl_max_x = box[1];
  d.cl_min_y = box[2];
  d.cl_max_y = box[3];
  d.num_points = num_points;
  qpso_box_from_centroid(centroid, 0.3f, 0.3f, d.t_lo, d.t_hi);  // main.cu:1285-1323
  if (particles) d.num_particles = (uint32_t)particles;
  if (iterations) d.iterations = (uint32_t)iterations;
  if (have_seed) d.seed = seed;
  if (have_stream) d.stream = (uint32_t)stream;
  d.raster_mode = raster_mode == 1 ? QPSO_RASTER_EDGE : QPSO_RASTER_REF;
  qpso_result r;
  if (qpso_solve(ctx, &d, &r) != QPSO_OK) return fail("solve");
  std::printf("Solution Best Pose: %f %f %f %f %f %f %f\nSolution Best Fit: %f\n", r.pose[0], r.pose[1],
              r.pose[2], r.pose[3], r.pose[4], r.pose[5], r.pose[6], r.fit);

  // ---- outputs ----
  if (::mkdir(results.c_str(), 0755) != 0 && errno != EEXIST) {
    qpso_destroy(ctx);
    return die("mkdir", results);
  }
  const std::string stem = results + "/" + base_name(rgb_path) + "-" + std::to_string(idx);
  FILE* out = std::fopen((stem + "-bestpose.csv").c_str(), "w");
  if (!out) {
    qpso_destroy(ctx);
    return die("cannot write", stem + "-bestpose.csv");
  }
  std::fprintf(out, "%f,%f,%f,%f,%f,%f,%f,%f", r.fit, r.pose[0], r.pose[1], r.pose[2], r.pose[3], r.pose[4],
               r.pose[5], r.pose[6]);
  std::fclose(out);

  std::vector<float> img((size_t)W * H);
  if (qpso_render_depth_f32(ctx, mesh_id, &cam, r.pose, img.data()) != QPSO_OK) return fail("render");
  std::printf("Rendering the Best Pose in %s-best.csv\n", stem.c_str());
  out = std::fopen((stem + "-best.csv").c_str(), "w");
  if (!out) {
    qpso_destroy(ctx);
    return die("cannot write", stem + "-best.csv");
  }
  // saveBestParticleRender2MatlabCSV (main.h:1994-2010): ostream << float
  // (6 significant digits), ", " between columns, a newline per row
  for (uint32_t y = 0; y < H; ++y) {
    for (uint32_t x = 0; x < W; ++x)
      std::fprintf(out, x + 1 < W ? "%g, " : "%g", (double)img[(size_t)y * W + x]);
    std::fputc('\n', out);
  }
  std::fclose(out);
  qpso_destroy(ctx);
  return r.flags == 0 ? 0 : 2;
}
