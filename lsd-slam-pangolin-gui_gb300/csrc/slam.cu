// slam.cu -- host-only: the full monocular SLAM loop over the GPU hot path (config 4 of the
// workloads: a 1,000-frame sequence).
//
// Upstream this is lsd-slam's SlamSystem (absent from the reference tree; the reference feeds it from
// InputThread, lib/App/InputThread.cpp:71 `system->nextImage(runningIdx, imageUndist, camera)`, and
// finalises it at the end, tools/LSD.cpp:139; results leave through OutputIOWrapper:
// PangolinOutputIOWrapper::publishKeyframeGraph, lib/Pangolin_IOWrapper/PangolinOutputIOWrapper.cpp:148-168,
// and TextOutputIOWrapper::publishTrackedFrame, lib/Pangolin_IOWrapper/TextOutputIOWrapper.cpp:100-120).
// Upstream runs three threads around the hot path; this loop keeps that division of work:
//   * tracking (the caller's thread, lsdg_slam_next_image): every frame is aligned to the current
//     keyframe (SE3Tracker::trackFrame, constant-velocity initial guess);
//   * mapping (same thread, after tracking): the frame updates the keyframe's depth
//     (DepthMap::updateKeyframe, 8-bit frame; the epipolar line's position variance raised to cover
//     the tracked pose's error), the tracking reference is refreshed from the smoothed depth (after
//     every frame by default), and after kf_dist metres of travel, a kf_angle turn, or when fewer than
//     kf_min_usage of the keyframe's points stay in view, the frame becomes the new keyframe
//     (DepthMap::createKeyFrame: propagation + regularisation);
//   * keyframe refinement (caller's thread, when the current keyframe is left): its frames tracked
//     again against its refined depth and mapped again from its starting depth with the new poses,
//     a few rounds;
//   * re-positioning (caller's thread, before a keyframe would be made): the earlier keyframes whose
//     camera is near the current one in the graph are tracked against the frame; one that keeps most
//     of its points in view at a pose close to the graph's prediction becomes the current keyframe
//     again (its depth map is refined further) and the keyframe left is tied to it in the graph;
//   * constraint search (a worker thread with a context of its own): each new keyframe is aligned
//     with Sim3Tracker::trackFrameSim3 to its parent and the nearest earlier keyframes in one
//     batched launch from device-resident keyframes -- in both directions, a constraint being kept
//     only when the two alignments agree -- and the Sim3 pose graph is optimised every few loop
//     constraints (and after each re-positioning's loop edge).  The worker runs while tracking and
//     mapping go on; it is joined before the graph is read or changed on the caller's thread (a
//     keyframe decision, the outputs), so the results do not depend on thread timing.
// The first keyframe's depth is given (lsdg_slam_bootstrap); upstream starts from a random map.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "lsdg.h"
#include "slam_math.h"

using lsdg::slam::M4;

namespace {

struct Keyframe {
  int frame_index = 0;
  int node = 0;
  int parent = -1;                 // the keyframe it was made from (tracked against, propagated from)
  lsdg_frame* frame = nullptr;     // tracking reference (refreshed while it is the current keyframe)
  lsdg_frame* snapshot = nullptr;  // its state at creation, read by the constraint search of its own job
};

struct FramePose {
  int keyframe;  // index into keyframes
  M4 f2k;        // frame-to-keyframe
};

}  // namespace

struct lsdg_slam {
  lsdg_params params{};
  lsdg_slam_params sp{};
  int w = 0, h = 0;
  lsdg_intrinsics intr{};
  lsdg_ctx* ctx = nullptr;       // tracking and mapping
  lsdg_ctx* ctx_cons = nullptr;  // constraint search (worker thread)
  lsdg_depthmap* dm = nullptr;
  lsdg_frame* pool[2] = {nullptr, nullptr};
  int pool_next = 0;
  std::vector<Keyframe> keyframes;
  std::vector<FramePose> traj;
  std::vector<int> traj_id;  // the caller's frame ids
  lsdg::slam::PoseGraph graph;
  std::map<int, lsdg_batch*> batches;  // Sim3 batches by size (worker context)
  std::thread worker;
  bool worker_running = false;
  lsdg_status worker_status = LSDG_OK;
  std::string worker_error;
  int since_refresh = 0;
  int loops_pending = 0;
  int cur = 0;                 // the current keyframe (tracked against, mapped)
  // the current keyframe's refinement state: its image and depth when it became current, and the
  // frames mapped into it since (8-bit images back to back, and their trajectory indices)
  std::vector<float> kf_image, kf_init_d, kf_init_v;
  std::vector<uint8_t> hist_images;
  std::vector<long> hist_traj;
  // the refinement's re-tracking runs as one batch of kRefineBatch pairs (frames uploaded into
  // hist_frames), created on first use
  std::vector<lsdg_frame*> hist_frames;
  lsdg_batch* refine_batch = nullptr;
  lsdg_slam_stats stats{};
  lsdg_slam_stats wstats{};  // counted by the worker's jobs, added to stats when the worker is joined
  std::vector<float> d_buf, v_buf;
  std::vector<int32_t> val_buf;
  std::string err;
};

namespace {

// The worker thread records its errors in the system's worker_error, the caller's thread in err.
thread_local std::string* t_err = nullptr;

lsdg_status fail(lsdg_slam* s, lsdg_status st, const char* what, const lsdg_ctx* c = nullptr) {
  if (s) {
    std::string& e = t_err ? *t_err : s->err;
    e = what;
    if (c) {
      e += ": ";
      e += lsdg_last_error(c);
    }
  }
  return st;
}

#define SLAM_CK(s, expr, ctx)                              \
  do {                                                     \
    const lsdg_status st_ = (expr);                        \
    if (st_ != LSDG_OK) return fail((s), st_, #expr, ctx); \
  } while (0)

double norm3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

double rotation_angle(const M4& T) {
  const double s = lsdg::slam::sim3_scale(T);
  double R[9], w[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = T(i, j) / s;
  lsdg::slam::so3_log(R, w);
  return norm3(w);
}

bool finite(const M4& T) {
  for (double v : T.a)
    if (!std::isfinite(v)) return false;
  return true;
}

// The depth map's smoothed inverse depth and variance (the planes the viewer reads) into a frame.
// With ref_min_validity > 0, hypotheses observed fewer times than that stay out, and with
// ref_max_var > 0 those less certain than that (neither applies to the bootstrap keyframe).
lsdg_status reference_depth(lsdg_slam* s, lsdg_frame* f) {
  const bool gate = s->sp.ref_min_validity > 0 && !s->keyframes.empty();
  SLAM_CK(s, lsdg_depth_get(s->ctx, s->dm, nullptr, nullptr, s->d_buf.data(), s->v_buf.data(),
                            gate ? s->val_buf.data() : nullptr, nullptr), s->ctx);
  if (gate)
    for (size_t i = 0; i < s->d_buf.size(); ++i)
      if (s->val_buf[i] < s->sp.ref_min_validity) s->d_buf[i] = -1.0f;
  if (s->sp.ref_max_var > 0.0f && !s->keyframes.empty())
    for (size_t i = 0; i < s->d_buf.size(); ++i)
      if (!(s->v_buf[i] < s->sp.ref_max_var)) s->d_buf[i] = -1.0f;
  SLAM_CK(s, lsdg_frame_set_depth(s->ctx, f, s->d_buf.data(), s->v_buf.data()), s->ctx);
  return LSDG_OK;
}

lsdg_status new_frame_with_depth(lsdg_slam* s, const uint8_t* image, lsdg_frame** out) {
  *out = nullptr;
  SLAM_CK(s, lsdg_frame_create(s->ctx, s->w, s->h, &s->intr, out), s->ctx);
  SLAM_CK(s, lsdg_frame_upload_u8(s->ctx, *out, image), s->ctx);
  return reference_depth(s, *out);
}

void hess_full(const lsdg_track_stats& st, int n, double* H) {  // upper triangle -> n x n
  int q = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      H[n * i + j] = H[n * j + i] = st.hessian[q];
      ++q;
    }
}

// ------------------------------------------------------------------------------------------
// Constraint search of keyframe `k` (worker thread: its own context, the graph is its own until
// joined)
// ------------------------------------------------------------------------------------------
struct Cand {
  double dist;
  int kf;
};

lsdg_status constraint_job(lsdg_slam* s, int k) {
  lsdg_ctx* ctx = s->ctx_cons;
  const Keyframe& kn = s->keyframes[k];
  const int parent = kn.parent;
  const M4 T_new = s->graph.poses[kn.node];
  std::vector<Cand> others;
  for (int c = 0; c < k; ++c) {
    if (c == parent) continue;
    const M4& Tc = s->graph.poses[s->keyframes[c].node];
    const double d[3] = {Tc(0, 3) - T_new(0, 3), Tc(1, 3) - T_new(1, 3), Tc(2, 3) - T_new(2, 3)};
    const double dist = norm3(d);
    if (dist < s->sp.cand_radius) others.push_back({dist, c});
  }
  std::stable_sort(others.begin(), others.end(), [](const Cand& a, const Cand& b) { return a.dist < b.dist; });
  std::vector<int> cands = {parent};
  for (const Cand& c : others) {
    if ((int)cands.size() >= s->sp.n_candidates) break;
    cands.push_back(c.kf);
  }
  const int nc = (int)cands.size();
  const bool both = s->sp.both_directions != 0;
  // one batch size for every job (the unused pairs repeat pair 0 and are not read): a batch is tuned
  // and captured once, instead of once per candidate count
  const int ncap = std::max(nc, std::max(1, s->sp.n_candidates));
  const int nb = both ? 2 * ncap : ncap;
  lsdg_batch*& b = s->batches[nb];
  if (!b) {
    std::vector<int> ws(nb, s->w), hs(nb, s->h);
    std::vector<lsdg_intrinsics> ks(nb, s->intr);
    SLAM_CK(s, lsdg_batch_create_sim3(ctx, nb, ws.data(), hs.data(), ks.data(), &b), ctx);
  }
  // pair i < ncap: the new keyframe tracked against candidate i (frame-to-ref = new-in-candidate);
  // pair ncap + i: the candidate tracked against the new keyframe
  std::vector<const lsdg_frame*> refs(nb), frames(nb);
  std::vector<double> init(13 * (size_t)nb);
  std::vector<M4> Zinit(nc);
  for (int i = 0; i < ncap; ++i) {
    const int ci = i < nc ? i : 0;
    const Keyframe& c = s->keyframes[cands[ci]];
    if (i < nc) Zinit[i] = lsdg::slam::mul(lsdg::slam::sim3_inv(s->graph.poses[c.node]), T_new);
    refs[i] = c.frame;
    frames[i] = kn.snapshot;
    lsdg::slam::to13(Zinit[ci], &init[13 * i]);
    if (both) {
      refs[ncap + i] = kn.snapshot;
      frames[ncap + i] = c.frame;
      lsdg::slam::to13(lsdg::slam::sim3_inv(Zinit[ci]), &init[13 * (ncap + i)]);
    }
  }
  SLAM_CK(s, lsdg_batch_load_frames(ctx, b, refs.data(), frames.data(), init.data()), ctx);
  SLAM_CK(s, lsdg_batch_run(ctx, b), ctx);
  std::vector<double> out(13 * (size_t)nb);
  std::vector<lsdg_track_stats> st(nb);
  SLAM_CK(s, lsdg_batch_read(ctx, b, out.data(), st.data()), ctx);
  bool loop = false;
  for (int i = 0; i < nc; ++i) {
    const double* o = &out[13 * i];
    bool ok = st[i].status == LSDG_OK && std::isfinite(o[12]) && o[12] > 0.5 && o[12] < 2.0;
    M4 Z = M4::identity();
    if (ok) {
      Z = lsdg::slam::from13(o);
      ok = finite(Z);
    }
    if (ok) {  // the result stays near the graph's prediction
      double dz[7];
      lsdg::slam::sim3_log(lsdg::slam::mul(lsdg::slam::sim3_inv(Zinit[i]), Z), dz);
      const double tz[3] = {Z(0, 3), Z(1, 3), Z(2, 3)};
      ok = norm3(dz) < 0.25 * std::max(1.0, norm3(tz)) && norm3(dz + 3) < 0.15 && std::fabs(dz[6]) < 0.1;
    }
    if (ok && both) {  // the reverse alignment agrees: Z_fwd Z_rev ~ identity
      const double* orv = &out[13 * (ncap + i)];
      ok = st[ncap + i].status == LSDG_OK && std::isfinite(orv[12]) && orv[12] > 0.0;
      if (ok) {
        double e[7];
        lsdg::slam::sim3_log(lsdg::slam::mul(Z, lsdg::slam::from13(orv)), e);
        const double tz[3] = {Z(0, 3), Z(1, 3), Z(2, 3)};
        ok = std::isfinite(e[0]) && norm3(e) < s->sp.consistency_trans * std::max(0.1, norm3(tz)) &&
             norm3(e + 3) < s->sp.consistency_rot && std::fabs(e[6]) < s->sp.consistency_scale;
      }
    }
    double H[49];
    if (ok) {
      hess_full(st[i], 7, H);
      for (double v : H) ok = ok && std::isfinite(v);
    }
    if (!ok) {
      s->wstats.sim3_rejected++;
      continue;
    }
    for (double& v : H) v *= s->sp.sim3_info_scale;
    s->graph.add_edge(s->keyframes[cands[i]].node, kn.node, Z, H);
    s->wstats.sim3_edges++;
    loop = loop || cands[i] != parent;
  }
  if (loop && ++s->loops_pending >= s->sp.optimize_every) {
    const std::vector<M4> keep = s->graph.poses;
    s->graph.optimize(5);
    bool good = true;
    for (const M4& T : s->graph.poses) good = good && finite(T);
    if (!good) s->graph.poses = keep;
    s->loops_pending = 0;
    s->wstats.graph_optimisations++;
  }
  return LSDG_OK;
}

void merge_worker_stats(lsdg_slam* s) {
  s->stats.sim3_edges += s->wstats.sim3_edges;
  s->stats.sim3_rejected += s->wstats.sim3_rejected;
  s->stats.graph_optimisations += s->wstats.graph_optimisations;
  s->wstats = lsdg_slam_stats{};
}

lsdg_status join_worker(lsdg_slam* s) {
  if (s->worker_running) {
    s->worker.join();
    s->worker_running = false;
    merge_worker_stats(s);
    // the new keyframe's snapshot was read by its own job only
    Keyframe& k = s->keyframes.back();
    if (k.snapshot) {
      lsdg_frame_destroy(s->ctx, k.snapshot);
      k.snapshot = nullptr;
    }
  }
  if (s->worker_status != LSDG_OK) {
    s->err = "constraint search: " + s->worker_error;
    return s->worker_status;
  }
  return LSDG_OK;
}

void optimize_graph(lsdg_slam* s, int iterations);

// The worker's next job: the constraint search of keyframe k (k >= 0), or, for k < 0, a few pose-graph
// iterations after a loop edge (re-positioning).  Inline when async_constraints is 0.
lsdg_status start_job(lsdg_slam* s, int k) {
  auto body = [s, k]() {
    std::string* keep = t_err;
    t_err = &s->worker_error;
    lsdg_status st = LSDG_OK;
    if (k >= 0) st = constraint_job(s, k);
    else optimize_graph(s, 5);
    if (st != LSDG_OK) s->worker_status = st;
    t_err = keep;
  };
  if (s->sp.async_constraints) {
    try {
      s->worker = std::thread(body);
    } catch (...) {
      return fail(s, LSDG_OUT_OF_MEMORY, "could not start the constraint-search thread");
    }
    s->worker_running = true;
    return LSDG_OK;
  }
  body();
  merge_worker_stats(s);
  if (k >= 0) {
    Keyframe& kn = s->keyframes[k];
    if (kn.snapshot) {
      lsdg_frame_destroy(s->ctx, kn.snapshot);
      kn.snapshot = nullptr;
    }
  }
  if (s->worker_status != LSDG_OK) {
    s->err = "constraint search: " + s->worker_error;
    return s->worker_status;
  }
  return LSDG_OK;
}

// SE3 part {R, t} of a Sim3 [[s R, t], [0, 1]].
M4 se3_part(const M4& S) {
  const double sc = lsdg::slam::sim3_scale(S);
  M4 T = S;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) T(r, c) = S(r, c) / sc;
  return T;
}

// SE3 information of a tracking result as a 7x7 graph information (scale tied by a prior as strong
// as the strongest direction times odometry_scale_weight); false when the Hessian is not usable.
bool se3_information(const lsdg_slam* s, const lsdg_track_stats& st, double W[49]) {
  double H6[36];
  hess_full(st, 6, H6);
  bool ok = true;
  double dmax = 0.0;
  for (int i = 0; i < 36; ++i) ok = ok && std::isfinite(H6[i]);
  for (int i = 0; i < 6; ++i) dmax = std::max(dmax, H6[7 * i]);
  if (!ok || !(dmax > 0)) return false;
  std::memset(W, 0, sizeof(double) * 49);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) W[7 * i + j] = H6[6 * i + j] * 1e-3;
  W[48] = dmax * 1e-3 * s->sp.odometry_scale_weight;
  return true;
}

// A few pose-graph iterations (worker thread), kept only when every pose stays finite.
void optimize_graph(lsdg_slam* s, int iterations) {
  const std::vector<M4> keep = s->graph.poses;
  s->graph.optimize(iterations);
  bool good = true;
  for (const M4& T : s->graph.poses) good = good && finite(T);
  if (!good) s->graph.poses = keep;
  s->wstats.graph_optimisations++;
}

// The state a keyframe's refinement starts from when it becomes current: its image (float) and the
// depth it starts with; no frames mapped yet.
void begin_keyframe_state(lsdg_slam* s, const float* image, const float* d, const float* v) {
  const size_t npix = (size_t)s->w * s->h;
  s->kf_image.assign(image, image + npix);
  s->kf_init_d.assign(d, d + npix);
  s->kf_init_v.assign(v, v + npix);
  s->hist_images.clear();
  s->hist_traj.clear();
}

// Refinement of the current keyframe before it is left (a block-coordinate pass over its window of
// frames): every frame mapped into it is tracked again against its refined depth (from the pose it
// had), then the depth map restarts from the keyframe's starting depth and maps the frames again with
// the new poses, and the tracking reference takes the result; retrack_iterations rounds.  Tracking
// and mapping feed each other inside one keyframe (a small error of the tracked translation tilts
// the map triangulated from it, and the tilted map biases the next tracked poses); re-estimating the
// window's poses against the map its own frames built, and the map from those poses, damps that.
// The re-tracking of a round is one batched launch; poses that do not track again keep their value.
constexpr int kRefineBatch = 16;
constexpr int kMaxWindow = 32;  // frames a keyframe's refinement keeps (the most recent)

lsdg_status refine_keyframe(lsdg_slam* s) {
  const int nh = (int)s->hist_traj.size();
  if (s->sp.retrack_iterations <= 0 || nh < 2) return LSDG_OK;
  const size_t npix = (size_t)s->w * s->h;
  std::vector<double> k2f12(12 * (size_t)nh);
  // the window's frames on the device, and the batch that re-tracks up to kRefineBatch at once
  while ((int)s->hist_frames.size() < std::min(nh, kRefineBatch)) {
    lsdg_frame* f = nullptr;
    SLAM_CK(s, lsdg_frame_create(s->ctx, s->w, s->h, &s->intr, &f), s->ctx);
    s->hist_frames.push_back(f);
  }
  if (!s->refine_batch) {
    std::vector<int> ws(kRefineBatch, s->w), hs(kRefineBatch, s->h);
    std::vector<lsdg_intrinsics> ks(kRefineBatch, s->intr);
    SLAM_CK(s, lsdg_batch_create(s->ctx, kRefineBatch, ws.data(), hs.data(), ks.data(), &s->refine_batch), s->ctx);
  }
  std::vector<const lsdg_frame*> refs(kRefineBatch, s->keyframes[s->cur].frame), frames(kRefineBatch);
  std::vector<double> init(12 * (size_t)kRefineBatch), out(12 * (size_t)kRefineBatch);
  std::vector<lsdg_track_stats> st(kRefineBatch);
  for (int it = 0; it < s->sp.retrack_iterations; ++it) {
    for (int c0 = 0; c0 < nh; c0 += kRefineBatch) {
      const int nc = std::min(kRefineBatch, nh - c0);
      for (int i = 0; i < kRefineBatch; ++i) {
        const int h = c0 + (i < nc ? i : 0);  // unused pairs repeat the chunk's first and are not read
        if (it == 0 || nh > kRefineBatch)
          if (i < nc) SLAM_CK(s, lsdg_frame_upload_u8(s->ctx, s->hist_frames[i], &s->hist_images[npix * h]), s->ctx);
        frames[i] = s->hist_frames[i < nc ? i : 0];
        lsdg::slam::to12(s->traj[s->hist_traj[h]].f2k, &init[12 * i]);
      }
      SLAM_CK(s, lsdg_batch_load_frames(s->ctx, s->refine_batch, refs.data(), frames.data(), init.data()), s->ctx);
      SLAM_CK(s, lsdg_batch_run(s->ctx, s->refine_batch), s->ctx);
      SLAM_CK(s, lsdg_batch_read(s->ctx, s->refine_batch, out.data(), st.data()), s->ctx);
      for (int i = 0; i < nc; ++i) {
        M4& pose = s->traj[s->hist_traj[c0 + i]].f2k;
        const M4 p2 = lsdg::slam::from12(&out[12 * i]);
        const double d[3] = {p2(0, 3) - pose(0, 3), p2(1, 3) - pose(1, 3), p2(2, 3) - pose(2, 3)};
        if (st[i].status == LSDG_OK && finite(p2) && norm3(d) <= 0.25 * s->sp.max_track_jump) pose = p2;
      }
    }
    SLAM_CK(s, lsdg_depth_set_keyframe(s->ctx, s->dm, s->kf_image.data(), s->kf_init_d.data(), s->kf_init_v.data()),
            s->ctx);
    for (int i = 0; i < nh; ++i) lsdg::slam::to12(lsdg::slam::sim3_inv(s->traj[s->hist_traj[i]].f2k), &k2f12[12 * i]);
    for (int c0 = 0; c0 < nh; c0 += LSDG_MAX_REFS) {
      const int nc = std::min(LSDG_MAX_REFS, nh - c0);
      SLAM_CK(s, lsdg_depth_update_u8(s->ctx, s->dm, nc, &s->hist_images[npix * c0], &k2f12[12 * c0], 1), s->ctx);
    }
    lsdg_status r = reference_depth(s, s->keyframes[s->cur].frame);
    if (r != LSDG_OK) return r;
  }
  return LSDG_OK;
}

// Re-positioning before a new keyframe (SlamSystem's re-activation of an earlier keyframe): the
// earlier keyframes whose camera lies within react_radius and react_angle_deg of the current camera
// in the graph are tracked against `frame` (nearest first, at most three); the first that keeps
// react_min_usage of its points in view with react_min_good of them inliers, at a pose within
// react_max_jump of the graph's prediction and within half of kf_dist / kf_angle_deg of the keyframe
// (so that the keyframe is not left again at the next frame), becomes the current keyframe again.
// *done: whether one did.
lsdg_status try_reactivate(lsdg_slam* s, lsdg_frame* frame, const M4& f2k, bool* done) {
  *done = false;
  lsdg_status r = join_worker(s);  // the graph is the caller's again
  if (r != LSDG_OK) return r;
  const int n_kf = (int)s->keyframes.size();
  const M4 T_cur = lsdg::slam::mul(s->graph.poses[s->keyframes[s->cur].node], f2k);
  std::vector<Cand> cands;
  for (int c = 0; c < n_kf - s->sp.react_min_age; ++c) {
    if (c == s->cur) continue;
    const M4& Tc = s->graph.poses[s->keyframes[c].node];
    const double d[3] = {Tc(0, 3) - T_cur(0, 3), Tc(1, 3) - T_cur(1, 3), Tc(2, 3) - T_cur(2, 3)};
    const double dist = norm3(d);
    if (dist > s->sp.react_radius) continue;
    if (rotation_angle(se3_part(lsdg::slam::mul(lsdg::slam::sim3_inv(Tc), T_cur))) >
        s->sp.react_angle_deg * M_PI / 180.0)
      continue;
    cands.push_back({dist, c});
  }
  std::stable_sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.dist < b.dist; });
  for (size_t i = 0; i < cands.size() && i < 3; ++i) {
    const int c = cands[i].kf;
    const M4 guess = se3_part(lsdg::slam::mul(lsdg::slam::sim3_inv(s->graph.poses[s->keyframes[c].node]), T_cur));
    double g12[12], o12[12];
    lsdg::slam::to12(guess, g12);
    lsdg_track_stats st{};
    const lsdg_status ts = lsdg_track_se3(s->ctx, s->keyframes[c].frame, frame, g12, o12, &st);
    if (ts != LSDG_OK && ts != LSDG_TRACKING_LOST) return fail(s, ts, "lsdg_track_se3 (re-positioning)", s->ctx);
    const M4 f2c = lsdg::slam::from12(o12);
    const double jump[3] = {f2c(0, 3) - guess(0, 3), f2c(1, 3) - guess(1, 3), f2c(2, 3) - guess(2, 3)};
    double W[49];
    const double tc[3] = {f2c(0, 3), f2c(1, 3), f2c(2, 3)};
    if (st.status != LSDG_OK || !finite(f2c) || st.usage < s->sp.react_min_usage ||
        st.good_ratio < s->sp.react_min_good || norm3(jump) > s->sp.react_max_jump ||
        norm3(tc) > 0.5 * s->sp.kf_dist || rotation_angle(f2c) > 0.5 * s->sp.kf_angle_deg * M_PI / 180.0 ||
        !se3_information(s, st, W))
      continue;
    // loop edge: the keyframe left, seen from the re-activated one -- a Sim3 alignment of the two
    // keyframes (both carry depth, so their relative scale is measured) started from the pose through
    // this frame; when that alignment fails, the SE3 pose through this frame with its scale prior
    const M4 z_frame = lsdg::slam::mul(f2c, lsdg::slam::sim3_inv(f2k));
    double z13[13], zo13[13];
    lsdg::slam::to13(z_frame, z13);
    lsdg_track_stats s7{};
    const lsdg_status ts7 =
        lsdg_track_sim3(s->ctx, s->keyframes[c].frame, s->keyframes[s->cur].frame, z13, zo13, &s7);
    if (ts7 != LSDG_OK && ts7 != LSDG_TRACKING_LOST) return fail(s, ts7, "lsdg_track_sim3 (re-positioning)", s->ctx);
    bool sim3_ok = s7.status == LSDG_OK && std::isfinite(zo13[12]) && zo13[12] > 0.5 && zo13[12] < 2.0;
    M4 z = z_frame;
    double H7[49];
    if (sim3_ok) {
      z = lsdg::slam::from13(zo13);
      double dz[7];
      lsdg::slam::sim3_log(lsdg::slam::mul(lsdg::slam::sim3_inv(z_frame), z), dz);
      const double tz[3] = {z(0, 3), z(1, 3), z(2, 3)};
      sim3_ok = finite(z) && norm3(dz) < 0.25 * std::max(1.0, norm3(tz)) && norm3(dz + 3) < 0.15 &&
                std::fabs(dz[6]) < 0.3;
      hess_full(s7, 7, H7);
      for (double v : H7) sim3_ok = sim3_ok && std::isfinite(v);
    }
    if (sim3_ok) {
      for (double& v : H7) v *= s->sp.sim3_info_scale;
      s->graph.add_edge(s->keyframes[c].node, s->keyframes[s->cur].node, z, H7);
    } else {
      s->graph.add_edge(s->keyframes[c].node, s->keyframes[s->cur].node, z_frame, W);
    }
    // the depth map takes the re-activated keyframe's state back (image and smoothed depth)
    const size_t npix = (size_t)s->w * s->h;
    std::vector<float> lvl(4 * npix), img(npix);  // level 0 comes back as {I, gx, gy, 0} per pixel
    SLAM_CK(s, lsdg_frame_get_level(s->ctx, s->keyframes[c].frame, 0, lvl.data()), s->ctx);
    for (size_t i = 0; i < npix; ++i) img[i] = lvl[4 * i];
    SLAM_CK(s, lsdg_frame_get_depth(s->ctx, s->keyframes[c].frame, 0, s->d_buf.data(), s->v_buf.data()), s->ctx);
    SLAM_CK(s, lsdg_depth_set_keyframe(s->ctx, s->dm, img.data(), s->d_buf.data(), s->v_buf.data()), s->ctx);
    begin_keyframe_state(s, img.data(), s->d_buf.data(), s->v_buf.data());
    s->cur = c;
    s->traj.back() = {c, f2c};
    s->since_refresh = 0;
    s->stats.reactivations++;
    *done = true;
    return start_job(s, -1);  // the graph takes the loop edge in on the worker thread
  }
  return LSDG_OK;
}

lsdg_status new_keyframe(lsdg_slam* s, int frame_index, const uint8_t* image, const M4& f2k,
                         const lsdg_track_stats& st) {
  lsdg_status r = join_worker(s);  // the graph is the caller's again
  if (r != LSDG_OK) return r;
  const M4 k2f = lsdg::slam::sim3_inv(f2k);
  double k2f12[12];
  lsdg::slam::to12(k2f, k2f12);
  std::vector<float> img((size_t)s->w * s->h);
  for (size_t i = 0; i < img.size(); ++i) img[i] = (float)image[i];
  SLAM_CK(s, lsdg_depth_create_keyframe(s->ctx, s->dm, img.data(), k2f12, 1), s->ctx);
  const Keyframe& prev = s->keyframes[s->cur];
  Keyframe kf;
  kf.frame_index = frame_index;
  kf.parent = s->cur;
  kf.node = s->graph.add_node(lsdg::slam::mul(s->graph.poses[prev.node], f2k));
  r = new_frame_with_depth(s, image, &kf.frame);
  if (r == LSDG_OK) r = new_frame_with_depth(s, image, &kf.snapshot);
  if (r != LSDG_OK) {
    if (kf.frame) lsdg_frame_destroy(s->ctx, kf.frame);
    if (kf.snapshot) lsdg_frame_destroy(s->ctx, kf.snapshot);
    return r;
  }
  const int prev_node = prev.node;
  s->keyframes.push_back(kf);
  begin_keyframe_state(s, img.data(), s->d_buf.data(), s->v_buf.data());
  s->cur = (int)s->keyframes.size() - 1;
  s->traj.back() = {s->cur, M4::identity()};
  s->since_refresh = 0;
  // odometry edge from the tracking chain (SE3 information; the scale tied by a prior as strong as
  // the strongest direction)
  double W[49];
  if (se3_information(s, st, W)) s->graph.add_edge(prev_node, kf.node, f2k, W);
  s->stats.keyframes = (int)s->keyframes.size();
  return start_job(s, (int)s->keyframes.size() - 1);
}

}  // namespace

extern "C" {

void lsdg_slam_default_params(lsdg_slam_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->kf_dist = 0.1f;
  p->kf_angle_deg = 6.0f;
  p->kf_min_usage = 0.55f;
  p->refresh_every = 1;
  p->n_candidates = 10;
  p->cand_radius = 1.2f;
  p->optimize_every = 5;
  p->final_iterations = 20;
  p->max_track_jump = 0.2f;
  p->both_directions = 1;
  p->consistency_trans = 0.1f;
  p->consistency_rot = 0.02f;
  p->consistency_scale = 0.02f;
  p->async_constraints = 1;
  p->graph_threads = 8;
  p->odometry_scale_weight = 1.0f;
  p->ref_min_validity = 0;
  p->sim3_info_scale = 1e-3f;
  p->epipolar_var = 4.0f;
  p->reactivate = 1;
  p->react_radius = 0.5f;
  p->react_angle_deg = 20.0f;
  p->react_min_usage = 0.75f;
  p->react_max_jump = 0.5f;
  p->react_min_age = 10;
  p->react_min_good = 0.9f;
  p->retrack_iterations = 4;
}

lsdg_status lsdg_slam_create(const lsdg_params* params, const lsdg_slam_params* sp, int device, int width, int height,
                             const lsdg_intrinsics* intr, lsdg_slam** out) {
  if (!out || !intr) return LSDG_INVALID_ARG;
  *out = nullptr;
  lsdg_slam* s = new (std::nothrow) lsdg_slam();
  if (!s) return LSDG_OUT_OF_MEMORY;
  if (params) s->params = *params;
  else lsdg_default_params(&s->params);
  if (sp) s->sp = *sp;
  else lsdg_slam_default_params(&s->sp);
  if (s->sp.epipolar_var > 0.0f) s->params.epipolar_var = s->sp.epipolar_var;
  s->w = width;
  s->h = height;
  s->intr = *intr;
  s->graph.threads = std::max(1, s->sp.graph_threads);
  s->d_buf.resize((size_t)width * height);
  s->v_buf.resize((size_t)width * height);
  s->val_buf.resize((size_t)width * height);
  lsdg_status st = lsdg_create(&s->ctx, &s->params, device);
  if (st == LSDG_OK) st = lsdg_create(&s->ctx_cons, &s->params, device);
  if (st == LSDG_OK) st = lsdg_depth_create(s->ctx, width, height, intr, &s->dm);
  for (int i = 0; i < 2 && st == LSDG_OK; ++i) st = lsdg_frame_create(s->ctx, width, height, intr, &s->pool[i]);
  if (st != LSDG_OK) {
    lsdg_slam_destroy(s);
    return st;
  }
  *out = s;
  return LSDG_OK;
}

lsdg_status lsdg_slam_destroy(lsdg_slam* s) {
  if (!s) return LSDG_INVALID_ARG;
  if (s->worker_running) s->worker.join();
  for (auto& kv : s->batches)
    if (kv.second) lsdg_batch_destroy(s->ctx_cons, kv.second);
  for (Keyframe& k : s->keyframes) {
    if (k.frame) lsdg_frame_destroy(s->ctx, k.frame);
    if (k.snapshot) lsdg_frame_destroy(s->ctx, k.snapshot);
  }
  for (lsdg_frame* f : s->pool)
    if (f) lsdg_frame_destroy(s->ctx, f);
  for (lsdg_frame* f : s->hist_frames)
    if (f) lsdg_frame_destroy(s->ctx, f);
  if (s->refine_batch) lsdg_batch_destroy(s->ctx, s->refine_batch);
  if (s->dm) lsdg_depth_destroy(s->ctx, s->dm);
  if (s->ctx_cons) lsdg_destroy(s->ctx_cons);
  if (s->ctx) lsdg_destroy(s->ctx);
  delete s;
  return LSDG_OK;
}

const char* lsdg_slam_last_error(const lsdg_slam* s) { return s ? s->err.c_str() : "null system"; }

lsdg_status lsdg_slam_bootstrap(lsdg_slam* s, int id, const uint8_t* image, const float* idepth, const float* var) {
  if (!s || !image || !idepth || !var) return LSDG_INVALID_ARG;
  if (!s->keyframes.empty()) return fail(s, LSDG_INVALID_ARG, "already bootstrapped");
  std::vector<float> img((size_t)s->w * s->h);
  for (size_t i = 0; i < img.size(); ++i) img[i] = (float)image[i];
  SLAM_CK(s, lsdg_depth_set_keyframe(s->ctx, s->dm, img.data(), idepth, var), s->ctx);
  begin_keyframe_state(s, img.data(), idepth, var);
  Keyframe kf;
  kf.frame_index = 0;
  kf.node = s->graph.add_node(M4::identity());
  const lsdg_status st = new_frame_with_depth(s, image, &kf.frame);
  if (st != LSDG_OK) return st;
  s->keyframes.push_back(kf);
  s->cur = 0;
  s->traj.push_back({0, M4::identity()});
  s->traj_id.push_back(id);
  s->stats.frames = 1;
  s->stats.keyframes = 1;
  return LSDG_OK;
}

lsdg_status lsdg_slam_next_image(lsdg_slam* s, int id, const uint8_t* image) {
  if (!s || !image) return LSDG_INVALID_ARG;
  if (s->keyframes.empty()) return fail(s, LSDG_INVALID_ARG, "bootstrap the first keyframe first");
  const int kfi = s->cur;
  const Keyframe& kf = s->keyframes[kfi];
  // constant-velocity guess in the keyframe's frame; the first frame after a keyframe switch starts
  // from the switch frame's pose (carrying the velocity across the switch let one poor alignment's
  // motion grow from keyframe to keyframe: measured, the 640x480 room sequence ran away in 30 frames)
  const FramePose& last = s->traj.back();
  const M4 c1 = last.keyframe == kfi ? last.f2k : M4::identity();
  M4 c0 = c1;
  const size_t n = s->traj.size();
  if (n > 1 && s->traj[n - 2].keyframe == kfi) c0 = s->traj[n - 2].f2k;
  M4 guess = lsdg::slam::mul(lsdg::slam::mul(c1, lsdg::slam::sim3_inv(c0)), c1);
  if (!finite(guess)) guess = c1;
  lsdg_frame* frame = s->pool[s->pool_next];
  s->pool_next ^= 1;
  SLAM_CK(s, lsdg_frame_upload_u8(s->ctx, frame, image), s->ctx);
  double g12[12], o12[12];
  lsdg::slam::to12(guess, g12);
  lsdg_track_stats st{};
  const lsdg_status ts = lsdg_track_se3(s->ctx, kf.frame, frame, g12, o12, &st);
  if (ts != LSDG_OK && ts != LSDG_TRACKING_LOST) return fail(s, ts, "lsdg_track_se3", s->ctx);
  M4 f2k = lsdg::slam::from12(o12);
  const double jump[3] = {f2k(0, 3) - guess(0, 3), f2k(1, 3) - guess(1, 3), f2k(2, 3) - guess(2, 3)};
  bool good = st.status == LSDG_OK && finite(f2k) && norm3(jump) <= s->sp.max_track_jump;
  if (!good) {
    s->stats.lost_frames++;
    f2k = guess;
  }
  s->traj.push_back({kfi, f2k});
  s->traj_id.push_back(id);
  s->stats.frames++;
  if (!good) return LSDG_OK;
  // mapping: this frame observes the keyframe's depth
  const M4 k2f = lsdg::slam::sim3_inv(f2k);
  double k2f12[12];
  lsdg::slam::to12(k2f, k2f12);
  SLAM_CK(s, lsdg_depth_update_u8(s->ctx, s->dm, 1, image, k2f12, 1), s->ctx);
  if (s->sp.retrack_iterations > 0) {
    // the refinement window: the keyframe's most recent kMaxWindow frames (a keyframe that is never
    // left, under a still camera, keeps a bounded window)
    const size_t npix = (size_t)s->w * s->h;
    if ((int)s->hist_traj.size() >= kMaxWindow) {
      s->hist_images.erase(s->hist_images.begin(), s->hist_images.begin() + (long)npix);
      s->hist_traj.erase(s->hist_traj.begin());
    }
    s->hist_images.insert(s->hist_images.end(), image, image + npix);
    s->hist_traj.push_back((long)s->traj.size() - 1);
  }
  if (++s->since_refresh >= s->sp.refresh_every) {
    lsdg_status r = reference_depth(s, s->keyframes[kfi].frame);
    if (r != LSDG_OK) return r;
    s->since_refresh = 0;
  }
  const double t[3] = {f2k(0, 3), f2k(1, 3), f2k(2, 3)};
  if (norm3(t) > s->sp.kf_dist || rotation_angle(f2k) > s->sp.kf_angle_deg * M_PI / 180.0 ||
      st.usage < s->sp.kf_min_usage) {
    // the keyframe is left: refine it (poses of its frames, its depth)
    lsdg_status rr = refine_keyframe(s);
    if (rr != LSDG_OK) return rr;
    f2k = s->traj.back().f2k;
    if (s->sp.reactivate) {
      bool done = false;
      lsdg_status r = try_reactivate(s, frame, f2k, &done);
      if (r != LSDG_OK || done) return r;
    }
    return new_keyframe(s, (int)s->traj.size() - 1, image, f2k, st);
  }
  return LSDG_OK;
}

lsdg_status lsdg_slam_finalize(lsdg_slam* s) {
  if (!s) return LSDG_INVALID_ARG;
  lsdg_status r = join_worker(s);
  if (r != LSDG_OK) return r;
  const std::vector<M4> keep = s->graph.poses;
  s->graph.optimize(s->sp.final_iterations);
  bool good = true;
  for (const M4& T : s->graph.poses) good = good && finite(T);
  if (!good) s->graph.poses = keep;
  s->stats.graph_optimisations++;
  return LSDG_OK;
}

lsdg_status lsdg_slam_get_stats(const lsdg_slam* s, lsdg_slam_stats* out) {
  if (!s || !out) return LSDG_INVALID_ARG;
  *out = s->stats;
  return LSDG_OK;
}

lsdg_status lsdg_slam_get_poses(lsdg_slam* s, double* cam_to_world, int capacity, int* n) {
  if (!s || !n) return LSDG_INVALID_ARG;
  lsdg_status r = join_worker(s);
  if (r != LSDG_OK) return r;
  *n = (int)s->traj.size();
  if (!cam_to_world) return LSDG_OK;
  if (capacity < *n) return fail(s, LSDG_INVALID_ARG, "capacity below the frame count");
  for (size_t i = 0; i < s->traj.size(); ++i) {
    const M4 T = lsdg::slam::mul(s->graph.poses[s->keyframes[s->traj[i].keyframe].node], s->traj[i].f2k);
    lsdg::slam::to13(T, cam_to_world + 13 * i);
  }
  return LSDG_OK;
}

lsdg_status lsdg_slam_keyframe_graph(lsdg_slam* s, lsdg_graph_frame_pose* out, int capacity, int* n) {
  if (!s || !n) return LSDG_INVALID_ARG;
  lsdg_status r = join_worker(s);
  if (r != LSDG_OK) return r;
  *n = (int)s->keyframes.size();
  if (!out) return LSDG_OK;
  if (capacity < *n) return fail(s, LSDG_INVALID_ARG, "capacity below the keyframe count");
  for (int k = 0; k < *n; ++k) {
    double p13[13];
    lsdg::slam::to13(s->graph.poses[s->keyframes[k].node], p13);
    out[k].id = s->traj_id[s->keyframes[k].frame_index];
    lsdg_sim3_to_sophus7(p13, out[k].cam_to_world);
  }
  return LSDG_OK;
}

lsdg_status lsdg_slam_keyframe_depth(lsdg_slam* s, int k, int* frame_id, float* idepth, float* var) {
  if (!s || !idepth || !var) return LSDG_INVALID_ARG;
  lsdg_status r = join_worker(s);
  if (r != LSDG_OK) return r;
  if (k < 0 || k >= (int)s->keyframes.size()) return fail(s, LSDG_INVALID_ARG, "keyframe index out of range");
  if (frame_id) *frame_id = s->traj_id[s->keyframes[k].frame_index];
  SLAM_CK(s, lsdg_frame_get_depth(s->ctx, s->keyframes[k].frame, 0, idepth, var), s->ctx);
  return LSDG_OK;
}

lsdg_status lsdg_slam_write_pose_file(lsdg_slam* s, const char* path) {
  if (!s || !path) return LSDG_INVALID_ARG;
  lsdg_status r = join_worker(s);
  if (r != LSDG_OK) return r;
  FILE* f = std::fopen(path, "w");
  if (!f) return fail(s, LSDG_INVALID_ARG, "cannot open the pose file");
  char line[256];
  for (size_t i = 0; i < s->traj.size(); ++i) {
    const int kfi = s->traj[i].keyframe;
    const M4& Tk = s->graph.poses[s->keyframes[kfi].node];
    double c2w[13], rel[13];
    lsdg::slam::to13(lsdg::slam::mul(Tk, s->traj[i].f2k), c2w);
    lsdg::slam::to13(s->traj[i].f2k, rel);  // the frame's pose relative to its parent keyframe
    const int len = lsdg_format_pose_row(s->traj_id[i], c2w, rel, line, (int)sizeof(line));
    if (len > 0) std::fwrite(line, 1, (size_t)len, f);
  }
  std::fclose(f);
  return LSDG_OK;
}

// ---- the pose graph alone (host only), for tests and for callers with their own front end ----
struct lsdg_posegraph {
  lsdg::slam::PoseGraph g;
};

lsdg_status lsdg_posegraph_create(lsdg_posegraph** out) {
  if (!out) return LSDG_INVALID_ARG;
  *out = new (std::nothrow) lsdg_posegraph();
  return *out ? LSDG_OK : LSDG_OUT_OF_MEMORY;
}

lsdg_status lsdg_posegraph_destroy(lsdg_posegraph* g) {
  delete g;
  return LSDG_OK;
}

int lsdg_posegraph_add_node(lsdg_posegraph* g, const double cam_to_world13[13]) {
  if (!g || !cam_to_world13) return -1;
  return g->g.add_node(lsdg::slam::from13(cam_to_world13));
}

lsdg_status lsdg_posegraph_add_edge(lsdg_posegraph* g, int i, int j, const double z13[13], const double info[49]) {
  if (!g || !z13 || !info || i < 0 || j < 0 || i >= (int)g->g.poses.size() || j >= (int)g->g.poses.size())
    return LSDG_INVALID_ARG;
  g->g.add_edge(i, j, lsdg::slam::from13(z13), info);
  return LSDG_OK;
}

lsdg_status lsdg_posegraph_optimize(lsdg_posegraph* g, int iterations, double* cost) {
  if (!g) return LSDG_INVALID_ARG;
  const double c = g->g.optimize(iterations);
  if (cost) *cost = c;
  return LSDG_OK;
}

lsdg_status lsdg_posegraph_get_pose(const lsdg_posegraph* g, int i, double cam_to_world13[13]) {
  if (!g || !cam_to_world13 || i < 0 || i >= (int)g->g.poses.size()) return LSDG_INVALID_ARG;
  lsdg::slam::to13(g->g.poses[i], cam_to_world13);
  return LSDG_OK;
}

void lsdg_sim3_exp13(const double xi[7], double out13[13]) { lsdg::slam::to13(lsdg::slam::sim3_exp(xi), out13); }

void lsdg_sim3_log13(const double pose13[13], double xi[7]) { lsdg::slam::sim3_log(lsdg::slam::from13(pose13), xi); }

}  // extern "C"
