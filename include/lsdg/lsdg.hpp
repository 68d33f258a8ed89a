// lsdg.hpp -- header-only C++ facade over the C-ABI (include/lsdg.h) with the names and calling
// conventions of the upstream objects the reference's threads use (lsd-slam: Frame, SE3Tracker,
// DepthMap).  Errors become lsdg::Error exceptions on this side of the ABI; tracking failure is not an
// error (trackFrame returns the pose and the stats say LSDG_TRACKING_LOST), as upstream.
//
// Mapping (upstream -> here):
//   SlamSystem::nextImage builds a Frame           -> lsdg::Frame(ctx, w, h, K).upload(img)
//   Frame::idepth(lvl) / idepthVar(lvl)            -> Frame::depth(lvl, idepth, var)
//   SE3Tracker::trackFrame(ref, frame, initial)    -> SE3Tracker::trackFrame(ref, frame, initial)
//   Sim3Tracker::trackFrameSim3(ref, frame, init)  -> Sim3Tracker::trackFrameSim3(ref, frame, initial)
//   DepthMap::updateKeyframe(referenceFrames)      -> DepthMap::updateKeyframe(images, poses)
//   DepthMap::createKeyFrame(newKeyframe)          -> DepthMap::createKeyFrame(image, keyToNew)
// New (no upstream counterpart): PhotometricEnergy, the energy of a keyframe against a frame with
// the forward / backward pair of an autograd Function (SavedContext = what forward saves).
#pragma once

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

#include "../lsdg.h"

namespace lsdg {

class Error : public std::runtime_error {
 public:
  Error(lsdg_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
  lsdg_status status;
};

// 3x4 row-major [R | t]: a_to_b maps camera-a coordinates into camera b.
using Pose = std::array<double, 12>;

inline Pose identity() { return Pose{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}; }

inline Pose inverse(const Pose& a) {
  Pose b;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) b[4 * i + j] = a[4 * j + i];
  for (int i = 0; i < 3; ++i) b[4 * i + 3] = -(b[4 * i + 0] * a[3] + b[4 * i + 1] * a[7] + b[4 * i + 2] * a[11]);
  return b;
}

class Context {
 public:
  explicit Context(int device = 0, const lsdg_params* params = nullptr) {
    const lsdg_status s = lsdg_create(&ctx_, params, device);
    if (s != LSDG_OK) throw Error(s, "lsdg_create failed (no usable sm_103 device?)");
  }
  ~Context() {
    if (ctx_) lsdg_destroy(ctx_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  lsdg_ctx* get() const { return ctx_; }
  void check(lsdg_status s, lsdg_status also_ok = LSDG_OK) const {
    if (s != LSDG_OK && s != also_ok) throw Error(s, lsdg_last_error(ctx_));
  }
  static lsdg_params default_params() {
    lsdg_params p;
    lsdg_default_params(&p);
    return p;
  }

 private:
  lsdg_ctx* ctx_ = nullptr;
};

class Frame {
 public:
  Frame(Context& ctx, int width, int height, const lsdg_intrinsics& K) : ctx_(ctx), w_(width), h_(height) {
    ctx_.check(lsdg_frame_create(ctx_.get(), width, height, &K, &f_));
  }
  ~Frame() {
    if (f_) lsdg_frame_destroy(ctx_.get(), f_);
  }
  Frame(const Frame&) = delete;
  Frame& operator=(const Frame&) = delete;
  Frame& upload(const float* image) {
    ctx_.check(lsdg_frame_upload(ctx_.get(), f_, image));
    return *this;
  }
  Frame& upload(const uint8_t* image) {
    ctx_.check(lsdg_frame_upload_u8(ctx_.get(), f_, image));
    return *this;
  }
  Frame& setDepth(const float* idepth, const float* idepth_var) {
    ctx_.check(lsdg_frame_set_depth(ctx_.get(), f_, idepth, idepth_var));
    return *this;
  }
  void depth(int level, float* idepth, float* idepth_var) const {
    ctx_.check(lsdg_frame_get_depth(ctx_.get(), f_, level, idepth, idepth_var));
  }
  int width(int level = 0) const { return w_ >> level; }
  int height(int level = 0) const { return h_ >> level; }
  const lsdg_frame* get() const { return f_; }

 private:
  Context& ctx_;
  lsdg_frame* f_ = nullptr;
  int w_, h_;
};

class SE3Tracker {
 public:
  explicit SE3Tracker(Context& ctx) : ctx_(ctx) {}
  // Aligns `frame` to the keyframe `reference`; returns frameToReference.
  Pose trackFrame(const Frame& reference, const Frame& frame, const Pose& frameToReference_initialEstimate) {
    Pose out;
    ctx_.check(lsdg_track_se3(ctx_.get(), reference.get(), frame.get(), frameToReference_initialEstimate.data(),
                              out.data(), &lastStats),
               LSDG_TRACKING_LOST);
    return out;
  }
  bool trackingWasGood() const { return lastStats.status == LSDG_OK; }
  lsdg_track_stats lastStats{};

 private:
  Context& ctx_;
};

// Sim3 pose: x_b = s R x_a + t.
struct Sim3 {
  std::array<double, 9> R{1, 0, 0, 0, 1, 0, 0, 0, 1};
  std::array<double, 3> t{0, 0, 0};
  double s = 1.0;
  std::array<double, 13> packed() const {
    std::array<double, 13> p;
    std::copy(R.begin(), R.end(), p.begin());
    std::copy(t.begin(), t.end(), p.begin() + 9);
    p[12] = s;
    return p;
  }
  static Sim3 unpack(const double* p) {
    Sim3 x;
    std::copy(p, p + 9, x.R.begin());
    std::copy(p + 9, p + 12, x.t.begin());
    x.s = p[12];
    return x;
  }
};

class Sim3Tracker {
 public:
  explicit Sim3Tracker(Context& ctx) : ctx_(ctx) {}
  // Aligns keyframe `frame` (with depth) to keyframe `reference`; returns frameToReference.
  Sim3 trackFrameSim3(const Frame& reference, const Frame& frame, const Sim3& frameToReference_initialEstimate) {
    const std::array<double, 13> in = frameToReference_initialEstimate.packed();
    std::array<double, 13> out;
    ctx_.check(lsdg_track_sim3(ctx_.get(), reference.get(), frame.get(), in.data(), out.data(), &lastStats),
               LSDG_TRACKING_LOST);
    return Sim3::unpack(out.data());
  }
  bool trackingWasGood() const { return lastStats.status == LSDG_OK; }
  lsdg_track_stats lastStats{};

 private:
  Context& ctx_;
};

// E(xi, rho) = sum_i h(r_i^2 / s_i) of a keyframe level's points against a frame (see
// lsdg_energy_forward).  Usage, as with an autograd Function:
//   PhotometricEnergy::SavedContext sc(ctx, keyframe, level);
//   double E = PhotometricEnergy::forward(sc, frame, refToFrame);
//   PhotometricEnergy::Grad g = PhotometricEnergy::backward(sc, dLdE);
class PhotometricEnergy {
 public:
  class SavedContext {
   public:
    SavedContext(Context& ctx, const Frame& keyframe, int level = 0) : ctx_(ctx) {
      ctx_.check(lsdg_energy_create(ctx_.get(), keyframe.get(), level, &e_));
      ctx_.check(lsdg_energy_size(ctx_.get(), e_, &n_));
    }
    ~SavedContext() {
      if (e_) lsdg_energy_destroy(ctx_.get(), e_);
    }
    SavedContext(const SavedContext&) = delete;
    SavedContext& operator=(const SavedContext&) = delete;
    int size() const { return n_; }
    std::vector<float> idepth() const {
      std::vector<float> r((size_t)n_);
      ctx_.check(lsdg_energy_get_idepth(ctx_.get(), e_, r.data()));
      return r;
    }
    void setIdepth(const std::vector<float>& rho) {
      if ((int)rho.size() != n_) throw Error(LSDG_INVALID_ARG, "one inverse depth per point");
      ctx_.check(lsdg_energy_set_idepth(ctx_.get(), e_, rho.data()));
    }
    // Photometric inverse-depth refinement over frames at fixed poses (see lsdg_energy_refine).
    void refine(const std::vector<const Frame*>& frames, const std::vector<Pose>& refToFrames, int steps = 50) {
      if (frames.size() != refToFrames.size()) throw Error(LSDG_INVALID_ARG, "one pose per frame");
      std::vector<const lsdg_frame*> fs;
      std::vector<double> poses;
      for (size_t j = 0; j < frames.size(); ++j) {
        fs.push_back(frames[j]->get());
        poses.insert(poses.end(), refToFrames[j].begin(), refToFrames[j].end());
      }
      ctx_.check(lsdg_energy_refine(ctx_.get(), e_, (int)fs.size(), fs.data(), poses.data(), steps, &energyBefore,
                                    &energyAfter, &refined));
    }
    double energyBefore = 0, energyAfter = 0;
    int refined = 0;
    int dof = 6;

   private:
    friend class PhotometricEnergy;
    Context& ctx_;
    lsdg_energy* e_ = nullptr;
    int n_ = 0;
  };
  struct Grad {
    std::vector<double> xi;      // dL/dxi (6, or 7 for Sim3)
    std::vector<float> idepth;   // dL/drho per point
  };
  static double forward(SavedContext& sc, const Frame& frame, const Pose& refToFrame, int dof = 6) {
    double E = 0;
    sc.ctx_.check(lsdg_energy_forward(sc.ctx_.get(), sc.e_, frame.get(), refToFrame.data(), dof, &E, nullptr));
    sc.dof = dof;
    return E;
  }
  static Grad backward(SavedContext& sc, double grad_output) {
    Grad g;
    g.xi.resize((size_t)sc.dof);
    g.idepth.resize((size_t)sc.n_);
    sc.ctx_.check(lsdg_energy_backward(sc.ctx_.get(), sc.e_, grad_output, g.xi.data(), g.idepth.data()));
    return g;
  }
};

class DepthMap {
 public:
  DepthMap(Context& ctx, int width, int height, const lsdg_intrinsics& K) : ctx_(ctx), w_(width), h_(height) {
    ctx_.check(lsdg_depth_create(ctx_.get(), width, height, &K, &dm_));
  }
  ~DepthMap() {
    if (dm_) lsdg_depth_destroy(ctx_.get(), dm_);
  }
  DepthMap(const DepthMap&) = delete;
  DepthMap& operator=(const DepthMap&) = delete;
  void initializeKeyframe(const float* image, const float* idepth, const float* idepth_var) {
    ctx_.check(lsdg_depth_set_keyframe(ctx_.get(), dm_, image, idepth, idepth_var));
  }
  // images: n reference frames back to back (w*h floats each); keyToReference: one pose each.
  void updateKeyframe(const std::vector<const float*>& images, const std::vector<Pose>& keyToReference,
                      bool regularize = true) {
    if (images.size() != keyToReference.size()) throw Error(LSDG_INVALID_ARG, "one pose per reference frame");
    std::vector<float> packed((size_t)w_ * h_ * images.size());
    std::vector<double> poses(12 * images.size());
    for (size_t r = 0; r < images.size(); ++r) {
      std::copy(images[r], images[r] + (size_t)w_ * h_, packed.begin() + (size_t)w_ * h_ * r);
      std::copy(keyToReference[r].begin(), keyToReference[r].end(), poses.begin() + 12 * r);
    }
    ctx_.check(lsdg_depth_update(ctx_.get(), dm_, (int)images.size(), packed.data(), poses.data(), regularize ? 1 : 0));
  }
  void regularizeDepthMap() { ctx_.check(lsdg_depth_regularize(ctx_.get(), dm_)); }
  void createKeyFrame(const float* newImage, const Pose& keyToNew, bool regularize = true) {
    ctx_.check(lsdg_depth_create_keyframe(ctx_.get(), dm_, newImage, keyToNew.data(), regularize ? 1 : 0));
  }
  // Frame::idepth(0) / idepthVar(0) of the keyframe: the smoothed map the viewer shows.
  void idepth(float* idepth_out, float* var_out) const {
    ctx_.check(lsdg_depth_get(ctx_.get(), dm_, nullptr, nullptr, idepth_out, var_out, nullptr, nullptr));
  }
  void state(float* idepth, float* var, int32_t* validity, int32_t* blacklist) const {
    ctx_.check(lsdg_depth_get(ctx_.get(), dm_, idepth, var, nullptr, nullptr, validity, blacklist));
  }

 private:
  Context& ctx_;
  lsdg_depthmap* dm_ = nullptr;
  int w_, h_;
};

}  // namespace lsdg
