// lsdg.hpp -- header-only C++ facade over the C-ABI (include/lsdg.h) with the names and calling
// conventions of the upstream objects the reference's threads use (lsd-slam: Frame, SE3Tracker,
// DepthMap).  Errors become lsdg::Error exceptions on this side of the ABI; tracking failure is not an
// error (trackFrame returns the pose and the stats say LSDG_TRACKING_LOST), as upstream.
//
// Mapping (upstream -> here):
//   SlamSystem::nextImage builds a Frame           -> lsdg::Frame(ctx, w, h, K).upload(img)
//   Frame::idepth(lvl) / idepthVar(lvl)            -> Frame::depth(lvl, idepth, var)
//   SE3Tracker::trackFrame(ref, frame, initial)    -> SE3Tracker::trackFrame(ref, frame, initial)
//   DepthMap::updateKeyframe(referenceFrames)      -> DepthMap::updateKeyframe(images, poses)
//   DepthMap::createKeyFrame(newKeyframe)          -> DepthMap::createKeyFrame(image, keyToNew)
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
