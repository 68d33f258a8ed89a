// Exercises the C++ facade (include/lsdg/lsdg.hpp) the way SlamSystem's threads would: a tracking
// thread aligning a frame to a keyframe, a mapping thread updating and propagating the keyframe's
// depth, the photometric energy's forward / backward, and a constraint-search Sim3 tracking.  Input planes are raw float32 files written by the Python test; prints one line of results.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lsdg/lsdg.hpp"

static std::vector<float> load(const char* path, size_t n) {
  std::vector<float> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), 4, n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  const int w = 320, h = 240;
  const size_t n = (size_t)w * h;
  const lsdg_intrinsics K{250.f, 250.f, 159.75f, 119.75f};
  auto key = load((dir + "/key.f32").c_str(), n);
  auto idepth = load((dir + "/idepth.f32").c_str(), n);
  auto var = load((dir + "/var.f32").c_str(), n);
  auto cur = load((dir + "/cur.f32").c_str(), n);
  try {
    lsdg::Context ctx(0);
    lsdg::Frame kf(ctx, w, h, K), fr(ctx, w, h, K);
    kf.upload(key.data()).setDepth(idepth.data(), var.data());
    fr.upload(cur.data());
    lsdg::SE3Tracker tracker(ctx);
    const lsdg::Pose T = tracker.trackFrame(kf, fr, lsdg::identity());
    std::printf("pose");
    for (double v : T) std::printf(" %.17g", v);
    std::printf(" good %d passes %d\n", tracker.trackingWasGood() ? 1 : 0, tracker.lastStats.total_passes);
    lsdg::DepthMap dm(ctx, w, h, K);
    dm.initializeKeyframe(key.data(), idepth.data(), var.data());
    // the tracked frame serves as the reference frame of the keyframe's depth update
    dm.updateKeyframe({cur.data()}, {lsdg::inverse(T)}, true);
    std::vector<float> d(n), v(n);
    dm.idepth(d.data(), v.data());
    size_t valid = 0;
    for (float x : d) valid += x > 0;
    std::printf("depth_valid %zu\n", valid);
    // differentiable energy at the tracked pose: forward / backward as an autograd Function
    lsdg::PhotometricEnergy::SavedContext sc(ctx, kf, 0);
    const double E = lsdg::PhotometricEnergy::forward(sc, fr, lsdg::inverse(T));
    const lsdg::PhotometricEnergy::Grad g = lsdg::PhotometricEnergy::backward(sc, 1.0);
    size_t nz = 0;
    for (float x : g.idepth) nz += x != 0.f;
    std::printf("energy %.17g", E);
    for (double v : g.xi) std::printf(" %.17g", v);
    std::printf(" points %d nonzero %zu\n", sc.size(), nz);
    // Sim3 constraint tracking between two keyframes with depth
    auto sk = load((dir + "/s_key.f32").c_str(), n), skd = load((dir + "/s_kid.f32").c_str(), n),
         skv = load((dir + "/s_kvar.f32").c_str(), n), sn = load((dir + "/s_new.f32").c_str(), n),
         snd = load((dir + "/s_nid.f32").c_str(), n), snv = load((dir + "/s_nvar.f32").c_str(), n);
    lsdg::Frame ki(ctx, w, h, K), kj(ctx, w, h, K);
    ki.upload(sk.data()).setDepth(skd.data(), skv.data());
    kj.upload(sn.data()).setDepth(snd.data(), snv.data());
    lsdg::Sim3Tracker st(ctx);
    const lsdg::Sim3 S = st.trackFrameSim3(ki, kj, lsdg::Sim3{});
    const auto sp = S.packed();
    std::printf("sim3");
    for (double v : sp) std::printf(" %.17g", v);
    std::printf(" good %d\n", st.trackingWasGood() ? 1 : 0);
  } catch (const lsdg::Error& e) {
    std::printf("error %d %s\n", (int)e.status, e.what());
    return 1;
  }
  return 0;
}
