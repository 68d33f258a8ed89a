"""Generates the golden fixtures in this directory from the CPU oracle.

The reference ships no golden vectors for this path (its only test is ASSERT_TRUE(true),
test/unit/test_test.cpp:4-7) and its lsd-slam code cannot be built here, so these fixtures freeze
the oracle's own outputs on small seeded cases: they pin the oracle across machines (x86 and Arm
hosts) and over time, and the GPU tests compare the library against them.

Inputs are stored in a platform-independent form (images rounded to uint8, depths as float32), so
the fixtures do not depend on the synthetic renderer's floating-point details.  Outputs that are
bit-exact by construction (pyramids, points, depth-filter planes) are stored as SHA-256 of their
bytes; poses and sums as values.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "lsd-slam-pangolin-gui_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


class Pair:
    pass


class Seq:
    pass


def load_inputs():
    z = np.load(os.path.join(HERE, "golden_small.npz"))
    import synth
    p = Pair()
    p.w, p.h = 160, 128
    p.intr = synth.Intrinsics.for_size(p.w, p.h)
    p.ref_image = z["t_key"].astype(np.float32)
    p.new_image = z["t_new"].astype(np.float32)
    p.ref_idepth = z["t_idepth"]
    p.ref_idepth_var = np.where(p.ref_idepth > 0, np.float32(0.01), np.float32(-1)).astype(np.float32)
    s = Seq()
    s.w, s.h = 160, 128
    s.intr = p.intr
    s.key_image = z["d_key"].astype(np.float32)
    s.ref_images = [r.astype(np.float32) for r in z["d_refs"]]
    s.ref_frame_to_key = [T for T in z["d_ref_poses"]]
    s.next_image = z["d_next"].astype(np.float32)
    s.next_to_key = z["d_next_pose"]
    s.init_idepth = (z["d_init_q12"].astype(np.float32) / np.float32(4096)).astype(np.float32)
    s.init_var = np.full((s.h, s.w), 0.5, np.float32)
    return p, s


def oracle_outputs(p, s):
    import lsdo
    out = {}
    pyr = lsdo.pyramid(p.new_image, 5)
    out["pyramid_sha"] = [sha(l) for l in pyr]
    D, V, P, PV = lsdo.keyframe(p.ref_image, p.ref_idepth, p.ref_idepth_var, p.intr, 5)
    out["points_sha"] = [sha(x) for x in P]
    out["points_count"] = [int(len(x)) for x in P]
    T0 = np.eye(3, 4)
    out["normal_equations_level1"] = lsdo.se3_normal_equations(p, T0, 1).tolist()
    rc, T, st = lsdo.track_se3(p)
    out["track_status"] = int(rc)
    out["track_pose"] = T.ravel().tolist()
    out["track_passes"] = list(st.passes)
    upd, prop = lsdo.depth_pipeline(s)
    out["depth_update_sha"] = {k: sha(v) for k, v in upd.items()}
    out["depth_propagate_sha"] = {k: sha(v) for k, v in prop.items()}
    out["depth_valid_after_update"] = int((upd["validity"] > 0).sum())
    return out


def make_inputs():
    import synth
    p = synth.tracking_pair(4, 160, 128)
    s = synth.depth_sequence(4, 160, 128, n_refs=4)
    q = lambda im: np.clip(np.rint(im), 0, 255).astype(np.uint8)
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"),
                        t_key=q(p.ref_image), t_new=q(p.new_image), t_idepth=p.ref_idepth.astype(np.float32),
                        d_key=q(s.key_image), d_refs=np.stack([q(r) for r in s.ref_images]),
                        d_ref_poses=np.stack(s.ref_frame_to_key), d_next=q(s.next_image), d_next_pose=s.next_to_key,
                        d_init_q12=np.rint(s.init_idepth * 4096).astype(np.uint16))


if __name__ == "__main__":
    make_inputs()
    p, s = load_inputs()
    with open(os.path.join(HERE, "golden_small.json"), "w") as f:
        json.dump(oracle_outputs(p, s), f, indent=1)
    print("wrote", os.listdir(HERE))
