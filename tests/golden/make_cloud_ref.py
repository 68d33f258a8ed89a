"""Generates tests/golden/cloud_ref.npz: outputs of the reference's own point-cloud loop
(Keyframe::computeVbo, lib/Pangolin_IOWrapper/Keyframe.h:66-143), compiled from its source by
oracle/ref_build.py, on seeded keyframes.  The fixture pins the cloud oracle and the cloud kernel
to reference code where the reference tree is absent.

Each case stores its InputPointDense array (w x h records of 12 bytes), the intrinsics, the
keyframe scale and the vertices computeVbo produced (16-byte records).

    python tests/golden/make_cloud_ref.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "lsd-slam-pangolin-gui_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

# (seed, w, h, fx, fy, cx, cy, scale): every filter branch and support counts around 9 occur
CASES = [
    (7, 64, 48, 60.0, 58.0, 31.5, 23.25, 1.0),
    (8, 64, 48, 60.0, 58.0, 31.5, 23.25, 12.0),
    (9, 96, 72, 90.0, 91.0, 47.0, 35.5, 0.5),
]


def main():
    import lsdo
    from test_oracle_cloud import random_keyframe

    if lsdo.ref_lib() is None:
        raise SystemExit("oracle/_ref could not be built: the reference tree is absent")
    out = {}
    for k, (seed, w, h, fx, fy, cx, cy, scale) in enumerate(CASES):
        pts = random_keyframe(seed, w, h)
        v = lsdo.ref_compute_vbo(pts, w, h, fx, fy, cx, cy, scale)
        out[f"points{k}"] = np.frombuffer(pts.tobytes(), np.uint8)
        out[f"vertices{k}"] = np.frombuffer(v.tobytes(), np.uint8)
        out[f"camera{k}"] = np.array([w, h, fx, fy, cx, cy, scale], np.float64)
        print(f"case {k}: {w}x{h} scale {scale}: {len(v)} vertices")
    np.savez_compressed(os.path.join(HERE, "cloud_ref.npz"), **out)


if __name__ == "__main__":
    main()
