"""One rank of the CPU multi-rank test (launched by torch.distributed.run with the gloo backend):
shards a mixed-size set of tracking pairs with shard.partition, tracks its share with the float CPU
oracle, takes the max of the ranks' times and gathers the poses to every rank.  Rank 0 writes what
it saw to argv[1] for the test to check.  This stands in for bench.py's N > 1 host logic; the GPU
work per rank is the same call on a different share."""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (os.path.join(ROOT, "lsd-slam-pangolin-gui_gb300"), os.path.join(ROOT, "oracle"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402
import torch.distributed as dist  # noqa: E402

import lsdo  # noqa: E402
import shard  # noqa: E402
import synth  # noqa: E402

SPECS = [(11, 160, 128), (12, 320, 240), (13, 160, 128), (14, 320, 256), (15, 160, 128)]


def main():
    rank, world, _ = shard.rank_env()
    dist.init_process_group("gloo")
    costs = [shard.pair_cost(w, h) for _, w, h in SPECS]
    mine = shard.my_share(costs, rank, world)
    t0 = time.perf_counter()
    poses, status = [], []
    for i in mine:
        s, w, h = SPECS[i]
        rc, T, st = lsdo.track_se3(synth.tracking_pair(s, w, h))
        poses.append(np.asarray(T).reshape(12))
        status.append(rc)
    elapsed = time.perf_counter() - t0
    tmax = shard.max_over_ranks(float(rank + 1), dist)  # every rank must see the largest value
    tsum = shard.sum_over_ranks(float(rank + 1), dist)
    allp = shard.gather_rows(mine, np.array(poses).reshape(len(mine), 12), len(SPECS), dist)
    alls = shard.gather_rows(mine, np.array(status, np.int64).reshape(len(mine)), len(SPECS), dist)
    if rank == 0:
        with open(sys.argv[1], "w") as f:
            json.dump({"world": world, "share0": mine, "tmax": tmax, "tsum": tsum, "poses": allp.tolist(), "status": alls.tolist(),
                       "elapsed": elapsed}, f)
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
