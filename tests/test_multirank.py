"""Multi-rank host logic on CPU: the pair partition (pure function) and a world_size-2 gloo run of
the sharded tracking through torch.distributed.run, as bench.py is launched for N > 1."""
import json
import os
import socket
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import shard

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MIXED = [(320, 240)] * 20 + [(640, 480)] * 32 + [(1280, 960)] * 12


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_covers_and_balances(world):
    costs = [shard.pair_cost(w, h) for w, h in MIXED]
    parts = shard.partition(costs, world)
    assert len(parts) == world
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) <= sum(costs) / world + max(costs)
    assert parts == shard.partition(costs, world)  # deterministic
    assert all(p == sorted(p) for p in parts)


def test_partition_edge_cases():
    assert shard.partition([], 2) == [[], []]
    assert shard.partition([5], 3) == [[0], [], []]
    assert shard.partition([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard.partition([1], 0)


def test_gather_rows_single_process():
    out = shard.gather_rows([2, 0], np.array([[2.0], [0.0]]), 3)
    assert out.shape == (3, 1) and out[0, 0] == 0.0 and out[2, 0] == 2.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gloo_shard_and_gather():
    """Two gloo ranks track disjoint shares of 5 mixed-size pairs on the CPU oracle; the gathered
    poses equal a single-process run bit for bit, and the max over ranks reaches every rank."""
    import lsdo
    import synth
    from multirank_worker import SPECS
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "r0.json")
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", OMP_NUM_THREADS="1")
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
               "--master-addr=127.0.0.1", "--master-port=%d" % _free_port(),
               os.path.join(ROOT, "tests", "multirank_worker.py"), out]
        r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        res = json.load(open(out))
    assert res["world"] == 2 and res["tmax"] == 2.0 and res["tsum"] == 3.0
    costs = [shard.pair_cost(w, h) for _, w, h in SPECS]
    assert res["share0"] == shard.partition(costs, 2)[0]
    for i, (s, w, h) in enumerate(SPECS):
        rc, T, st = lsdo.track_se3(synth.tracking_pair(s, w, h))
        assert res["status"][i] == rc
        np.testing.assert_array_equal(np.array(res["poses"][i]), np.asarray(T).reshape(12))
