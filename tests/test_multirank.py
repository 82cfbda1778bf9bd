"""Two ranks over gloo on the CPU (torch.distributed.run, 127.0.0.1).

They cover the multi-rank logic of this build, and the reference's own
scheme:
* this build shards by cell with no data exchange: each rank integrates its
  cell range of the same Illum with the oracle, and the shards, gathered,
  equal the single-process result.  The residual of a step is a max
  all-reduce of the ranks' residuals;
* the reference shards by out-direction (GetSend / GetDisp): each rank takes
  its rts_partition section, and the all-gathered sections form the full S;
* bench.py's timing reduction takes the slowest rank's time
  (max_over_ranks), and the whole-job value counts every rank's replica."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parents[1]

RANK_SCRIPT = r"""
import json, os, sys
import numpy as np
import torch
import torch.distributed as dist
sys.path.insert(0, os.environ["RTS_ROOT"])
import oracle
import bench
from relativistic_solver_hllc_gb300 import _native

rank, world, _ = bench.dist_env()
dist.init_process_group("gloo")
N, M = 257, 24
xyz, area, fa = oracle.fibonacci_directions(M)
il = oracle.illum(5, 0.0, 1.0, N, M, independent_faces=True)
full = oracle.calculate_int_cpu(N, xyz, area, fa, il)

# cell shards (this build): no exchange on the data path
c0, c1 = rank * N // world, (rank + 1) * N // world
part = oracle.calculate_int_cells(N, xyz, area, fa, il, np.arange(c0, c1))
shards = [None] * world
dist.all_gather_object(shards, (c0, c1, part.tolist()))
cells_ok = all(np.array_equal(np.array(p), full[:, a:b]) for a, b, p in shards)
res = bench.max_over_ranks(float(np.abs(part).max()), dist, device="cpu")

# out-direction sections (the reference's GetSend / GetDisp)
send, disp = _native.partition(world, M)
sec = oracle.calculate_int_cpu(N, xyz, area, fa, il, disp[rank], send[rank])
secs = [None] * world
dist.all_gather_object(secs, sec.tolist())
dirs_ok = np.array_equal(np.concatenate([np.array(s) for s in secs], axis=0), full)

# the bench's reduction: the slowest rank's time, whole-job value of all replicas
t = bench.max_over_ranks(1.0 + rank, dist, device="cpu")
value = bench.replicas_value(N, M, 3, world, t)
out = {"rank": rank, "cells_ok": bool(cells_ok), "dirs_ok": bool(dirs_ok),
       "residual": res, "full_residual": float(np.abs(full).max()), "t": t, "value": value,
       "send": send, "disp": disp}
with open(os.path.join(os.environ["RTS_OUT"], f"rank{rank}.json"), "w") as f:
    json.dump(out, f)
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks(tmp_path):
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT)
    env = dict(os.environ, RTS_ROOT=str(ROOT), RTS_OUT=str(tmp_path), OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(script)]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    outs = [json.loads((tmp_path / f"rank{i}.json").read_text()) for i in range(2)]
    for o in outs:
        assert o["cells_ok"] and o["dirs_ok"]
        assert o["residual"] == o["full_residual"]
        assert o["t"] == 2.0  # the slower rank's time
        assert abs(o["value"] - 257 * 24 * 3 * 2 / 2.0 / 1e9) < 1e-15
        assert o["send"] == [12, 12] and o["disp"] == [0, 12]
