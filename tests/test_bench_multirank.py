"""bench.py --gpus 2 launches its own ranks (CPU, gloo, stand-in engine).

Outside torchrun, `bench.py --gpus N` re-launches itself under
torch.distributed.run with N ranks.  Here the engine binding is replaced by a
stand-in module with the same interface (EDMD_BENCH_ENGINE_MODULE), so the
real launch path -- rank set-up, per-rank device selection, per-rank system
shards, barriers, max/sum reductions, rank 0's single JSON line -- runs on CPU.
Each rank's stand-in records the seeds of the systems it was given.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

FAKE = r'''
import os
import numpy as np

OK = 0
F_STOP_AT_GROW, F_COUNT_NORMAL, F_EXACT = 2, 8, 32
ENGINE_WARP, ENGINE_LANE = 1, 2
_out = os.environ["EDMD_FAKE_OUT"]
_rank = os.environ.get("RANK", "0")


class _Lib:
    def edmd_set_device(self, d):
        with open(os.path.join(_out, "device_%s" % _rank), "w") as f:
            f.write(str(d))
        return 0


def load():
    return _Lib()


class _Desc:
    def __init__(self, N, Lx, Ly):
        self.N, self.Lx, self.Ly = N, Lx, Ly


def default_desc(N, Lx, Ly, vr_base=0.0, tmax=4000.0):
    return _Desc(N, Lx, Ly)


def grow_start(N, phi, seed, xs=0.3, q=0.4):
    with open(os.path.join(_out, "seeds_%s" % _rank), "a") as f:
        f.write("%d\n" % seed)
    L = (N * 3.14159 / phi) ** 0.5
    return dict(N=N, Lx=L, Ly=L, vr_base=0.1, x=np.zeros(N), y=np.zeros(N), vx=np.zeros(N),
                vy=np.zeros(N), rad=np.ones(N), m=np.ones(N), vr=np.zeros(N))


def set_warp_group(g):
    pass


class Engine:
    def __init__(self, systems, engine=ENGINE_WARP):
        self.n = len(systems)
        self.TN = sum(s["N"] for s in systems)
        self.ncol = np.zeros(self.n, np.int64)

    def advance(self, max_coll=2**62, flags=0, **kw):
        if max_coll < 2**62:
            self.ncol += max_coll
        return 0, 1.0

    def last_launches(self):
        return 1

    def all_counters(self):
        z = np.zeros(self.n, np.int64)
        return dict(ncol=self.ncol.copy(), npair=self.ncol * 19, npred=self.ncol * 2, growing=z)

    def sync(self):
        pass

    def states(self, out=None):
        return {k: np.zeros(self.TN) for k in ("x", "y", "vx", "vy", "rad", "m")}

    def load_state(self, *a):
        pass

    def close(self):
        pass


class PinnedArray:
    def __init__(self, n):
        self.a = np.zeros(n)

    def free(self):
        pass
'''


def test_bench_launches_two_ranks_itself(tmp_path):
    pytest.importorskip("torch.distributed")
    fake = tmp_path / "fake_edmd.py"
    fake.write_text(FAKE)
    env = dict(os.environ, EDMD_BENCH_ENGINE_MODULE=str(fake), EDMD_FAKE_OUT=str(tmp_path))
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--steps", "2",
                          "--warmup", "3", "--nsys", "16", "--coll", "100", "--no-cpu-baseline",
                          "--no-secondary", "--no-tune"], capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2
    assert d["config"]["parallelism"] == "replicas x2"
    # every rank: 16 systems x 100 collisions per step, 2 steps, 1 ms per step
    assert d["value"] == pytest.approx(2 * 16 * 100 * 2 / (2 * 1e-3))
    seeds = [set((tmp_path / f"seeds_{r}").read_text().split()) for r in (0, 1)]
    assert len(seeds[0]) == len(seeds[1]) == 16 and not seeds[0] & seeds[1]
    assert (tmp_path / "device_0").read_text() == "0" and (tmp_path / "device_1").read_text() == "1"
