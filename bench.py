#!/usr/bin/env python
"""Throughput benchmark of the GB300 event-driven hard-disk engine.

Metric: accepted pair collisions per second on one GB300 (the reference's
``ncol`` increments, src/EDMD.c:3558; growth-phase collisions excluded).

Default workload ("batched"): 4096 independent periodic systems, N uniform in
[256, 4096], area fraction uniform in [0.30, 0.75], 50:50 bidisperse diameters
1.0/1.4 (-x 0.5 -q 0.7142857), per-system seeds, the reference's growth start
(untimed set-up), then one step = 10^5 accepted collisions per system in one
persistent launch.  Data are synthetic (the reference has no dataset); the
state (~1 GB) is far larger than L2, so no flush is needed between steps.

``--workload plain_small`` runs the single 1980-disk Hex system (phi 0.70)
instead, one step = 10^5 collisions.

The JSON line carries the device-resident throughput (``value``), the
end-to-end throughput through the C ABI with host buffers (``e2e``: restart
from pinned host state, run, read the state back), the roofline of the run
kernel, the CPU baseline (the oracle on all host cores) and the SM clocks
sampled during the timed region.  ``--impl reference`` times the reference
algorithm on the host cores (the oracle restatement; the reference's own C
cannot be compiled where the benchmark runs).
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
METRIC = "collisions/s on 1 GB300 (batched systems)"
UNIT = "collisions/s"
XS, Q = 0.5, 0.7142857


def _load_edmd():
    import importlib.util
    key = "edmd_gb300_edmd"
    if key in sys.modules:
        return sys.modules[key]
    spec = importlib.util.spec_from_file_location(key, os.path.join(ROOT, "graphical-edmd_gb300", "edmd.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[key] = mod
    spec.loader.exec_module(mod)
    return mod


def batched_params(nsys, seed, rank):
    rng = np.random.default_rng(seed + 7919 * rank)
    Ns = rng.integers(256, 4097, nsys)
    phis = rng.uniform(0.30, 0.75, nsys)
    seeds = seed + rank * nsys + np.arange(nsys)
    return [(int(n), float(p), int(s)) for n, p, s in zip(Ns, phis, seeds)]


# ------------------------------------------------------------------ CPU side

def _cpu_worker(conn, params, coll):
    """One reference-semantics system per process (the oracle), single-threaded."""
    from oracle import oracle as orc
    N, phi, seed, hex_ = params
    if hex_:
        o = orc.Oracle(N=N, phi=phi, seed=seed, start=orc.HEX, tmax=1e30)
    else:
        o = orc.Oracle(N=N, phi=phi, seed=seed, start=orc.GROW, xs=XS, q=Q, tmax=1e30)
        vr = orc.load().orc_vr(o.h)
        o.run(10 ** 12, t_stop=1 / vr + 1e-9, cap=1)         # growth phase, untimed
    conn.send("ready")
    while True:
        msg = conn.recv()
        if msg == "stop":
            break
        t0 = time.perf_counter()
        _, n = o.run(coll, cap=1)
        conn.send((n, time.perf_counter() - t0))


class CpuPool:
    def __init__(self, params, coll):
        ctx = mp.get_context("spawn")
        self.p = []
        for prm in params:
            a, b = ctx.Pipe()
            pr = ctx.Process(target=_cpu_worker, args=(b, prm, coll), daemon=True)
            pr.start()
            self.p.append((pr, a))
        for _, a in self.p:
            assert a.recv() == "ready"

    def step(self):
        t0 = time.perf_counter()
        for _, a in self.p:
            a.send("go")
        res = [a.recv() for _, a in self.p]
        wall = time.perf_counter() - t0
        return sum(r[0] for r in res), wall, sum(r[0] / r[1] for r in res)

    def close(self):
        for pr, a in self.p:
            a.send("stop")
            pr.join(timeout=10)


def cpu_sample_params(workload, ncores, seed):
    if workload == "plain_small":
        return [(2000, 0.70, seed + k, True) for k in range(ncores)]
    return [(n, p, s, False) for n, p, s in batched_params(ncores, seed, 0)]


# ------------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0])); mx.append(float(f[1]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ distributed plumbing

def dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist.get_rank(), dist.get_world_size(), dist


def barrier(dist):
    if dist:
        dist.barrier()


def max_over_ranks(dist, v):
    if not dist:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v):
    if not dist:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------ reference arm

def run_reference(a, rank, world, dist):
    if rank != 0:
        return 0
    ncores = os.cpu_count() or 1
    coll = a.ref_coll
    pool = CpuPool(cpu_sample_params(a.workload, ncores, a.seed), coll)
    for _ in range(a.warmup):
        pool.step()
    tot, wall = 0, 0.0
    for _ in range(a.steps):
        n, w, _ = pool.step()
        tot += n; wall += w
    pool.close()
    v = tot / wall
    line = {"impl": "reference", "metric": METRIC if a.workload == "batched" else "collisions/s on 1 GB300 (plain single system)",
            "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1000 * wall / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": a.workload, "sample": f"{ncores} systems, one per process, "
                                                         f"{coll} collisions each per step"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": f"{ncores} processes x {coll} collisions per step, oracle restatement "
                                       f"(-O2 IEEE), growth untimed"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm

def build_systems(edmd, a, rank):
    systems = []
    if a.workload == "plain_small":
        for k in range(a.nsys):
            s = edmd.hex_start(2000, 0.70, a.seed + rank * a.nsys + k)
            s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"], 0.0, 1e30)
            systems.append(s)
        return systems
    for N, phi, seed in batched_params(a.nsys, a.seed, rank):
        s = edmd.grow_start(N, phi, seed, xs=XS, q=Q)
        s["desc"] = edmd.default_desc(N, s["Lx"], s["Ly"], s["vr_base"], 1e30)
        systems.append(s)
    return systems


def run_ours(a, rank, world, dist):
    cpu_pool = None
    ncores = os.cpu_count() or 1
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        # spawn the CPU-baseline processes before the first GPU call
        cpu_pool = CpuPool(cpu_sample_params(a.workload, ncores, a.seed), a.cpu_coll)
    edmd = _load_edmd()
    L = edmd.load()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        L.edmd_set_device(dev)
    systems = build_systems(edmd, a, rank)
    eng = edmd.Engine(systems)
    TN = sum(s["desc"].N for s in systems)
    TC = sum(int(s["desc"].Lx / 2) * int(s["desc"].Ly / 2) for s in systems)
    # set-up: growth phase to completion (untimed), then warm-up steps
    if a.workload == "batched":
        eng.advance(flags=edmd.F_STOP_AT_GROW)
        c = eng.all_counters()
        assert not c["growing"].any(), "growth did not finish"
    for _ in range(a.warmup):
        eng.advance(max_coll=a.coll, flags=edmd.F_COUNT_NORMAL)
    c0 = eng.all_counters()
    clk = ClockSampler(dev)
    barrier(dist)
    clk.start()
    kern_ms = []
    t0 = time.perf_counter()
    for _ in range(a.steps):
        _, ms = eng.advance(max_coll=a.coll, flags=edmd.F_COUNT_NORMAL)
        kern_ms.append(ms)
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    c1 = eng.all_counters()
    ncoll = int((c1["ncol"] - c0["ncol"]).sum())
    npair = int((c1["npair"] - c0["npair"]).sum())
    npred = int((c1["npred"] - c0["npred"]).sum())
    t_dev = sum(kern_ms) / 1000.0
    t_max = max_over_ranks(dist, t_dev)
    coll_all = sum_over_ranks(dist, ncoll)
    value = coll_all / t_max
    # ---- end to end through the C ABI with pinned host buffers
    eng.sync()
    st = eng.states()
    pin = {k: edmd.PinnedArray(TN) for k in ("x", "y", "vx", "vy", "rad", "m")}
    for k in pin:
        pin[k].a[:] = st[k]
    outs = {k: pin[k].a for k in pin}
    e2e_steps = max(1, min(a.steps, 3))
    barrier(dist)
    t0 = time.perf_counter()
    e2e_coll = 0
    for _ in range(e2e_steps):
        eng.load_state(*(pin[k].a for k in ("x", "y", "vx", "vy", "rad", "m")))
        eng.advance(max_coll=a.coll, flags=edmd.F_COUNT_NORMAL)
        eng.sync()
        eng.states(outs)
        e2e_coll += a.coll * len(systems)
    e2e_wall = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = sum_over_ranks(dist, e2e_coll) / e2e_wall
    for p in pin.values():
        p.free()
    h2d = TN * (64 + 12) + TC * 4 + len(systems) * 176
    d2h = TN * 6 * 8 + len(systems) * 4
    eng.close()
    if rank != 0:
        if cpu_pool:
            cpu_pool.close()
        return 0
    cpu = None
    if cpu_pool:
        n, w, rate = cpu_pool.step()
        cpu_pool.close()
        cpu = {"value": n / w, "unit": UNIT, "cores": ncores, "kind": "port",
               "sample": f"{ncores} systems of the same workload, one per process, {a.cpu_coll} collisions "
                         f"each, oracle restatement (-O2 IEEE), growth untimed"}
    # roofline: algorithmic bytes per collision B = P_pair*S + P_pred*(S+24) + 4*S,
    # S = 48 B (x, y, vx, vy, t, r in FP64) -- see the design doc
    S = 48
    p_pair = npair / max(ncoll, 1)
    p_pred = npred / max(ncoll, 1)
    Bcoll = p_pair * S + p_pred * (S + 24) + 4 * S
    achieved = Bcoll * ncoll / t_dev / 1e9
    peak = json.load(open(PEAKS))["hbm_gbs"] if os.path.exists(PEAKS) else 6800.0
    line = {
        "metric": METRIC if a.workload == "batched" else "collisions/s on 1 GB300 (plain single system)",
        "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1000 * t_max / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload if a.workload != "batched" else
                   "batched: 4096 systems/GPU, N~U[256,4096], phi~U[0.30,0.75], bidisperse 1.0/1.4, growth start",
                   "systems_per_gpu": len(systems), "disks_per_gpu": TN,
                   "collisions_per_system_per_step": a.coll,
                   "l2": "state (~%.0f MB/GPU) larger than L2, no flush" % (TN * 160 / 1e6),
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "edmd_load_state (pinned host) + edmd_advance + edmd_get_states (pinned host)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "kernel": "k_run",
                     "bytes_per_collision": Bcoll, "p_pair": p_pair, "p_pred": p_pred,
                     "peak_source": "measured hbm_gbs" if os.path.exists(PEAKS) else "fallback"},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": a.steps,
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "plain_small"])
    ap.add_argument("--nsys", type=int, default=None)
    ap.add_argument("--coll", type=int, default=100000)
    ap.add_argument("--cpu-coll", type=int, default=1000000)
    ap.add_argument("--ref-coll", type=int, default=300000)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    a = ap.parse_args()
    if a.nsys is None:
        a.nsys = 4096 if a.workload == "batched" else 1
    if a.warmup < 3 and a.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    rank, world, dist = dist_init(a.gpus)
    if a.impl == "reference":
        return run_reference(a, rank, world, dist)
    return run_ours(a, rank, world, dist)


if __name__ == "__main__":
    sys.exit(main())
