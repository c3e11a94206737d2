#!/usr/bin/env python
"""Throughput benchmark of the GB300 event-driven hard-disk engine.

Metric: accepted pair collisions per second on one GB300 (the reference's
``ncol`` increments, src/EDMD.c:3558; growth-phase collisions excluded).

Workloads (``--workload``):
  batched       (default) 4096 independent periodic systems, N uniform in
                [256, 4096], area fraction uniform in [0.30, 0.75], 50:50
                bidisperse diameters 1.0/1.4 (-x 0.5 -q 0.7142857), per-system
                seeds, the reference's growth start (untimed set-up), then one
                step = 10^5 accepted collisions per system.  Serial-exact warp
                engine by default (one persistent launch per step).
  single_large  one Hex system of 10^6 monodisperse disks at phi = 0.72,
                10^5 equilibration collisions (untimed), one step = 2*10^7
                collisions in the round-parallel engine (exact mode).
  single_4m     the same at 4*10^6 disks and phi = 0.78 (one step = 10^8
                collisions), the scale of the precision configuration, run in
                full FP64.
  plain_small   one 1980-disk Hex system at phi = 0.70, one step = 10^5
                collisions, serial-exact warp engine (the plain GPU path).
Data are synthetic (the reference has no dataset).  The batched state
(~1.4 GB) and the single_large state (~0.2 GB) are larger than L2, so no
flush is needed between steps.

The JSON line carries the device-resident throughput (``value``), the
end-to-end throughput through the C ABI with host buffers (``e2e``: restart
from pinned host state, run, read the state back), the roofline of the run
kernels, the CPU baseline (the oracle restatement on the host cores) and the SM
clocks sampled during the timed region.  The default run also measures the
single_large workload and reports it under ``other_workloads``.
``--impl reference`` times the reference algorithm on the host cores (the
oracle restatement; the reference's own C cannot be compiled where the
benchmark runs).
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
UNIT = "collisions/s"
XS, Q = 0.5, 0.7142857
METRICS = {
    "batched": "collisions/s on 1 GB300 (batched systems)",
    "single_large": "collisions/s on 1 GB300 (single 10^6-disk system, round-parallel)",
    "single_4m": "collisions/s on 1 GB300 (single 4*10^6-disk system, phi 0.78, round-parallel)",
    "plain_small": "collisions/s on 1 GB300 (plain single system)",
}
DEFAULT_COLL = {"batched": 100000, "single_large": 20000000, "single_4m": 100000000, "plain_small": 100000}
DEFAULT_ENGINE = {"batched": "warp", "single_large": "round", "single_4m": "round", "plain_small": "warp"}
LARGE_N, LARGE_PHI, LARGE_EQUIL = 1000000, 0.72, 100000
SINGLE = {"single_large": (LARGE_N, LARGE_PHI), "single_4m": (4000000, 0.78)}


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
    N, phi, seed, kind = params
    if kind == "hex":
        o = orc.Oracle(N=N, phi=phi, seed=seed, start=orc.HEX, tmax=1e30)
        if N >= LARGE_N:
            o.run(LARGE_EQUIL, cap=1)                          # equilibration, untimed
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
        return [(2000, 0.70, seed + k, "hex") for k in range(ncores)]
    if workload in SINGLE:
        return [(SINGLE[workload][0], SINGLE[workload][1], seed, "hex")]   # one system: one thread
    return [(n, p, s, "grow") for n, p, s in batched_params(ncores, seed, 0)]


def cpu_sample_coll(workload, a):
    return a.cpu_coll if workload not in SINGLE else 2000000


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

def describe_workload(workload, systems, TN):
    """The workload named in both arms' config."""
    if workload == "batched":
        return ("batched: %d systems/GPU, N~U[256,4096], phi~U[0.30,0.75], bidisperse 1.0/1.4, growth start"
                % systems)
    if workload == "single_large":
        return "single Hex system, N=%d, phi=%.2f, %d equilibration collisions" % (TN, LARGE_PHI, LARGE_EQUIL)
    if workload == "single_4m":
        return ("single Hex system, N=%d, phi=%.2f, %d equilibration collisions, full FP64"
                % (TN, SINGLE["single_4m"][1], LARGE_EQUIL))
    return "single Hex system, N=1980, phi=0.70"


def run_reference(a, rank, world, dist):
    if rank != 0:
        return 0
    ncores = os.cpu_count() or 1
    coll = a.ref_coll if a.workload not in SINGLE else 2000000
    params = cpu_sample_params(a.workload, ncores, a.seed)
    pool = CpuPool(params, coll)
    for _ in range(a.warmup):
        pool.step()
    tot, wall = 0, 0.0
    for _ in range(a.steps):
        n, w, _ = pool.step()
        tot += n; wall += w
    pool.close()
    v = tot / wall
    sample = (f"{len(params)} systems of the workload, one per process, {coll} collisions each per step, "
              f"oracle restatement (-O2 IEEE), set-up untimed")
    line = {"impl": "reference", "metric": METRICS[a.workload],
            "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1000 * wall / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": describe_workload(a.workload, a.nsys or (4096 if a.workload == "batched" else 1),
                                                     SINGLE[a.workload][0] if a.workload in SINGLE else None),
                       "sample": sample},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": len(params), "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm

def build_systems(edmd, workload, nsys, seed, rank):
    systems = []
    if workload == "plain_small":
        for k in range(nsys):
            s = edmd.hex_start(2000, 0.70, seed + rank * nsys + k)
            s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"], 0.0, 1e30)
            systems.append(s)
        return systems
    if workload in SINGLE:
        s = edmd.hex_start(SINGLE[workload][0], SINGLE[workload][1], seed + rank)
        s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"], 0.0, 1e30)
        return [s]
    for N, phi, sd in batched_params(nsys, seed, rank):
        s = edmd.grow_start(N, phi, sd, xs=XS, q=Q)
        s["desc"] = edmd.default_desc(N, s["Lx"], s["Ly"], s["vr_base"], 1e30)
        systems.append(s)
    return systems


class Stepper:
    """One timed step of a workload through the engine selected for it."""

    def __init__(self, edmd, eng, engine, coll, radius):
        self.edmd, self.eng, self.engine, self.coll, self.radius = edmd, eng, engine, coll, radius
        self.launches = 0

    def step(self):
        if self.engine == "round":
            _, ms, rounds, _ = self.eng.advance_rounds(max_coll=self.coll, radius=self.radius,
                                                       flags=self.edmd.F_EXACT)
            self.launches += 6 * rounds + 4
            return ms
        _, ms = self.eng.advance(max_coll=self.coll, flags=self.edmd.F_COUNT_NORMAL)
        self.launches += 1
        return ms


def measure(edmd, a, workload, engine, coll, steps, warmup, rank, world, dist, dev, e2e_steps):
    nsys = a.nsys if a.nsys is not None else (4096 if workload == "batched" else 1)
    systems = build_systems(edmd, workload, nsys, a.seed, rank)
    edmd.set_warp_group(a.warp_group)
    eng = edmd.Engine(systems, engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
    TN = sum(s["desc"].N for s in systems)
    TC = sum(int(s["desc"].Lx / 2) * int(s["desc"].Ly / 2) for s in systems)
    # untimed set-up: growth phase, or equilibration of the large system
    if workload == "batched":
        eng.advance(flags=edmd.F_STOP_AT_GROW)
        c = eng.all_counters()
        assert not c["growing"].any(), "growth did not finish"
    elif workload in SINGLE:
        eng.advance_rounds(max_coll=LARGE_EQUIL, radius=a.radius, flags=edmd.F_EXACT)
    st = Stepper(edmd, eng, engine, coll, a.radius)
    for _ in range(warmup):
        st.step()
    c0 = eng.all_counters()
    clk = ClockSampler(dev)
    barrier(dist)
    clk.start()
    st.launches = 0
    kern_ms = []
    t0 = time.perf_counter()
    for _ in range(steps):
        kern_ms.append(st.step())
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    launches = st.launches
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
    stt = eng.states()
    pin = {k: edmd.PinnedArray(TN) for k in ("x", "y", "vx", "vy", "rad", "m")}
    for k in pin:
        pin[k].a[:] = stt[k]
    outs = {k: pin[k].a for k in pin}
    barrier(dist)
    t0 = time.perf_counter()
    e2e_coll = 0
    for _ in range(e2e_steps):
        ca = eng.all_counters()["ncol"].sum()
        eng.load_state(*(pin[k].a for k in ("x", "y", "vx", "vy", "rad", "m")))
        cb = eng.all_counters()["ncol"].sum()
        st.step()
        e2e_coll += int(eng.all_counters()["ncol"].sum() - cb)
        eng.sync()
        eng.states(outs)
    e2e_wall = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = sum_over_ranks(dist, e2e_coll) / e2e_wall
    for p in pin.values():
        p.free()
    h2d = TN * 6 * 8
    d2h = TN * 6 * 8
    eng.close()
    # roofline: algorithmic bytes per collision B = P_pair*S + P_pred*(S+24) + 4*S,
    # S = 48 B (x, y, vx, vy, t, r in FP64)
    S = 48
    p_pair = npair / max(ncoll, 1)
    p_pred = npred / max(ncoll, 1)
    Bcoll = p_pair * S + p_pred * (S + 24) + 4 * S
    achieved = Bcoll * ncoll / t_dev / 1e9
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    # DRAM bytes per accepted collision of k_run from one ncu capture of a
    # 2000-collision step of the batched workload (dram__bytes_read.sum +
    # dram__bytes_write.sum = 41.51 + 5.54 GB for 8.192e6 collisions), scaled
    # to a launch; the same capture gives the FP64 pipe's busy fraction, the
    # resource that bounds this kernel
    traffic = 5744.0 * ncoll / steps if engine == "warp" else None
    kernel = ("k_run (one persistent launch per step)" if engine == "warp" else
              "k_lane_run" if engine == "lane" else
              "round engine graph: k_select + k_process + k_recompute + k_barrier per round")
    return dict(value=value, ms_per_step=1000 * t_max / steps, wall=wall, clocks=clocks, launches=launches,
                systems=len(systems), TN=TN, e2e=e2e, h2d=h2d, d2h=d2h,
                roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": traffic, "kernel": kernel,
                          "traffic_source": ("ncu capture of a 2000-collision step, 5.74 KB per collision "
                                             "(profiles/warp_k_run_batched.md), scaled to the launch"
                                             if traffic else None),
                          "fp64_pipe_active": 0.558 if engine == "warp" else None,
                          "bytes_per_collision": Bcoll, "p_pair": p_pair, "p_pred": p_pred,
                          "peak_source": "measured hbm_gbs" if "hbm_gbs" in peaks else "fallback"})


def measure_differentiation(edmd, ncoll=10000):
    """The tangent and adjoint forms on one 1024-disk Hex system at phi = 0.60:
    32 tangent vectors re-orthonormalised every 100 collisions (Lyapunov
    spectrum), and the adjoint of the final mean-square displacement with
    checkpoints every 500 collisions.  Accepted collisions per second of each
    call, host-timed around the synchronous C-ABI call."""
    try:
        s = edmd.hex_start(1024, 0.60, 11)
        s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
        eng = edmd.Engine([s])
        eng.advance(max_coll=2000)                       # untimed: leave the lattice
        eng.tangent(32, 1000, qr_every=100, seed=17)     # warm-up
        t0 = time.perf_counter()
        _, lam = eng.tangent(32, ncoll, qr_every=100, seed=17)
        t_tan = time.perf_counter() - t0
        eng.msd_gradient(1000, ckpt_every=500)           # warm-up
        t0 = time.perf_counter()
        eng.msd_gradient(ncoll, ckpt_every=500)
        t_adj = time.perf_counter() - t0
        eng.close()
        return {"config": "single Hex system, N=1024, phi=0.60, %d collisions per call" % ncoll,
                "tangent": {"metric": "collisions/s, 32 tangent vectors, CholQR2 every 100 collisions",
                            "value": ncoll / t_tan, "unit": UNIT, "lambda_max": float(lam.max())},
                "adjoint": {"metric": "collisions/s, adjoint of the final MSD (forward + reverse), "
                                      "checkpoints every 500 collisions",
                            "value": ncoll / t_adj, "unit": UNIT},
                "timing": "host wall clock around the synchronous call"}
    except Exception as e:                               # the main line stands without it
        return {"error": repr(e)[:200]}


def run_ours(a, rank, world, dist):
    cpu_pool = None
    ncores = os.cpu_count() or 1
    workload = a.workload
    engine = a.engine if a.engine != "auto" else DEFAULT_ENGINE[workload]
    coll = a.coll if a.coll is not None else DEFAULT_COLL[workload]
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        # spawn the CPU-baseline processes before the first GPU call
        cpu_pool = CpuPool(cpu_sample_params(workload, ncores, a.seed), cpu_sample_coll(workload, a))
    edmd = _load_edmd()
    L = edmd.load()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        L.edmd_set_device(dev)
    r = measure(edmd, a, workload, engine, coll, a.steps, a.warmup, rank, world, dist, dev,
                max(1, min(a.steps, 3)))
    other = {}
    if workload == "batched" and not a.no_secondary:
        s = measure(edmd, a, "single_large", "round", DEFAULT_COLL["single_large"], 3, 3, rank, world,
                    dist, dev, 1)
        other["single_large"] = {"metric": METRICS["single_large"], "value": s["value"], "unit": UNIT,
                                 "engine": "round (exact mode, radius %d)" % a.radius,
                                 "ms_per_step": s["ms_per_step"], "e2e": s["e2e"],
                                 "roofline": s["roofline"], "clocks": s["clocks"],
                                 "gpu_launches": s["launches"]}
        other["differentiation"] = measure_differentiation(edmd)
    if rank != 0:
        if cpu_pool:
            cpu_pool.close()
        return 0
    cpu = None
    if cpu_pool:
        n, w, rate = cpu_pool.step()
        cpu_pool.close()
        nproc = len(cpu_pool.p)
        cpu = {"value": n / w, "unit": UNIT, "cores": nproc, "kind": "port",
               "sample": f"{nproc} system(s) of the same workload, one per process, "
                         f"{cpu_sample_coll(workload, a)} collisions each, oracle restatement (-O2 IEEE), "
                         f"set-up untimed"}
    workload_desc = describe_workload(workload, r["systems"], r["TN"])
    line = {
        "metric": METRICS[workload], "value": r["value"], "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc, "engine": engine, "systems_per_gpu": r["systems"],
                   "disks_per_gpu": r["TN"], "collisions_per_system_per_step": coll,
                   "l2": "state (~%.0f MB/GPU) larger than L2, no flush" % (r["TN"] * 160 / 1e6),
                   "parallelism": f"replicas x{world}",
                   "lanes_per_system": a.warp_group if engine == "warp" else None},
        "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"],
                "path": "edmd_load_state (pinned host) + advance + edmd_sync + edmd_get_states (pinned host)"},
        "roofline": r["roofline"],
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
        "gpu_launches": r["launches"],
        "wall_s": r["wall"],
    }
    if other:
        line["other_workloads"] = other
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "single_large", "single_4m", "plain_small"])
    ap.add_argument("--engine", default="auto", choices=["auto", "warp", "lane", "round"])
    ap.add_argument("--radius", type=int, default=4)
    ap.add_argument("--nsys", type=int, default=None)
    ap.add_argument("--coll", type=int, default=None)
    ap.add_argument("--cpu-coll", type=int, default=1000000)
    ap.add_argument("--ref-coll", type=int, default=300000)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--warp-group", type=int, default=32, choices=[16, 32],
                    help="warp engine lanes per system (16: two systems per warp)")
    a = ap.parse_args()
    if a.warmup < 3 and a.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    rank, world, dist = dist_init(a.gpus)
    if a.impl == "reference":
        return run_reference(a, rank, world, dist)
    return run_ours(a, rank, world, dist)


if __name__ == "__main__":
    sys.exit(main())
