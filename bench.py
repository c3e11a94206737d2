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
                collisions, round-parallel engine in exact mode (measured
                4x the serial-exact warp engine's rate; --engine warp for
                that one).
Data are synthetic (the reference has no dataset).  The batched state
(~1.4 GB) and the single_4m state (~0.6 GB) are more than twice the L2 size
and are not flushed; smaller states (the 1980-disk system, the single_large
state at ~0.16 GB, the single-system differentiation form) get an L2 flush
before every timed call, outside the device-timed region.

The JSON line carries the device-resident throughput (``value``), the
end-to-end throughput through the C ABI with host buffers (``e2e``: restart
from pinned host state, run, read the state back), the roofline of the run
kernels, the CPU baseline (the oracle restatement on the host cores) and the SM
clocks sampled during the timed region.  The default run also measures the
single_large workload and the differentiation forms, each with its own CPU
baseline, and reports them under ``other_workloads``.

CPU baselines run the oracle restatement (bit-identical to the reference's C),
one system per process at a time on every usable host core
(``os.sched_getaffinity``).  The batched sample is stratified: one system per
cell of an 8 x 8 grid over (N, phi) of the 4096-system workload, weighted by
the cell's share; the aggregate is cores / (weighted mean time per collision),
the rate at which the cores would get through the whole batch.

``--impl reference`` times the same CPU path as the reference arm.  With
``--gpus N`` (N > 1) outside torchrun, the script re-launches itself under
``torch.distributed.run`` with N ranks, one GPU each.
"""
import argparse
import json
import multiprocessing as mp
import os
import socket
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
DEFAULT_ENGINE = {"batched": "warp", "single_large": "round", "single_4m": "round", "plain_small": "round"}
# window radius of the round engine: 3 for the small system (~1.5x the
# collisions a round of 4 gives, no replays), 4 for the large ones (3 gives
# them no more collisions a round, and its rarer causality violations
# replay whole calls)
DEFAULT_RADIUS = {"batched": 4, "single_large": 4, "single_4m": 4, "plain_small": 3}
LARGE_N, LARGE_PHI, LARGE_EQUIL = 1000000, 0.72, 100000
SINGLE = {"single_large": (LARGE_N, LARGE_PHI), "single_4m": (4000000, 0.78)}
DIFF_N, DIFF_PHI, DIFF_SEED, DIFF_COLL = 1024, 0.60, 11, 10000

# DRAM traffic and FP64-pipe activity of the dominant kernel, from one ncu
# capture of the configuration they belong to; reported only for that
# configuration (workload, engine, lanes per system)
PROFILED = {
    ("batched", "warp", 32): dict(
        kernel="k_run<32, false>", dram_bytes_per_collision=5765.0, fp64_pipe_active=0.543,
        capture="ncu --set full --clock-control none -k regex:k_run -s 4 -c 1 python bench.py --workload batched "
                "--nsys 4096 --coll 2000 --steps 1 --warmup 3 --no-cpu-baseline --no-secondary --no-tune "
                "(dram__bytes_read.sum + dram__bytes_write.sum = 47.23 GB for 8.192e6 collisions)"),
    ("single_large", "round", None): dict(
        kernel="k_select<4> + k_process + k_recompute_barrier", dram_bytes_per_collision=4990.0,
        fp64_pipe_active=0.606,
        capture="ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --cache-control none "
                "--clock-control none -k regex:'k_select|k_process$|k_recompute_barrier' -s 480 -c 60 python bench.py "
                "--workload single_large --coll 300000 --steps 1 --warmup 3 --no-cpu-baseline --no-secondary "
                "(20 rounds in the middle of a call, warm caches: 19.76 MB per round, over the workload's mean "
                "of 3960 collisions per round; FP64 pipe of k_process from one --set full capture of a round)"),
}


def usable_cores():
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def _load_pkg(name):
    """A module of the engine package (graphical-edmd_gb300/<name>.py)."""
    import importlib.util
    key = "edmd_gb300_" + name
    if key in sys.modules:
        return sys.modules[key]
    spec = importlib.util.spec_from_file_location(key, os.path.join(ROOT, "graphical-edmd_gb300", name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[key] = mod
    spec.loader.exec_module(mod)
    return mod


def _load_edmd():
    """The engine's Python binding; EDMD_BENCH_ENGINE_MODULE names a stand-in
    module with the same interface (used by the CPU test of the multi-rank
    launch, which has no GPU)."""
    import importlib.util
    key = "edmd_gb300_edmd"
    if key in sys.modules:
        return sys.modules[key]
    path = os.environ.get("EDMD_BENCH_ENGINE_MODULE") or os.path.join(ROOT, "graphical-edmd_gb300", "edmd.py")
    spec = importlib.util.spec_from_file_location(key, path)
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


def stratified_sample(params, nb_n=8, nb_phi=8):
    """One system per cell of an nb_n x nb_phi grid over (N, phi) -- the first
    system of the workload in that cell -- with the cell's share of the
    workload as its weight."""
    cells = {}
    for N, phi, sd in params:
        bn = min(nb_n - 1, int((N - 256) * nb_n / (4097 - 256)))
        bp = min(nb_phi - 1, max(0, int((phi - 0.30) * nb_phi / 0.45)))
        cells.setdefault((bn, bp), []).append((N, phi, sd))
    return [(m[0], len(m) / len(params)) for _, m in sorted(cells.items())]


# ------------------------------------------------------------------ CPU side

def _cpu_worker(conn, systems, coll):
    """Reference-semantics systems (the oracle), single-threaded, one process."""
    from oracle import oracle as orc
    objs = []
    for (N, phi, seed, kind, w) in systems:
        if kind == "hex":
            o = orc.Oracle(N=N, phi=phi, seed=seed, start=orc.HEX, tmax=1e30)
            if N >= LARGE_N:
                o.run(LARGE_EQUIL, cap=1)                      # equilibration, untimed
        else:
            o = orc.Oracle(N=N, phi=phi, seed=seed, start=orc.GROW, xs=XS, q=Q, tmax=1e30)
            vr = orc.load().orc_vr(o.h)
            o.run(10 ** 12, t_stop=1 / vr + 1e-9, cap=1)     # growth phase, untimed
        objs.append((o, w))
    conn.send("ready")
    while True:
        msg = conn.recv()
        if msg == "stop":
            break
        res = []
        for o, w in objs:
            t0 = time.perf_counter()
            _, n = o.run(coll, cap=1)
            res.append((n, time.perf_counter() - t0, w))
        conn.send(res)


class CpuPool:
    """Processes over the usable host cores, each holding a share of the
    sample's systems (built untimed).  step() runs every system `coll`
    collisions and returns (collisions, wall seconds, aggregate rate), the
    aggregate being cores / (weighted mean seconds per collision)."""

    def __init__(self, systems, coll, ncores):
        ctx = mp.get_context("spawn")
        self.nproc = max(1, min(ncores, len(systems)))
        self.coll = coll
        self.nsys = len(systems)
        self.p = []
        for k in range(self.nproc):
            a, b = ctx.Pipe()
            pr = ctx.Process(target=_cpu_worker, args=(b, systems[k::self.nproc], coll), daemon=True)
            pr.start()
            self.p.append((pr, a))
        for _, a in self.p:
            assert a.recv() == "ready"

    def step(self):
        t0 = time.perf_counter()
        for _, a in self.p:
            a.send("go")
        res = [r for _, a in self.p for r in a.recv()]
        wall = time.perf_counter() - t0
        wsum = sum(w for _, _, w in res)
        tau = sum(w * dt / max(n, 1) for n, dt, w in res) / wsum
        return sum(n for n, _, _ in res), wall, self.nproc / tau

    def close(self):
        for pr, a in self.p:
            try:
                a.send("stop")
            except (BrokenPipeError, OSError):
                pass
            pr.join(timeout=10)


def cpu_sample(workload, ncores, seed):
    """Systems (N, phi, seed, start, weight) of the CPU sample of a workload."""
    if workload == "plain_small":
        return [(2000, 0.70, seed + k, "hex", 1.0) for k in range(ncores)]
    if workload in SINGLE:
        return [(SINGLE[workload][0], SINGLE[workload][1], seed, "hex", 1.0)]   # one system: one thread
    return [(n, p, s, "grow", w) for (n, p, s), w in stratified_sample(batched_params(4096, seed, 0))]


def cpu_sample_coll(workload, a):
    if workload in SINGLE:
        return 2000000
    return a.cpu_coll if workload == "batched" else 1000000


def describe_sample(pool, workload, kind="port"):
    what = {"batched": f"{pool.nsys} systems, one per cell of an 8x8 (N, phi) grid over the 4096-system "
                       f"workload, weighted by the cell's share",
            "plain_small": f"{pool.nsys} Hex systems (N=1980, phi=0.70, seeds seed..seed+{pool.nsys - 1})",
            "single_large": "the 10^6-disk Hex system (phi 0.72) after its 10^5 equilibration collisions",
            "single_4m": "the 4*10^6-disk Hex system (phi 0.78) after its 10^5 equilibration collisions"}[workload]
    return (f"{what}; {pool.coll} collisions each per step on {pool.nproc} process(es), one core each; "
            f"oracle restatement (-O2 IEEE, bit-identical to the reference's C); set-up untimed; "
            f"aggregate = cores / weighted mean time per collision")


def cpu_line(pool, workload, n, wall, rate):
    return {"value": rate, "unit": UNIT, "cores": pool.nproc, "kind": "port",
            "sample": describe_sample(pool, workload), "collisions": n, "wall_s": wall}


# ---- CPU comparator of the adjoint: central finite differences of the final MSD

def _diff_base_state():
    """The differentiation configuration: Hex N=1024, phi=0.60, 2000 collisions
    from the lattice (the same state the GPU arm differentiates)."""
    from oracle import oracle as orc
    o = orc.Oracle(N=DIFF_N, phi=DIFF_PHI, seed=DIFF_SEED, start=orc.HEX, tmax=1e30)
    o.run(2000, cap=1)
    o.sync()
    st = o.state()
    Lx, Ly, _, _ = o.box()
    init = {k: st[k].copy() for k in ("x", "y", "vx", "vy", "rad", "m", "type")}
    return init, Lx, Ly


def _msd_after(orc, init, Lx, Ly, ncoll, t_obs=None):
    o = orc.Oracle(arrays=init, Lx=Lx, Ly=Ly, tmax=1e30)
    if t_obs is None:
        o.run(ncoll, cap=1)
        t_obs = o.t
    else:
        o.run(10 ** 12, t_stop=t_obs, cap=1)
    st = o.state()
    x = st["x"] + st["vx"] * (t_obs - st["tl"])
    y = st["y"] + st["vy"] * (t_obs - st["tl"])
    dx = x - init["x"]; dx -= Lx * np.rint(dx / Lx)
    dy = y - init["y"]; dy -= Ly * np.rint(dy / Ly)
    dx -= dx.mean(); dy -= dy.mean()
    return float(np.mean(dx * dx + dy * dy)), t_obs


def _fd_worker(conn, comps, ncoll, eps):
    from oracle import oracle as orc
    init, Lx, Ly = _diff_base_state()
    _, t_obs = _msd_after(orc, init, Lx, Ly, ncoll)
    conn.send("ready")
    if conn.recv() == "stop":
        return
    t0 = time.perf_counter()
    g = []
    for c in comps:
        key, i = ("vx", c) if c < DIFF_N else ("vy", c - DIFF_N)
        m = []
        for sign in (1, -1):
            a = {k: v.copy() for k, v in init.items()}
            a[key][i] += sign * eps
            m.append(_msd_after(orc, a, Lx, Ly, ncoll, t_obs)[0])
        g.append((m[0] - m[1]) / (2 * eps))
    conn.send((len(comps), time.perf_counter() - t0))


def cpu_fd_gradient(ncores, ncoll, ncomp, eps=1e-7):
    """Wall time of the FP64 central-difference gradient of the final MSD with
    respect to the initial velocities (2N components, 2 runs each) on the
    host cores; `ncomp` components are timed and the full gradient's time
    scaled from them when ncomp < 2N."""
    ctx = mp.get_context("spawn")
    comps = list(range(min(ncomp, 2 * DIFF_N)))
    nproc = max(1, min(ncores, len(comps)))
    procs = []
    for k in range(nproc):
        a, b = ctx.Pipe()
        pr = ctx.Process(target=_fd_worker, args=(b, comps[k::nproc], ncoll, eps), daemon=True)
        pr.start()
        procs.append((pr, a))
    return procs, comps


def cpu_fd_finish(procs, comps):
    for _, a in procs:
        assert a.recv() == "ready"
    t0 = time.perf_counter()
    for _, a in procs:
        a.send("go")
    res = [a.recv() for _, a in procs]
    wall = time.perf_counter() - t0
    for pr, _ in procs:
        pr.join(timeout=10)
    full = wall * (2 * DIFF_N) / len(comps)
    return {"gradient_wall_s": full, "timed_components": len(comps), "timed_wall_s": wall,
            "cores": len(procs), "kind": "port",
            "sample": (f"central differences (eps 1e-7) of the final MSD after {DIFF_COLL} collisions, "
                       f"{len(comps)} of the {2 * DIFF_N} velocity components timed, two oracle runs each"
                       + ("" if len(comps) == 2 * DIFF_N else "; full-gradient time scaled from them"))}


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


class L2Flusher:
    """Between timed calls of a workload whose device state is less than
    twice the L2 size, writes a device buffer of twice the L2 size, so that
    no timed call starts from the cache the previous call left warm.  The
    engine's CUDA events bracket its own work only, so the write stays
    outside the device-timed region.  Larger states are not flushed: the
    calls themselves stream more than L2 holds."""

    def __init__(self, dev, state_bytes):
        self.state_mb = state_bytes / 1e6
        self.buf = None
        self.k = 0
        self.l2_mb = None
        self.why = "no CUDA device to torch"
        try:
            import torch
            if torch.cuda.is_available():
                l2 = int(getattr(torch.cuda.get_device_properties(dev), "L2_cache_size", 0) or 0)
                self.why = "torch gives no L2 size"
                if l2 > 0:
                    self.l2_mb = l2 / 1e6
                    if state_bytes < 2 * l2:
                        self.torch = torch
                        self.buf = torch.empty(2 * l2, dtype=torch.uint8, device="cuda:%d" % dev)
        except Exception as e:                             # no CUDA torch: nothing to flush with
            self.buf = None
            self.l2_mb = None
            self.why = "flush buffer unavailable: %s" % repr(e)[:80]

    def __call__(self):
        if self.buf is None:
            return
        self.k += 1
        self.buf.fill_(self.k & 255)
        self.torch.cuda.synchronize(self.buf.device)

    def describe(self):
        if self.buf is not None:
            return ("state (~%.1f MB/GPU) within twice L2 (%.0f MB): L2 flushed before every timed call "
                    "(a %.0f MB device write outside the timed calls)"
                    % (self.state_mb, self.l2_mb, self.buf.numel() / 1e6))
        if self.l2_mb is None:
            return "state (~%.1f MB/GPU); L2 size unknown (%s), no flush" % (self.state_mb, self.why)
        return "state (~%.0f MB/GPU) larger than twice L2 (%.0f MB), no flush" % (self.state_mb, self.l2_mb)


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


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def relaunch_ranks(n):
    """Run this script under torch.distributed.run with n ranks (one GPU each)."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.run(cmd).returncode


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
    ncores = usable_cores()
    coll = a.ref_coll if a.workload not in SINGLE else 2000000
    pool = CpuPool(cpu_sample(a.workload, ncores, a.seed), coll, ncores)
    for _ in range(a.warmup):
        pool.step()
    rates, walls = [], []
    for _ in range(a.steps):
        _, w, r = pool.step()
        rates.append(r); walls.append(w)
    pool.close()
    v = statistics.mean(rates)
    sample = describe_sample(pool, a.workload)
    line = {"impl": "reference", "metric": METRICS[a.workload],
            "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1000 * statistics.mean(walls), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": describe_workload(a.workload, a.nsys or (4096 if a.workload == "batched" else 1),
                                                     SINGLE[a.workload][0] if a.workload in SINGLE else None),
                       "sample": sample},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": pool.nproc, "kind": "port", "sample": sample},
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
        self.rounds = 0
        self.violations = 0
        self.extra_flags = 0

    def step(self):
        if self.engine == "round":
            _, ms, rounds, viol = self.eng.advance_rounds(max_coll=self.coll, radius=self.radius,
                                                          flags=self.edmd.F_EXACT | self.extra_flags)
            self.launches += self.eng.last_launches()
            self.rounds += rounds
            self.violations += viol
            return ms
        _, ms = self.eng.advance(max_coll=self.coll, flags=self.edmd.F_COUNT_NORMAL | self.extra_flags)
        self.launches += self.eng.last_launches()
        return ms


def measure(edmd, a, workload, engine, coll, steps, warmup, rank, world, dist, dev, e2e_steps):
    nsys = a.nsys if a.nsys is not None else (4096 if workload == "batched" else 1)
    radius = a.radius if a.radius is not None else DEFAULT_RADIUS[workload]
    systems = build_systems(edmd, workload, nsys, a.seed, rank)
    edmd.set_warp_group(a.warp_group)
    eng = edmd.Engine(systems, engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
    TN = sum(s["desc"].N for s in systems)
    # untimed set-up: growth phase, or equilibration of the large system
    if workload == "batched":
        eng.advance(flags=edmd.F_STOP_AT_GROW)
        c = eng.all_counters()
        assert not c["growing"].any(), "growth did not finish"
    elif workload in SINGLE:
        eng.advance_rounds(max_coll=LARGE_EQUIL, radius=radius, flags=edmd.F_EXACT)
    tuned = None
    extra = edmd.F_SMEM if (getattr(a, "smem", False) and engine == "warp") else 0
    if workload == "batched" and engine == "warp" and getattr(a, "tune", False):
        # untimed: every candidate engine and launch shape on the grown
        # systems themselves (all give the same trajectories); the timed
        # steps run the fastest
        tune = _load_pkg("tune")
        eng.sync()
        descs = [edmd.default_desc(s["desc"].N, s["desc"].Lx, s["desc"].Ly, 0.0, 1e30) for s in systems]
        grown = tune.systems_from_states(descs, eng.states(), [s["desc"].N for s in systems])
        tuned = tune.tune(edmd, grown, coll=2000)
        if (tuned["engine"], tuned["lanes"]) != ("warp", a.warp_group):
            eng.close()
            if tuned["lanes"] is not None:
                edmd.set_warp_group(tuned["lanes"])
            eng = edmd.Engine(grown, engine=edmd.ENGINE_LANE if tuned["engine"] == "lane" else edmd.ENGINE_WARP)
            engine = tuned["engine"]
        extra = tuned["flags"]
    st = Stepper(edmd, eng, engine, coll, radius)
    if engine == "round" and getattr(a, "round_block", False):
        extra |= edmd.F_ROUND_BLOCK
    st.extra_flags = extra
    for _ in range(warmup):
        st.step()
    flush = L2Flusher(dev, TN * 160)
    c0 = eng.all_counters()
    clk = ClockSampler(dev)
    barrier(dist)
    clk.start()
    st.launches = st.rounds = st.violations = 0
    kern_ms = []
    t0 = time.perf_counter()
    for _ in range(steps):
        flush()
        kern_ms.append(st.step())
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    launches = st.launches
    rounds, violations = st.rounds, st.violations
    c1 = eng.all_counters()
    ncoll = int((c1["ncol"] - c0["ncol"]).sum())
    npair = int((c1["npair"] - c0["npair"]).sum())
    npred = int((c1["npred"] - c0["npred"]).sum())
    t_dev = sum(kern_ms) / 1000.0
    t_max = max_over_ranks(dist, t_dev)
    coll_all = sum_over_ranks(dist, ncoll)
    value = coll_all / t_max
    screen = None
    if workload == "single_4m" and getattr(a, "screen_compare", False):
        screen = compare_screen(edmd, a, systems[0], eng, steps, coll, c1, radius)
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
    lanes_used = (tuned["lanes"] if tuned else a.warp_group) if engine == "warp" else None
    prof = PROFILED.get((workload, engine, lanes_used)) if (a.nsys is None and not extra) else None
    kernel = ("k_run (one persistent launch per step)" if engine == "warp" else
              "k_lane_run" if engine == "lane" else
              "round engine graph: k_select + k_process + k_recompute + k_barrier per round")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": prof["dram_bytes_per_collision"] * ncoll / steps if prof else None,
            "kernel": kernel, "bytes_per_collision": Bcoll, "p_pair": p_pair, "p_pred": p_pred,
            "peak_source": "measured hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"}
    if prof:
        roof.update(traffic_source=("DRAM bytes per accepted collision of %s from one ncu capture of this "
                                    "configuration, scaled to the launch's collisions: %s"
                                    % (prof["kernel"], prof["capture"])),
                    fp64_pipe_active=prof["fp64_pipe_active"],
                    fp64_pipe_source=("sm__pipe_fp64_cycles_active of the same capture" if engine == "warp" else
                                      "sm__pipe_fp64_cycles_active of k_process in a --set full capture"))
    else:
        roof["traffic_source"] = "no ncu capture of this configuration"
    if engine == "round":
        roof["rounds_per_step"] = rounds / steps
        roof["causality_violations_replayed"] = violations
    if screen:
        roof["fp32_screen"] = screen
    return dict(value=value, ms_per_step=1000 * t_max / steps, wall=wall, clocks=clocks, launches=launches,
                engine=engine, lanes=(tuned["lanes"] if tuned else a.warp_group) if engine == "warp" else None,
                l2=flush.describe(), radius=radius if engine == "round" else None,
                smem=bool(extra), tuned=tuned,
                systems=len(systems), TN=TN, e2e=e2e, h2d=h2d, d2h=d2h, roofline=roof)


def _kinetic(st):
    return 0.5 * float(np.sum(st["m"] * (st["vx"] ** 2 + st["vy"] ** 2)))


def compare_screen(edmd, a, sysd, eng_fp64, steps, coll, c_fp64, radius):
    """The precision configuration: the same system, equilibration and timed
    steps again with the FP32 screen of separating pairs (EDMD_F_SCREEN),
    against the all-FP64 run just measured.  Missed collisions show as a
    different collision count or final state (identical states mean the
    FP64 run has the same drift and Z); also reported: the relative energy
    drift over the timed steps and Z = P A / (N kT) from their virial."""
    eng_fp64.sync()
    st64 = eng_fp64.states()
    e2 = edmd.Engine([sysd])
    e2.advance_rounds(max_coll=LARGE_EQUIL, radius=radius, flags=edmd.F_EXACT)
    for _ in range(a.warmup):
        e2.advance_rounds(max_coll=coll, radius=radius, flags=edmd.F_EXACT | edmd.F_SCREEN)
    # velocities only: a free flight of every disk here would change the
    # rounding of the positions and part the two runs
    e_start = _kinetic(e2.states())
    t0 = e2.counters(0)["t"]
    e2.virial(0, reset=True)
    c0 = e2.counters(0)
    ms = 0.0
    for _ in range(steps):
        ms += e2.advance_rounds(max_coll=coll, radius=radius, flags=edmd.F_EXACT | edmd.F_SCREEN)[1]
    c1 = e2.counters(0)
    e2.sync()
    st32 = e2.states()
    vir = e2.virial(0)
    dt = c1["t"] - t0
    E = _kinetic(st32)
    z = 1.0 - (vir[0] + vir[1]) / (2.0 * E * dt) if dt > 0 else None
    same = all(np.array_equal(st32[k], st64[k]) for k in ("x", "y", "vx", "vy"))
    out = {"value": (c1["ncol"] - c0["ncol"]) / (ms / 1000.0), "unit": UNIT,
           "collisions_timed": int(c1["ncol"] - c0["ncol"]), "pairs_screened": int(c1["nscreen"] - c0["nscreen"]),
           "pairs_tested": int(c1["npair"] - c0["npair"]),
           "collisions_total": int(c1["ncol"]), "collisions_total_fp64": int(c_fp64["ncol"].sum()),
           "identical_final_state": bool(same),
           "missed_collisions": abs(int(c1["ncol"]) - int(c_fp64["ncol"].sum())),
           "energy_drift": E / e_start - 1.0, "Z": z, "t_span": dt}
    e2.close()
    return out


def measure_differentiation(edmd, dev=0, ncoll=DIFF_COLL):
    """The tangent and adjoint forms on one 1024-disk Hex system at phi = 0.60
    (2000 collisions from the lattice): 32 tangent vectors re-orthonormalised
    every 100 collisions (Lyapunov spectrum), and the adjoint of the final
    mean-square displacement with checkpoints every 500 collisions.  Each call
    is timed twice: device time (CUDA events on the context's stream around
    the whole call, edmd_get_last_ms) and host wall time."""
    try:
        s = edmd.hex_start(DIFF_N, DIFF_PHI, DIFF_SEED)
        s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
        eng = edmd.Engine([s])
        eng.advance(max_coll=2000)                       # untimed: leave the lattice
        eng.tangent(32, 1000, qr_every=100, seed=17)     # warm-up
        # state and 32 tangent vectors: 1024 disks x (160 + 32 x 32) bytes
        flush = L2Flusher(dev, DIFF_N * (160 + 32 * 32))
        flush()
        t0 = time.perf_counter()
        _, lam = eng.tangent(32, ncoll, qr_every=100, seed=17)
        t_tan = time.perf_counter() - t0
        ms_tan = eng.last_ms()
        eng.msd_gradient(1000, ckpt_every=500)           # warm-up
        flush()
        t0 = time.perf_counter()
        eng.msd_gradient(ncoll, ckpt_every=500)
        t_adj = time.perf_counter() - t0
        ms_adj = eng.last_ms()
        eng.close()
        return {"config": "single Hex system, N=1024, phi=0.60, %d collisions per call" % ncoll,
                "tangent": {"metric": "collisions/s, 32 tangent vectors, CholQR2 every 100 collisions",
                            "value": ncoll / (ms_tan / 1000), "unit": UNIT, "device_ms": ms_tan,
                            "e2e": {"value": ncoll / t_tan, "unit": UNIT, "wall_s": t_tan},
                            "lambda_max": float(lam.max())},
                "adjoint": {"metric": "collisions/s, adjoint of the final MSD (forward + reverse), "
                                      "checkpoints every 500 collisions",
                            "value": ncoll / (ms_adj / 1000), "unit": UNIT, "device_ms": ms_adj,
                            "gradient_wall_s": t_adj,
                            "e2e": {"value": ncoll / t_adj, "unit": UNIT, "wall_s": t_adj}},
                "timing": "value: CUDA events on the context's stream around the call (edmd_get_last_ms); "
                          "e2e: host wall clock around the synchronous C-ABI call",
                "l2": flush.describe()}
    except Exception as e:                               # the main line stands without it
        return {"error": repr(e)[:200]}


def measure_differentiation_batched(edmd, dev=0, nsys=256, ncoll=DIFF_COLL):
    """The differentiation forms batched: nsys replicas of the 1024-disk
    configuration (Hex starts with seeds DIFF_SEED + k, 2000 collisions from
    the lattice), all systems in one context; the tangent form (32 vectors,
    CholQR2 every 100 collisions) and the adjoint of each system's final MSD
    (checkpoints every 500 collisions).  Aggregate accepted collisions of the
    differentiated trajectories per second."""
    try:
        systems = []
        for k in range(nsys):
            s = edmd.hex_start(DIFF_N, DIFF_PHI, DIFF_SEED + k)
            s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
            systems.append(s)
        eng = edmd.Engine(systems)
        eng.advance(max_coll=2000)                       # untimed: leave the lattice
        eng.tangent_batch(32, 200, 100, seed=17)         # warm-up
        flush = L2Flusher(dev, nsys * DIFF_N * (160 + 32 * 32))
        flush()
        t0 = time.perf_counter()
        lam = eng.tangent_batch(32, ncoll, 100, seed=17)
        t_tan = time.perf_counter() - t0
        ms_tan = eng.last_ms()
        eng.msd_gradient_batch(500, ckpt_every=500)      # warm-up
        flush()
        t0 = time.perf_counter()
        eng.msd_gradient_batch(ncoll, ckpt_every=500)
        t_adj = time.perf_counter() - t0
        ms_adj = eng.last_ms()
        eng.close()
        tot = nsys * ncoll
        return {"config": "%d systems, each N=1024, phi=0.60, %d collisions per system per call" % (nsys, ncoll),
                "tangent": {"metric": "aggregate collisions/s, 32 tangent vectors per system, CholQR2 every 100",
                            "value": tot / (ms_tan / 1000), "unit": UNIT, "device_ms": ms_tan,
                            "e2e": {"value": tot / t_tan, "unit": UNIT, "wall_s": t_tan},
                            "lambda_max_mean": float(lam.max(axis=1).mean())},
                "adjoint": {"metric": "aggregate collisions/s, adjoint of each system's final MSD, "
                                      "checkpoints every 500 collisions",
                            "value": tot / (ms_adj / 1000), "unit": UNIT, "device_ms": ms_adj,
                            "gradient_wall_s_per_system": t_adj / nsys,
                            "e2e": {"value": tot / t_adj, "unit": UNIT, "wall_s": t_adj}},
                "timing": "value: CUDA events on the context's stream around the call; e2e: host wall clock",
                "l2": flush.describe()}
    except Exception as e:                               # the main line stands without it
        return {"error": repr(e)[:200]}


def run_ours(a, rank, world, dist):
    ncores = usable_cores()
    workload = a.workload
    engine = a.engine if a.engine != "auto" else DEFAULT_ENGINE[workload]
    coll = a.coll if a.coll is not None else DEFAULT_COLL[workload]
    secondary = workload == "batched" and not a.no_secondary
    pools = {}
    fd = None
    if rank == 0 and not a.no_cpu_baseline:
        # spawn the CPU-baseline processes before the first GPU call
        pools[workload] = CpuPool(cpu_sample(workload, ncores, a.seed), cpu_sample_coll(workload, a), ncores)
        if secondary:
            pools["single_large"] = CpuPool(cpu_sample("single_large", ncores, a.seed),
                                            cpu_sample_coll("single_large", a), 1)
            fd = cpu_fd_gradient(ncores, DIFF_COLL, a.fd_components)
    edmd = _load_edmd()
    L = edmd.load()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        L.edmd_set_device(dev)
    r = measure(edmd, a, workload, engine, coll, a.steps, a.warmup, rank, world, dist, dev,
                max(1, min(a.steps, 3)))
    other = {}
    if secondary:
        s = measure(edmd, a, "single_large", "round", DEFAULT_COLL["single_large"], 3, 3, rank, world,
                    dist, dev, 1)
        other["single_large"] = {"metric": METRICS["single_large"], "value": s["value"], "unit": UNIT,
                                 "engine": "round (exact mode, radius %d)" % s["radius"], "l2": s["l2"],
                                 "ms_per_step": s["ms_per_step"], "e2e": s["e2e"],
                                 "roofline": s["roofline"], "clocks": s["clocks"],
                                 "gpu_launches": s["launches"]}
        other["differentiation"] = measure_differentiation(edmd, dev)
        other["differentiation_batched"] = measure_differentiation_batched(edmd, dev)
    if rank != 0:
        return 0
    cpu = None
    if workload in pools:
        p = pools[workload]
        n, w, rate = p.step()
        p.close()
        cpu = cpu_line(p, workload, n, w, rate)
    if "single_large" in pools and "single_large" in other:
        p = pools["single_large"]
        n, w, rate = p.step()
        p.close()
        other["single_large"]["cpu_baseline"] = cpu_line(p, "single_large", n, w, rate)
    if fd is not None and "differentiation" in other and "adjoint" in other["differentiation"]:
        fdr = cpu_fd_finish(*fd)
        fdr["value"] = DIFF_COLL / fdr["gradient_wall_s"]
        fdr["unit"] = UNIT + " (collisions of the differentiated trajectory per second of gradient time)"
        other["differentiation"]["adjoint"]["cpu_baseline"] = fdr
        if "adjoint" in other.get("differentiation_batched", {}):
            # the CPU computes one system's gradient after another on all cores
            other["differentiation_batched"]["adjoint"]["cpu_baseline"] = dict(
                fdr, sample=fdr["sample"] + "; per system, systems one after another")
    workload_desc = describe_workload(workload, r["systems"], r["TN"])
    line = {
        "metric": METRICS[workload], "value": r["value"], "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc, "engine": r["engine"], "window_radius": r["radius"],
                   "systems_per_gpu": r["systems"],
                   "disks_per_gpu": r["TN"], "collisions_per_system_per_step": coll,
                   "l2": r["l2"],
                   "parallelism": f"replicas x{world}",
                   "lanes_per_system": r["lanes"], "shared_memory_kernel": r["smem"],
                   "tuned": r["tuned"]},
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
    ap.add_argument("--radius", type=int, default=None,
                    help="round engine window radius (default: 3 for plain_small, 4 otherwise)")
    ap.add_argument("--nsys", type=int, default=None)
    ap.add_argument("--coll", type=int, default=None)
    ap.add_argument("--cpu-coll", type=int, default=250000, help="collisions per sampled system (CPU baseline)")
    ap.add_argument("--ref-coll", type=int, default=250000, help="collisions per sampled system (reference arm)")
    ap.add_argument("--fd-components", type=int, default=2 * DIFF_N,
                    help="velocity components timed for the finite-difference gradient")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--smem", action="store_true",
                    help="warp engine: systems that fit a block's shared memory run from there (EDMD_F_SMEM)")
    ap.add_argument("--no-tune", dest="tune", action="store_false",
                    help="batched workload: skip the untimed choice of engine and launch shape")
    ap.add_argument("--round-block", action="store_true",
                    help="round engine: one block per system, rounds between block barriers (EDMD_F_ROUND_BLOCK)")
    ap.add_argument("--screen-compare", action="store_true",
                    help="single_4m: rerun the timed steps with the FP32 screen and compare with the FP64 run")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--warp-group", type=int, default=32, choices=[4, 8, 16, 32],
                    help="warp engine lanes per system (16: two systems per warp, 8: four, 4: eight)")
    a = ap.parse_args()
    if a.warmup < 3 and a.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if a.gpus > 1 and "RANK" not in os.environ:
        return relaunch_ranks(a.gpus)
    rank, world, dist = dist_init(a.gpus)
    if a.impl == "reference":
        return run_reference(a, rank, world, dist)
    return run_ours(a, rank, world, dist)


if __name__ == "__main__":
    sys.exit(main())
