"""Python mirror of the engine's C ABI (include/edmd_gpu.h, include/edmd_host.h).

Thin ctypes layer over ``libedmd_gpu.so`` for the tests and the benchmark; the
product's own host is the C driver ``edmd`` (host/edmd_main.c).  Everything
here goes through the C ABI: there is no Python or CPU fallback, and loading
fails loudly when the library has not been built.

Reference flow being mirrored (src/EDMD.c:498-661):
    constantInit / particlesInit   -> hex_start() / grow_start()   (host C)
    cellListInit / eventListInit   -> Engine(...)                   (edmd_create)
    while (t <= tmax) { ... }      -> Engine.advance(...)           (edmd_advance)
    takeAScreenshot's freeFly-all  -> Engine.sync()                 (edmd_sync)
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libedmd_gpu.so")

OK, ERR_ARG, ERR_CUDA, ERR_OVERLAP, ERR_BUDGET, ERR_CAPACITY, ERR_NODEV = range(7)
STOP_COLL, STOP_TIME, STOP_TMAX, STOP_SCREEN, STOP_GROW = 1, 2, 3, 4, 5
F_STOP_AT_SCREEN, F_STOP_AT_GROW, F_TRACE, F_COUNT_NORMAL, F_LOG, F_EXACT = 1, 2, 4, 8, 16, 32
F_ROUND_GRID, F_ROUND_BLOCK, F_SCREEN, F_ROUND_THREAD, F_ROUND_WARP = 64, 128, 256, 512, 1024
F_SMEM = 2048
ENGINE_AUTO, ENGINE_WARP, ENGINE_LANE = 0, 1, 2


class SystemDesc(C.Structure):
    _fields_ = [("N", C.c_int32), ("Lx", C.c_double), ("Ly", C.c_double), ("res", C.c_double),
                ("Einit", C.c_double), ("first_screen", C.c_double), ("dtime", C.c_double),
                ("first_thermo", C.c_double), ("dtime_thermo", C.c_double),
                ("t_growstop", C.c_double), ("tmax", C.c_double), ("contact", C.c_int32)]


# contact rules (edmd_system_desc.contact): 2 sqrt(r1 r2) or r1 + r2
CONTACT_NONADDITIVE = 0
CONTACT_ADDITIVE = 1


class Collision(C.Structure):
    _fields_ = [("i", C.c_int32), ("j", C.c_int32), ("cell_i", C.c_int32), ("cell_j", C.c_int32),
                ("t", C.c_double)]


LOG_DTYPE = np.dtype([("i", "<i4"), ("j", "<i4"), ("t", "<f8"), ("dx", "<f8"), ("dy", "<f8"),
                      ("dvx", "<f8"), ("dvy", "<f8"), ("f", "<f8")])

COLLISION_DTYPE = np.dtype([("i", "<i4"), ("j", "<i4"), ("cell_i", "<i4"), ("cell_j", "<i4"),
                            ("t", "<f8")])


class Counters(C.Structure):
    _fields_ = [("ncol", C.c_uint64), ("ncol_total", C.c_uint64), ("ncross", C.c_uint64),
                ("nstale", C.c_uint64), ("npair", C.c_uint64), ("npred", C.c_uint64),
                ("nevents", C.c_uint64), ("t", C.c_double), ("growing", C.c_int32),
                ("stop_reason", C.c_int32), ("nscreen", C.c_uint64)]


# every symbol the public headers declare, in declaration order
EXPORTS = [
    "edmd_create", "edmd_load_state", "edmd_advance", "edmd_advance_rounds", "edmd_sync",
    "edmd_get_pcf", "edmd_get_state",
    "edmd_get_states", "edmd_get_counters", "edmd_get_all_counters", "edmd_get_virial",
    "edmd_get_thermo", "edmd_take_thermo", "edmd_get_trace", "edmd_set_engine", "edmd_set_lane_threads",
    "edmd_set_warp_group",
    "edmd_get_engine", "edmd_get_last_ms", "edmd_get_last_launches", "edmd_set_device", "edmd_host_alloc", "edmd_host_free", "edmd_run_noalloc",
    "edmd_set_log_capacity", "edmd_clear_log", "edmd_get_log", "edmd_checkpoint_save",
    "edmd_checkpoint_restore", "edmd_tangent_run", "edmd_msd_gradient", "edmd_tangent_run_batch",
    "edmd_msd_gradient_batch", "edmd_destroy",
    "edmd_last_error", "edmd_device_info",
    "edmd_mt_seed", "edmd_mt_u32", "edmd_mt_double", "edmd_hex_size", "edmd_random_size",
    "edmd_grow_rate", "edmd_normalize", "edmd_init_hex", "edmd_init_grow", "edmd_default_desc",
]

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def load(path=LIB_PATH):
    """Load libedmd_gpu.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; run __graft_entry__.build()")
    L = C.CDLL(path)
    L.edmd_create.argtypes = [C.c_int32, C.POINTER(SystemDesc), _dp, _dp, _dp, _dp, _dp, _dp,
                              C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]
    L.edmd_advance.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.c_uint32, C.c_int64,
                               C.POINTER(C.c_float)]
    L.edmd_load_state.argtypes = [C.c_void_p] + [C.c_void_p] * 6
    L.edmd_advance_rounds.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.c_uint32, C.c_int32,
                                      C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64)]
    L.edmd_get_states.argtypes = [C.c_void_p] + [C.c_void_p] * 6
    L.edmd_get_pcf.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_void_p, C.c_int32,
                               C.POINTER(C.c_int32)]
    L.edmd_get_all_counters.argtypes = [C.c_void_p, C.c_void_p]
    L.edmd_host_alloc.argtypes = [C.POINTER(C.c_void_p), C.c_int64]
    L.edmd_host_free.argtypes = [C.c_void_p]
    L.edmd_set_device.argtypes = [C.c_int32]
    L.edmd_set_engine.argtypes = [C.c_int32]
    L.edmd_set_log_capacity.argtypes = [C.c_void_p, C.c_int64]
    L.edmd_clear_log.argtypes = [C.c_void_p]
    L.edmd_get_log.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
    L.edmd_checkpoint_save.argtypes = [C.c_void_p, C.c_int32]
    L.edmd_checkpoint_restore.argtypes = [C.c_void_p, C.c_int32]
    L.edmd_tangent_run.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_int64, C.c_uint64,
                                   C.c_void_p, C.c_void_p]
    L.edmd_msd_gradient.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_double] + [C.c_void_p] * 5
    L.edmd_tangent_run_batch.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_uint64, C.c_void_p]
    L.edmd_msd_gradient_batch.argtypes = [C.c_void_p, C.c_int64, C.c_int64] + [C.c_void_p] * 5
    L.edmd_run_noalloc.argtypes = [C.POINTER(SystemDesc)] + [C.c_void_p] * 6 + [
        C.c_int64, C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.c_void_p]
    L.edmd_set_lane_threads.argtypes = [C.c_int32]
    L.edmd_set_warp_group.argtypes = [C.c_int32]
    L.edmd_get_engine.argtypes = [C.c_void_p]
    L.edmd_get_last_ms.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    L.edmd_get_last_launches.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.edmd_sync.argtypes = [C.c_void_p]
    L.edmd_get_state.argtypes = [C.c_void_p, C.c_int32] + [C.c_void_p] * 8
    L.edmd_get_counters.argtypes = [C.c_void_p, C.c_int32, C.POINTER(Counters)]
    L.edmd_get_virial.argtypes = [C.c_void_p, C.c_int32, _dp, C.c_int32]
    L.edmd_get_thermo.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
    L.edmd_take_thermo.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
    L.edmd_get_trace.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
    L.edmd_destroy.argtypes = [C.c_void_p]
    L.edmd_last_error.argtypes = [C.c_void_p]
    L.edmd_last_error.restype = C.c_char_p
    L.edmd_device_info.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_int32)]
    L.edmd_mt_seed.argtypes = [C.c_uint32]
    L.edmd_mt_u32.restype = C.c_uint32
    L.edmd_mt_double.restype = C.c_double
    L.edmd_hex_size.argtypes = [C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int),
                                C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.edmd_random_size.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.edmd_grow_rate.argtypes = [C.c_double]
    L.edmd_grow_rate.restype = C.c_double
    L.edmd_normalize.argtypes = [C.c_int, C.c_double, _dp, _dp, _dp]
    L.edmd_init_hex.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint32,
                                _dp, _dp, _dp, _dp, _dp, _dp, _ip,
                                C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.edmd_init_grow.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint32,
                                 _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip,
                                 C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.edmd_default_desc.argtypes = [C.POINTER(SystemDesc), C.c_int, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_double, C.c_double]
    _lib = L
    return L


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"edmd error {code}: {msg}")
        self.code = code


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


# ------------------------------------------------------------------ host init

def hex_start(N, phi, seed, aspect=1.0, Einit=1.0):
    """Triangular-lattice start of the reference (Hex = 1) on the host."""
    L = load()
    arrs = [np.zeros(N) for _ in range(6)]
    typ = np.zeros(N, np.int32)
    Lx, Ly = C.c_double(), C.c_double()
    n = L.edmd_init_hex(N, phi, aspect, Einit, seed, *arrs, typ, C.byref(Lx), C.byref(Ly))
    if n < 0:
        raise EngineError(ERR_ARG, "bad Hex parameters")
    x, y, vx, vy, rad, m = (a[:n].copy() for a in arrs)
    return dict(N=n, Lx=Lx.value, Ly=Ly.value, x=x, y=y, vx=vx, vy=vy, rad=rad, m=m,
                type=typ[:n].copy(), vr=None, vr_base=0.0)


def grow_start(N, phi, seed, xs=0.3, q=0.4, aspect=1.0):
    """Random start with Lubachevsky-Stillinger growth (the reference default)."""
    L = load()
    arrs = [np.zeros(N) for _ in range(7)]
    typ = np.zeros(N, np.int32)
    Lx, Ly, vrb = C.c_double(), C.c_double(), C.c_double()
    L.edmd_init_grow(N, phi, xs, q, aspect, seed, *arrs, typ, C.byref(Lx), C.byref(Ly), C.byref(vrb))
    x, y, vx, vy, rad, m, vr = arrs
    return dict(N=N, Lx=Lx.value, Ly=Ly.value, x=x, y=y, vx=vx, vy=vy, rad=rad, m=m,
                type=typ, vr=vr, vr_base=vrb.value)


def default_desc(N, Lx, Ly, vr_base=0.0, tmax=4000.0, dtime=100.0, dtime_thermo=100.0,
                 contact=CONTACT_NONADDITIVE):
    d = SystemDesc()
    load().edmd_default_desc(C.byref(d), N, Lx, Ly, vr_base, tmax, dtime, dtime_thermo)
    d.contact = contact
    return d


def set_warp_group(lanes):
    """Lanes per system of the warp engine, 4, 8, 16 or 32 (edmd_set_warp_group)."""
    rc = load().edmd_set_warp_group(int(lanes))
    if rc != 0:
        raise ValueError("lanes must be 4, 8, 16 or 32")


# ------------------------------------------------------------------ engine

class Engine:
    """A set of independent systems on the GPU (one edmd_ctx)."""

    def __init__(self, systems, trace_cap=0, engine=ENGINE_AUTO, lane_threads=32):
        """systems: list of dicts with N, x, y, vx, vy, rad, m, [vr] and 'desc'."""
        L = load()
        L.edmd_set_engine(engine)
        L.edmd_set_lane_threads(lane_threads)
        self._L = L
        n = len(systems)
        descs = (SystemDesc * n)(*[s["desc"] for s in systems])
        cat = lambda k: np.ascontiguousarray(np.concatenate([np.asarray(s[k], np.float64) for s in systems]))
        x, y, vx, vy, rad, m = (cat(k) for k in ("x", "y", "vx", "vy", "rad", "m"))
        vr = None
        if any(s.get("vr") is not None for s in systems):
            vr = np.ascontiguousarray(np.concatenate(
                [np.asarray(s["vr"], np.float64) if s.get("vr") is not None else np.zeros(s["desc"].N)
                 for s in systems]))
        h = C.c_void_p()
        rc = L.edmd_create(n, descs, x, y, vx, vy, rad, m, _ptr(vr), int(trace_cap), C.byref(h))
        if h.value is None and rc != OK:
            raise EngineError(rc, "edmd_create failed")
        self.h = h
        self.n = n
        self.N = [s["desc"].N for s in systems]
        self._desc = [s["desc"] for s in systems]
        self.trace_cap = trace_cap
        if rc != OK:
            msg = self.last_error()
            self.close()
            raise EngineError(rc, msg)

    @property
    def engine(self):
        return self._L.edmd_get_engine(self.h)

    def last_error(self):
        return self._L.edmd_last_error(self.h).decode()

    def last_ms(self):
        """Device time of the last advance / round / tangent / adjoint call (edmd_get_last_ms)."""
        ms = C.c_float()
        self._ck(self._L.edmd_get_last_ms(self.h, C.byref(ms)))
        return ms.value

    def last_launches(self):
        """Kernels launched by the last advance or round call (edmd_get_last_launches)."""
        n = C.c_int64()
        self._ck(self._L.edmd_get_last_launches(self.h, C.byref(n)))
        return n.value

    def _ck(self, rc):
        if rc != OK:
            raise EngineError(rc, self.last_error())

    def advance(self, max_coll=2**62, t_stop=float("inf"), flags=0, max_events=2**62, check=True):
        ms = C.c_float()
        rc = self._L.edmd_advance(self.h, int(max_coll), float(t_stop), int(flags), int(max_events),
                                  C.byref(ms))
        if check:
            self._ck(rc)
        return rc, ms.value

    def advance_rounds(self, max_coll=2**62, t_stop=float("inf"), flags=0, radius=3,
                       max_rounds=2**24, check=True):
        """Round-parallel advance; returns (status, ms, rounds, violations)."""
        ms = C.c_float()
        rounds = C.c_int64()
        viol = C.c_int64()
        rc = self._L.edmd_advance_rounds(self.h, int(max_coll), float(t_stop), int(flags), int(radius),
                                         int(max_rounds), C.byref(ms), C.byref(rounds), C.byref(viol))
        if check:
            self._ck(rc)
        return rc, ms.value, rounds.value, viol.value

    def sync(self):
        self._ck(self._L.edmd_sync(self.h))

    def pcf(self, s=0, dr=0.1, max_r=None):
        """(r, g) of calculate_pcf on the stored positions of system s."""
        if max_r is None:
            d = self._desc[s]
            max_r = min(d.Lx, d.Ly) / 2
        cap = int(max_r / dr) + 1
        g = np.zeros(cap)
        nb = C.c_int32()
        self._ck(self._L.edmd_get_pcf(self.h, s, float(dr), float(max_r), _ptr(g), cap, C.byref(nb)))
        return (np.arange(nb.value) + 0.5) * dr, g[: nb.value]

    def state(self, s=0):
        N = self.N[s]
        out = {k: np.zeros(N) for k in ("x", "y", "vx", "vy", "rad", "m")}
        cell = np.zeros(N, np.int32)
        coll = np.zeros(N, np.uint32)
        self._ck(self._L.edmd_get_state(self.h, s, *[_ptr(out[k]) for k in ("x", "y", "vx", "vy", "rad", "m")],
                                        _ptr(cell), _ptr(coll)))
        out["cell"] = cell
        out["coll"] = coll
        return out

    def load_state(self, x, y, vx, vy, rad, m):
        """Restart every system from concatenated host arrays (-l semantics)."""
        self._ck(self._L.edmd_load_state(self.h, *[_ptr(np.ascontiguousarray(a, np.float64))
                                                   for a in (x, y, vx, vy, rad, m)]))

    def states(self, out=None):
        """x, y, vx, vy, rad, m of every system, concatenated (optionally into `out`)."""
        T = sum(self.N)
        if out is None:
            out = {k: np.zeros(T) for k in ("x", "y", "vx", "vy", "rad", "m")}
        self._ck(self._L.edmd_get_states(self.h, *[_ptr(out[k]) for k in ("x", "y", "vx", "vy", "rad", "m")]))
        return out

    def all_counters(self):
        arr = (Counters * self.n)()
        self._ck(self._L.edmd_get_all_counters(self.h, C.cast(arr, C.c_void_p)))
        return {k: np.array([getattr(c, k) for c in arr]) for k, _ in Counters._fields_}

    # ---- differentiation
    def checkpoint_save(self, slot):
        self._ck(self._L.edmd_checkpoint_save(self.h, slot))

    def checkpoint_restore(self, slot):
        self._ck(self._L.edmd_checkpoint_restore(self.h, slot))

    def log(self, s=0, cap=1 << 20):
        out = np.zeros(cap, LOG_DTYPE)
        n = C.c_int64()
        rc = self._L.edmd_get_log(self.h, s, _ptr(out), cap, C.byref(n))
        if rc not in (OK, ERR_CAPACITY):
            self._ck(rc)
        return out[: min(n.value, cap)]

    def tangent(self, K, n_coll, qr_every=0, vectors=None, seed=1, s=0):
        """Propagate K tangent vectors ([K][N][4] array or random); returns (vectors, exponents)."""
        N = self.N[s]
        vec = None if vectors is None else np.ascontiguousarray(vectors, np.float64).reshape(K, N, 4).copy()
        lyap = np.zeros(K)
        self._ck(self._L.edmd_tangent_run(self.h, s, K, int(n_coll), int(qr_every), int(seed),
                                          _ptr(vec), _ptr(lyap)))
        return vec, lyap

    def msd_gradient(self, n_coll, ckpt_every=500, t_obs=-1.0, s=0):
        """Final MSD and its gradient w.r.t. the current velocities and positions."""
        N = self.N[s]
        g = {k: np.zeros(N) for k in ("vx", "vy", "x", "y")}
        msd = C.c_double()
        self._ck(self._L.edmd_msd_gradient(self.h, s, int(n_coll), int(ckpt_every), float(t_obs), C.byref(msd),
                                           _ptr(g["vx"]), _ptr(g["vy"]), _ptr(g["x"]), _ptr(g["y"])))
        return msd.value, g

    def tangent_batch(self, K, n_coll, qr_every, seed=1):
        """Lyapunov exponents of every system ([nsys][K]), system s seeded with seed + s."""
        lyap = np.zeros(self.n * K)
        self._ck(self._L.edmd_tangent_run_batch(self.h, K, int(n_coll), int(qr_every), int(seed), _ptr(lyap)))
        return lyap.reshape(self.n, K)

    def msd_gradient_batch(self, n_coll, ckpt_every=500):
        """Final MSD of every system and its gradients (concatenated over systems)."""
        T = sum(self.N)
        g = {k: np.zeros(T) for k in ("vx", "vy", "x", "y")}
        msd = np.zeros(self.n)
        self._ck(self._L.edmd_msd_gradient_batch(self.h, int(n_coll), int(ckpt_every), _ptr(msd), _ptr(g["vx"]),
                                                 _ptr(g["vy"]), _ptr(g["x"]), _ptr(g["y"])))
        return msd, g

    def counters(self, s=0):
        c = Counters()
        self._ck(self._L.edmd_get_counters(self.h, s, C.byref(c)))
        return {k: getattr(c, k) for k, _ in Counters._fields_}

    def virial(self, s=0, reset=False):
        v = np.zeros(4)
        self._ck(self._L.edmd_get_virial(self.h, s, v, int(reset)))
        return v

    def thermo(self, s=0, cap=1024, take=False):
        """Thermo rows of system s; take=True empties its row buffer too
        (edmd_take_thermo)."""
        rows = np.zeros((cap, 9))
        n = C.c_int32()
        f = self._L.edmd_take_thermo if take else self._L.edmd_get_thermo
        rc = f(self.h, s, _ptr(rows), cap, C.byref(n))
        if rc not in (OK, ERR_CAPACITY):
            self._ck(rc)
        return rows[: min(n.value, cap)]

    def trace(self, s=0):
        cap = max(self.trace_cap, 1)
        out = np.zeros(cap, COLLISION_DTYPE)
        n = C.c_int64()
        rc = self._L.edmd_get_trace(self.h, s, _ptr(out), cap, C.byref(n))
        if rc not in (OK, ERR_CAPACITY):
            self._ck(rc)
        return out[: min(n.value, cap)]

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._L.edmd_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """float64 array in page-locked host memory (edmd_host_alloc)."""

    def __init__(self, n):
        self._p = C.c_void_p()
        rc = load().edmd_host_alloc(C.byref(self._p), max(int(n), 1) * 8)
        if rc != OK:
            raise EngineError(rc, "edmd_host_alloc failed")
        buf = (C.c_double * max(int(n), 1)).from_address(self._p.value)
        self.a = np.ctypeslib.as_array(buf)[: int(n)]

    def free(self):
        if self._p.value:
            load().edmd_host_free(self._p)
            self._p = C.c_void_p()


def device_info():
    L = load()
    name = C.create_string_buffer(256)
    sms = C.c_int32()
    rc = L.edmd_device_info(name, 256, C.byref(sms))
    if rc != OK:
        return None
    return name.value.decode(), sms.value
