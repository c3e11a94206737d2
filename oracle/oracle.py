"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, always as the checker or the timed CPU
reference, never by the product.  See edmd_oracle.h for what it restates.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

HEX, GROW = 1, 2


class Params(C.Structure):
    _fields_ = [("N", C.c_int), ("phi", C.c_double), ("xs", C.c_double), ("q", C.c_double),
                ("aspect", C.c_double), ("Einit", C.c_double), ("res", C.c_double),
                ("tmax", C.c_double), ("dtime", C.c_double), ("dtimeThermo", C.c_double),
                ("firstScreen", C.c_double), ("firstThermo", C.c_double), ("seed", C.c_uint32),
                ("start", C.c_int)]


COLL_DTYPE = np.dtype([("i", "<i4"), ("j", "<i4"), ("cell_i", "<i4"), ("cell_j", "<i4"), ("t", "<f8")])

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Params)]
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        L.orc_create_from_arrays.restype = C.c_void_p
        L.orc_create_from_arrays.argtypes = [C.c_int, C.c_double, C.c_double, dp, dp, dp, dp, dp, dp, ip,
                                             C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_default_params.argtypes = [C.POINTER(Params)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_run.restype = C.c_int64
        L.orc_run.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_int64,
                              C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
        L.orc_sync_all.argtypes = [C.c_void_p]
        L.orc_N.argtypes = [C.c_void_p]
        L.orc_time.argtypes = [C.c_void_p]
        L.orc_time.restype = C.c_double
        L.orc_vr.argtypes = [C.c_void_p]
        L.orc_vr.restype = C.c_double
        L.orc_set_stop_at_grow.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_contact.argtypes = [C.c_int]
        L.orc_set_contact.restype = C.c_int
        L.orc_growing.argtypes = [C.c_void_p]
        L.orc_box.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_counters.argtypes = [C.c_void_p] + [C.POINTER(C.c_uint64)] * 5
        L.orc_state.argtypes = [C.c_void_p] + [C.c_void_p] * 10
        L.orc_physicalq.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 3
        L.orc_virial.argtypes = [C.c_void_p, dp, C.c_int]
        L.orc_pcf.restype = C.c_int
        L.orc_pcf.argtypes = [C.c_void_p, C.c_double, C.c_double, dp, C.c_int]
        L.orc_thermo_rows.restype = C.c_int
        L.orc_thermo_rows.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.orc_mt_seed.argtypes = [C.c_uint32]
        L.orc_mt_next.restype = C.c_uint32
        _lib = L
    return _lib


class Oracle:
    """One serial reference-semantics system on the CPU."""

    def __init__(self, N=None, phi=0.7, seed=1, start=HEX, xs=0.0, q=0.4, aspect=1.0, tmax=4000.0,
                 dtime=100.0, dtime_thermo=100.0, arrays=None, Lx=None, Ly=None, first_thermo=None,
                 additive=False, res=1.0, Einit=1.0):
        L = load()
        self._L = L
        old = L.orc_set_contact(1 if additive else 0)
        try:
            self._create(L, N, phi, seed, start, xs, q, aspect, tmax, dtime, dtime_thermo, arrays, Lx, Ly,
                         first_thermo, res, Einit)
        finally:
            L.orc_set_contact(old)
        self.N = L.orc_N(self.h)

    def _create(self, L, N, phi, seed, start, xs, q, aspect, tmax, dtime, dtime_thermo, arrays, Lx, Ly,
                first_thermo, res, Einit):
        if arrays is not None:
            a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
            self.h = L.orc_create_from_arrays(len(a["x"]), Lx, Ly, a["x"], a["y"], a["vx"], a["vy"],
                                              a["rad"], a["m"], a["type"].astype(np.int32), 1.0,
                                              1.0, dtime, 1000.0, dtime_thermo)
        else:
            p = Params()
            L.orc_default_params(C.byref(p))
            p.N, p.phi, p.seed, p.start, p.xs, p.q, p.aspect = N, phi, seed, start, xs, q, aspect
            p.tmax, p.dtime, p.dtimeThermo = tmax, dtime, dtime_thermo
            p.res, p.Einit = res, Einit
            if first_thermo is not None:
                p.firstThermo = first_thermo
            self.h = L.orc_create(C.byref(p))

    def run(self, max_coll, t_stop=float("inf"), cap=None):
        cap = max_coll if cap is None else cap
        buf = np.zeros(max(int(min(cap, max_coll)), 1), COLL_DTYPE)
        nev = C.c_int64()
        n = self._L.orc_run(self.h, int(max_coll), float(t_stop), buf.ctypes.data_as(C.c_void_p),
                            len(buf), None, 0, C.byref(nev))
        return buf[: min(n, len(buf))], n

    def run_growth(self):
        """Run a growth start up to and including its growth-stop event."""
        self._L.orc_set_stop_at_grow(self.h, 1)
        try:
            return self.run(10 ** 15, cap=1)
        finally:
            self._L.orc_set_stop_at_grow(self.h, 0)

    def sync(self):
        self._L.orc_sync_all(self.h)

    @property
    def t(self):
        return self._L.orc_time(self.h)

    def box(self):
        Lx, Ly, nx, ny = C.c_double(), C.c_double(), C.c_int(), C.c_int()
        self._L.orc_box(self.h, C.byref(Lx), C.byref(Ly), C.byref(nx), C.byref(ny))
        return Lx.value, Ly.value, nx.value, ny.value

    def counters(self):
        v = [C.c_uint64() for _ in range(5)]
        self._L.orc_counters(self.h, *[C.byref(x) for x in v])
        return dict(zip(("ncol", "ncross", "nstale", "npair", "npred"), (x.value for x in v)))

    def state(self):
        N = self.N
        out = {k: np.zeros(N) for k in ("x", "y", "vx", "vy", "tl", "rad", "m")}
        typ = np.zeros(N, np.int32)
        cell = np.zeros(N, np.int32)
        coll = np.zeros(N, np.uint64)
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        self._L.orc_state(self.h, *[p(out[k]) for k in ("x", "y", "vx", "vy", "tl", "rad", "m")],
                          p(typ), p(cell), p(coll))
        out.update(type=typ, cell=cell, coll=coll)
        return out

    def physicalq(self):
        E, px, py = C.c_double(), C.c_double(), C.c_double()
        self._L.orc_physicalq(self.h, C.byref(E), C.byref(px), C.byref(py))
        return E.value, px.value, py.value

    def virial(self, reset=False):
        v = np.zeros(4)
        self._L.orc_virial(self.h, v, int(reset))
        return v

    def thermo(self, cap=4096):
        rows = np.zeros((cap, 9))
        n = self._L.orc_thermo_rows(self.h, rows.ctypes.data_as(C.c_void_p), cap)
        return rows[: min(n, cap)]

    def pcf(self, dr=0.1, max_r=None):
        Lx, Ly, _, _ = self.box()
        max_r = min(Lx, Ly) / 2 if max_r is None else max_r
        nb = int(max_r / dr)
        g = np.zeros(nb)
        n = self._L.orc_pcf(self.h, dr, max_r, g, nb)
        return (np.arange(n) + 0.5) * dr, g[:n]

    def close(self):
        if getattr(self, "h", None):
            self._L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
