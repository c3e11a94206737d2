// edmd_lane.cu -- thread-per-system engine for large batches of independent systems.
//
// GB300 executes FP64 at one warp instruction per ~20 cycles per SM whatever
// the number of active lanes, so scalar FP64 work repeated by all lanes of a
// warp is wasted.  Here every lane owns one system and runs the reference's
// serial event loop (src/EDMD.c:523-618) on it: one FP64 warp instruction
// advances up to 32 systems.
//
// The queue is the reference's own calendar (src/EDMD.c:2144-2327: N buckets
// of width 5/N plus an overflow bucket) with the BST of the current bucket
// replaced by CAL_SUB time-ordered sub-buckets per bucket.  A sub-bucket is a
// short array of event ids; the pop takes the lexicographic minimum of
// (t, tie) over the first non-empty sub-bucket of the current bucket, where
// `tie` reproduces the BST insertion order exactly (see edmd_engine.cu).  The
// sub-bucket of an event is a monotone function of its time inside its
// bucket, so the order is exactly the reference's.  Buckets advance, and the
// overflow bucket is redistributed at each wrap, exactly as addNextPaulEvent
// (2287-2307) does.
#include "edmd_device.cuh"
#include "../../include/edmd_gpu.h"

namespace edmd {

namespace {

// A sub-bucket line is 64 bytes: u16 count, 29 u16 event ids, and the i32
// head of a spill list that takes the events beyond 29 (many events can share
// one time, e.g. disks of a lattice start sitting on cell edges).  The spill
// list reuses the overflow links on/op: an event is never in both.
constexpr int CAP = 29;
constexpr uint32_t SPILLED = 31;

__device__ __forceinline__ uint16_t* line_of(const SysDev& S, uint32_t rb, int sub) {
  return S.cal + ((size_t)rb * CAL_SUB + sub) * CAL_LINE;
}
__device__ __forceinline__ int32_t* spill_head(uint16_t* L) { return (int32_t*)(L + 30); }

// sub-bucket of time T inside absolute bucket b: monotone in T
__device__ __forceinline__ int sub_of(const SysDev& S, double T, uint32_t b) {
  long long g = (long long)(T * S.invw) - (long long)CAL_SUB * (long long)b;
  return g < 0 ? 0 : (g >= CAL_SUB ? CAL_SUB - 1 : (int)g);
}

// per-thread view of one system
struct Lane {
  SysState R;
  uint32_t actual;     // current bucket index in [0, N) (actualPaulList)
  int status;
};

__device__ __forceinline__ void cal_insert(const SysDev& S, int e, Ev& ev, uint32_t rb) {
  int sub = sub_of(S, ev.t, ev.b);
  uint16_t* L = line_of(S, rb, sub);
  int cnt = L[0];
  uint32_t pos;
  if (cnt < CAP) {
    L[1 + cnt] = (uint16_t)e;
    L[0] = (uint16_t)(cnt + 1);
    pos = (uint32_t)cnt;
  } else {
    int32_t* H = spill_head(L);
    int h = *H;
    S.on[e] = h; S.op[e] = NIL;
    if (h != NIL) S.op[h] = e;
    *H = e;
    pos = SPILLED;
  }
  S.mask[rb] |= (uint16_t)(1u << sub);
  ev.st = ST_QUEUED | ((uint32_t)sub << 2) | (pos << 6) | (rb << 11);
}

__device__ __forceinline__ void cal_remove(const SysDev& S, int e, uint32_t st) {
  int sub = (st >> 2) & 15;
  uint32_t pos = (st >> 6) & 31;
  uint32_t rb = st >> 11;
  uint16_t* L = line_of(S, rb, sub);
  int cnt = L[0];
  int32_t* H = spill_head(L);
  if (pos == SPILLED) {
    int p = S.op[e], n = S.on[e];
    if (p != NIL) S.on[p] = n; else *H = n;
    if (n != NIL) S.op[n] = p;
  } else {
    int last = L[cnt];
    L[1 + pos] = (uint16_t)last;
    if (last != e) S.ev[last].st = (S.ev[last].st & ~(31u << 6)) | (pos << 6);
    L[0] = (uint16_t)(cnt - 1);
    cnt--;
  }
  if (cnt == 0 && *H == NIL) S.mask[rb] &= (uint16_t)~(1u << sub);
}

// addEventToQueue (src/EDMD.c:2144) in key form; cls_direct 2 from a handler,
// 0 for the re-add of a wrap
__device__ void schedule(const SysDev& S, Lane& W, int e, double T, int32_t j, uint32_t ca,
                         uint64_t cls_direct) {
  const Box& B = S.B;
  SysState& R = W.R;
  Ev ev;
  ev.t = T; ev.j = j; ev.ca = ca;
  double dt = T - R.P;
  if (dt < B.dtP) {
    ev.b = (uint32_t)R.k; ev.tie = (cls_direct << 62) | R.C;
    cal_insert(S, e, ev, W.actual);
  } else if (dt >= B.dtPN) {
    ev.b = BINF; ev.tie = R.C; ev.st = ST_OVF;
    S.on[e] = R.ovf; S.op[e] = NIL;
    if (R.ovf != NIL) S.op[R.ovf] = e;
    R.ovf = e;
  } else {
    int d = bucket_offset(dt, B.dtP, S.rdtP);
    uint32_t rb = W.actual + (uint32_t)d;
    if (rb >= (uint32_t)B.N) rb -= (uint32_t)B.N;
    ev.b = (uint32_t)(R.k + (uint64_t)d); ev.tie = (1ull << 62) | (TIE_MAX - R.C);
    cal_insert(S, e, ev, rb);
  }
  R.C++;
  S.ev[e] = ev;
}

__device__ void unqueue(const SysDev& S, Lane& W, int e) {
  uint32_t st = S.ev[e].st;
  uint32_t s0 = st & 3u;
  if (s0 == ST_OVF) {
    int p = S.op[e], n = S.on[e];
    if (p != NIL) S.on[p] = n;
    else W.R.ovf = n;
    if (n != NIL) S.op[n] = p;
  } else if (s0 == ST_QUEUED) {
    cal_remove(S, e, st);
  }
  S.ev[e].st = ST_NONE;
}

__device__ void do_wrap(const SysDev& S, Lane& W) {
  int e = W.R.ovf;
  W.R.ovf = NIL;
  int guard = 0;                       // the overflow list holds at most 2N + 3 events
  while (e != NIL && guard++ <= 2 * S.B.N + NSPECIAL) {
    int n = S.on[e];
    Ev ev = S.ev[e];
    schedule(S, W, e, ev.t, ev.j, ev.ca, 0ull);
    e = n;
  }
  if (e != NIL) W.status = EDMD_ERR_BUDGET;   // a longer list is corrupt
}

__device__ __forceinline__ void fly(const SysDev& S, Disk& p, int i, double t, bool grow) {
  double dt = t - p.tl;
  free_fly_i(S.B, p, t);
  if (grow) p.rad += dt * S.vr[i];
}

// collisionEventNormal / Grow (src/EDMD.c:2829 / 3104): 3x3 cells, dy outer,
// dx inner, list order, first strict minimum; returns dt, partner, collActual
__device__ void predict(const SysDev& S, Lane& W, int a, double* dt_out, int* p_out,
                        uint32_t* ca_out) {
  const Box& B = S.B;
  const bool grow = W.R.grow != 0;
  double bd = grow ? 10000000 : NEVER;
  int bp = 0;
  uint32_t bc = 0;
  bool any = false;
  const Disk A = S.d[a];
  const double vra = grow ? S.vr[a] : 0.0;
  const int X = S.cx[a], Y = S.cy[a];
  uint64_t np = 0;
  bool ovl = false;
  int ovp = -1;                        // first partner found overlapping
  for (int q = 0; q < 9; q++) {
    int cell = pbc_cy(B, Y + q / 3 - 1) * B.Nxc + pbc_cx(B, X + q % 3 - 1);
    int p = S.head[cell];
    int guard = 0;                     // a list is never longer than N
    while (p != NIL && guard++ < B.N) {
      Disk P = S.d[p];
      if (p != a) {
        bool o2 = false;
        double d = grow ? coll_time_grow(B, A, vra, P, S.vr[p], W.R.t, &o2)
                        : coll_time_normal_i(B, A, P, W.R.t, &o2);
        if (o2 && !ovl) ovp = p;
        ovl |= o2;
        np++;
        if (time_key(bd) > time_key(d)) { bd = d; bp = p; bc = P.coll; any = true; }
      }
      p = P.nxt;
    }
    if (p != NIL) { W.status = EDMD_ERR_BUDGET; W.R.err_a = -2; W.R.err_b = a; }  // longer than N: corrupt
  }
  if (!any) bc = S.d[0].coll;
  if (ovl) { W.status = EDMD_ERR_OVERLAP; W.R.err_a = a; W.R.err_b = ovp; }
  W.R.npair += np;
  W.R.npred++;
  *dt_out = bd; *p_out = bp; *ca_out = bc;
}

__device__ void predict_and_schedule(const SysDev& S, Lane& W, int a) {
  double dt; int p; uint32_t ca;
  predict(S, W, a, &dt, &p, &ca);
  schedule(S, W, S.B.N + a, W.R.t + dt, p, ca, 2ull);
}

__device__ void cross_schedule(const SysDev& S, Lane& W, int i, const Disk& di) {
  int dir;
  double tc = crossing_time_i(S.B, di, S.cx[i], S.cy[i], W.R.t, &dir);
  schedule(S, W, i, tc, dir, 0, 2ull);
}

// physicalQ (src/EDMD.c:5968-6013)
__device__ void physical_q(const SysDev& S, double* E, double* px, double* py) {
  double a = 0, b = 0, e = 0;
  for (int i = 0; i < S.B.N; i++) {
    Disk p = S.d[i];
    a += p.vx * p.m;
    b += p.vy * p.m;
    double vx = p.vx;
    e += 0.5 * p.m * (vx * vx + p.vy * p.vy);
  }
  *E = e; *px = a; *py = b;
}

// takeAThermo + saveThermo (src/EDMD.c:4679, 5232-5697) with Nthermo = 1
__device__ void do_thermo(const SysDev& S, Lane& W) {
  SysState& R = W.R;
  const int N = S.B.N;
  double E, px, py;
  physical_q(S, &E, &px, &py);
  double area = S.B.Lx * S.B.Ly;
  double dT = R.t - R.lastThermo;
  R.lastThermo = R.t;
  double eX = 0, eY = 0, eXY = 0, eYX = 0;
  for (int i = 0; i < N; i++) {
    Disk p = S.d[i];
    eX += p.m * p.vx * p.vx; eY += p.m * p.vy * p.vy;
    eXY += p.m * p.vx * p.vy; eYX += p.m * p.vy * p.vx;
  }
  double row[9];
  row[0] = R.t; row[1] = (double)R.ncol; row[2] = E / N;
  row[4] = -1 * R.collT[0] / (area * dT) + eX / area;
  row[5] = -1 * R.collT[1] / (area * dT) + eY / area;
  row[6] = -1 * R.collT[2] / (area * dT) + eXY / area;
  row[7] = -1 * R.collT[3] / (area * dT) + eYX / area;
  row[3] = (-1 / (dT)) * (R.collT[0] + R.collT[1]) / (2 * area) + E / area;
  R.collT[0] = R.collT[1] = R.collT[2] = R.collT[3] = 0;
  double vxa = 0;
  for (int i = 0; i < N; i++) vxa += S.d[i].vx;
  vxa /= N;
  double v2 = 0, v4 = 0;
  for (int i = 0; i < N; i++) { double d = S.d[i].vx - vxa; double d2 = d * d; v2 += d2; v4 += d2 * d2; }
  v2 /= N; v4 /= N;
  row[8] = (v2 > 0.0) ? v4 / (3.0 * v2 * v2) - 1.0 : 0.0;
  if (R.t != 0) {
    if (R.nrows < S.rows_cap)
      for (int k = 0; k < 9; k++) S.rows[(int64_t)R.nrows * 9 + k] = row[k];
    R.nrows++;
  }
}

// stopGrow (src/EDMD.c:4740-4800)
__device__ void do_growstop(const SysDev& S, Lane& W) {
  SysState& R = W.R;
  const int N = S.B.N;
  for (int i = 0; i < N; i++) {
    Disk p = S.d[i];
    fly(S, p, i, R.t, true);
    p.coll = 0;
    S.d[i] = p;
    S.crossX[i] = 0; S.crossY[i] = 0;
  }
  R.ncol = 0; R.ncross = 0;
  R.grow = 0;
  double E, px, py;
  physical_q(S, &E, &px, &py);
  for (int i = 0; i < N; i++) {
    Disk p = S.d[i];
    p.vx -= px / (N * p.m);
    p.vy -= py / (N * p.m);
    S.d[i] = p;
  }
  physical_q(S, &E, &px, &py);
  for (int i = 0; i < N; i++) {
    Disk p = S.d[i];
    p.vx /= sqrt(E / N / S.Einit);
    p.vy /= sqrt(E / N / S.Einit);
    S.d[i] = p;
  }
  for (int i = 0; i < N; i++) {
    S.d[i].coll = S.d[i].coll + 1;
    unqueue(S, W, N + i);
    predict_and_schedule(S, W, i);
    unqueue(S, W, i);
    cross_schedule(S, W, i, S.d[i]);
  }
}

// One event of every lane's system per iteration, along a single predicated
// path: the collision, stale-collision and crossing handlers of the reference
// (src/EDMD.c:3542, 3553-3556, 2501) are merged so that the 32 systems of a
// warp issue their loads and FP64 together instead of serialising divergent
// branches.  Each system still performs its own queue operations in the
// reference's order.
__device__ void lane_run(const SysDev& S, const RunArgs& A) {
  const Box& B = S.B;
  const int N = B.N;
  Lane W;
  W.R = *S.st;
  W.status = EDMD_OK;
  if (W.R.status != EDMD_OK) return;
  W.actual = (uint32_t)(W.R.k % (uint64_t)N);
  SysState& R = W.R;
  int64_t logged = 0, nev = 0;
  int stop = 0;
  for (;;) {
    if (!le_i(R.t, S.tmax)) { stop = EDMD_STOP_TMAX; break; }
    if (logged >= A.max_coll) { stop = EDMD_STOP_COLL; break; }
    if (nev >= A.max_events) { W.status = EDMD_ERR_BUDGET; break; }
    // ---- findNextEvent: advance over empty buckets, wrapping as addNextPaulEvent
    uint32_t m = S.mask[W.actual];
    int guard = 0;
    while (m == 0) {
      R.k++;
      R.P += B.dtP;
      W.actual++;
      if (W.actual == (uint32_t)N) W.actual = 0;
      if (R.k == R.next_wrap) {
        do_wrap(S, W);
        R.next_wrap += (uint64_t)N;
      }
      m = S.mask[W.actual];
      if (++guard > (1 << 26)) { W.status = EDMD_ERR_BUDGET; break; }
    }
    if (W.status != EDMD_OK) break;
    uint16_t* Lp = line_of(S, W.actual, __ffs(m) - 1);
    int cnt = Lp[0];
    int e = -1;
    uint64_t bt = 0, bk = 0;
    for (int k = 1; k <= cnt; k++) {
      int f = Lp[k];
      uint64_t ft = time_key(S.ev[f].t);
      uint64_t fk = S.ev[f].tie;
      if (e < 0 || ft < bt || (ft == bt && fk < bk)) { e = f; bt = ft; bk = fk; }
    }
    for (int f = *spill_head(Lp); f != NIL; f = S.on[f]) {
      uint64_t ft = time_key(S.ev[f].t);
      uint64_t fk = S.ev[f].tie;
      if (e < 0 || ft < bt || (ft == bt && fk < bk)) { e = f; bt = ft; bk = fk; }
    }
    Ev E = S.ev[e];
    if (le_i(A.t_stop, E.t)) { stop = EDMD_STOP_TIME; break; }
    R.t = E.t;
    nev++;
    R.nevents++;
    cal_remove(S, e, E.st);
    S.ev[e].st = ST_NONE;
    const bool grow = R.grow != 0;
    if (e >= 2 * N) {
      // ---------------- sampling events (rare): screenshot, thermo, growth stop
      if (e == 2 * N + SP_SCREEN) {
        for (int i = 0; i < N; i++) {
          Disk p = S.d[i];
          fly(S, p, i, R.t, grow);
          S.d[i] = p;
        }
        schedule(S, W, e, R.t + S.dtime, 0, 0, 2ull);
        if (A.flags & EDMD_F_STOP_AT_SCREEN) stop = EDMD_STOP_SCREEN;
      } else if (e == 2 * N + SP_THERMO) {
        do_thermo(S, W);
        schedule(S, W, e, R.t + S.dtimeTh, 0, 0, 2ull);
      } else {
        do_growstop(S, W);
        if (A.flags & EDMD_F_STOP_AT_GROW) stop = EDMD_STOP_GROW;
      }
      if (W.status != EDMD_OK || stop) break;
      continue;
    }
    const bool isColl = e >= N;
    const bool cross = !isColl;
    const int a = isColl ? e - N : e;
    const int b = isColl ? E.j : a;
    Disk Da = S.d[a];
    Disk Db = S.d[b];
    fly(S, Da, a, R.t, grow);
    const bool valid = isColl && (E.ca == Db.coll);
    if (isColl && !valid) R.nstale++;
    if (valid) {
      // ---------------- collision (doTheCollisionNormal 3542 / Grow 3465)
      if ((A.flags & EDMD_F_TRACE) && S.trace && (int64_t)R.ntrace < S.trace_cap) {
        edmd_collision* tr = (edmd_collision*)S.trace + R.ntrace;
        tr->i = a; tr->j = b;
        tr->cell_i = S.cy[a] * B.Nxc + S.cx[a];
        tr->cell_j = S.cy[b] * B.Nxc + S.cx[b];
        tr->t = R.t;
      }
      R.ntrace++;
      if (!(A.flags & EDMD_F_COUNT_NORMAL) || !grow) logged++;
      R.ncol++;
      R.ncol_total++;
      fly(S, Db, b, R.t, grow);
      Da.coll++;
      Db.coll++;
      double dx = Db.x - Da.x, dy = Db.y - Da.y;
      double dvx = Db.vx - Da.vx, dvy = Db.vy - Da.vy;
      if (!grow) {   // elastic branch src/EDMD.c:3802-3827
        // 1/(1+1) and x/4 are exact, so the shortcuts below round identically
        double msum = Da.m + Db.m;
        double invMass = __double_as_longlong(msum) == 0x4000000000000000ll ? 0.5 : 1 / msum;
        pbc(B, dx, dy);
        double collKernel = invMass * (1 + S.res) * (dx * dvx + dy * dvy);
        double distSquared = contact2(B, Da.rad, Db.rad);
        double f = __double_as_longlong(distSquared) == 0x4010000000000000ll
            ? collKernel * 0.25 : collKernel / distSquared;
        double ct = Da.m * Db.m * f;
        R.collT[0] += ct * dx * dx;
        R.collT[1] += ct * dy * dy;
        R.collT[2] += ct * dx * dy;
        R.collT[3] += ct * dy * dx;
        Da.vx += f * Db.m * dx;
        Da.vy += f * Db.m * dy;
        Db.vx -= f * Da.m * dx;
        Db.vy -= f * Da.m * dy;
      } else {       // growth rule src/EDMD.c:3479-3520
        double delta = 0.1 * 0;
        double res = 0.75 * 0 + 1;
        double dvr = S.vr[a] + S.vr[b];
        pbc(B, dx, dy);
        double dist = sqrt(dx * dx + dy * dy);
        double dxr = dx / dist, dyr = dy / dist;
        double invMass = 1 / (Da.m + Db.m);
        double collKernel = invMass * (1 + res) * (dxr * dvx + dyr * dvy - dvr);
        Da.vx += collKernel * Db.m * dxr - 2 * Db.m * invMass * delta * dxr;
        Da.vy += collKernel * Db.m * dyr - 2 * Db.m * invMass * delta * dyr;
        Db.vx -= collKernel * Da.m * dxr - 2 * Da.m * invMass * delta * dxr;
        Db.vy -= collKernel * Da.m * dyr - 2 * Da.m * invMass * delta * dyr;
      }
    }
    if (cross) {
      // ---------------- cell crossing (doTheCrossing 2501)
      R.ncross++;
      int cx = S.cx[a], cy = S.cy[a];
      int pv = S.prv[a], nx = Da.nxt;
      if (pv == NIL) S.head[cy * B.Nxc + cx] = nx;
      else S.d[pv].nxt = nx;
      if (nx != NIL) S.prv[nx] = pv;
      switch (E.j) {
        case 1: if (cx - 1 == -1) { cx = B.Nxc - 1; S.crossX[a] -= 1; } else cx -= 1; break;
        case 2: if (cx + 1 == B.Nxc) { cx = 0; S.crossX[a] += 1; } else cx += 1; break;
        case 3: if (cy - 1 == -1) { cy = B.Nyc - 1; S.crossY[a] -= 1; } else cy -= 1; break;
        case 4: if (cy + 1 == B.Nyc) { cy = 0; S.crossY[a] += 1; } else cy += 1; break;
      }
      int c = cy * B.Nxc + cx;
      int h = S.head[c];
      S.cx[a] = cx; S.cy[a] = cy;
      S.prv[a] = NIL;
      Da.nxt = h;
      S.head[c] = a;
      if (h != NIL) S.prv[h] = a;
    }
    S.d[a] = Da;
    if (valid) S.d[b] = Db;
    // queue operations in the reference's order (3872-3879 / 2587-2589)
    if (valid) { unqueue(S, W, a); unqueue(S, W, b); }
    if (valid || cross) cross_schedule(S, W, a, Da);
    if (valid) cross_schedule(S, W, b, Db);
    if (valid) unqueue(S, W, N + b);
    if (cross) unqueue(S, W, N + a);
    double dta, dtb = 0;
    int pa, pb = 0;
    uint32_t caa, cab = 0;
    predict(S, W, a, &dta, &pa, &caa);
    if (valid) predict(S, W, b, &dtb, &pb, &cab);
    schedule(S, W, N + a, R.t + dta, pa, caa, 2ull);
    if (valid) schedule(S, W, N + b, R.t + dtb, pb, cab, 2ull);
    if (W.status != EDMD_OK) break;
  }
  R.stop_reason = stop;
  R.status = W.status;
  *S.st = R;
}

__global__ void __launch_bounds__(64) k_lane_run(const SysDev* __restrict__ sys, RunArgs A) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= A.nsys) return;
  lane_run(sys[s], A);
}

// build the calendar of every system from its scheduled events (one thread per system)
__global__ void k_lane_build(const SysDev* __restrict__ sys, int nsys) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const SysDev& S = sys[s];
  const int N = S.B.N;
  const int E = 2 * N + NSPECIAL;
  for (int k = 0; k < N; k++) S.mask[k] = 0;
  for (int k = 0; k < N * CAL_SUB; k++) {
    uint16_t* L = S.cal + (size_t)k * CAL_LINE;
    L[0] = 0;
    *spill_head(L) = NIL;
  }
  for (int e = 0; e < E; e++) {
    Ev ev = S.ev[e];
    if ((ev.st & 3u) != ST_QUEUED) continue;
    cal_insert(S, e, ev, ev.b);            // the calendar starts at bucket 0
    S.ev[e].st = ev.st;
  }
}

}  // namespace

cudaError_t lane_build(const SysDev* ds, int nsys, cudaStream_t st) {
  k_lane_build<<<(nsys + 63) / 64, 64, 0, st>>>(ds, nsys);
  return cudaGetLastError();
}

cudaError_t lane_run_launch(const SysDev* ds, const RunArgs& A, int threads_per_block,
                            cudaStream_t st) {
  int tpb = threads_per_block > 0 ? threads_per_block : 32;
  k_lane_run<<<(A.nsys + tpb - 1) / tpb, tpb, 0, st>>>(ds, A);
  return cudaGetLastError();
}

}  // namespace edmd
