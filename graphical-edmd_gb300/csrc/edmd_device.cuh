// edmd_device.cuh -- device data layout and exact FP64 event arithmetic of the
// hard-disk engine.  Every formula follows the reference routine cited beside
// it operation for operation; the translation unit is compiled with
// --fmad=false so no multiply-add is contracted, which makes the results
// bit-identical to the reference built with IEEE flags.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace edmd {

constexpr double NEVER = 100000000000000000000000000.0;  // src/EDMD.h:8
constexpr int32_t NIL = -1;
constexpr uint32_t BINF = 0xFFFFFFFFu;                   // "not in the emulated tree"
constexpr uint64_t TIE_MAX = (1ull << 62) - 1;

// event states
constexpr uint32_t ST_NONE = 0, ST_QUEUED = 1, ST_OVF = 2;
// event kinds by slot: [0,N) crossing, [N,2N) collision, 2N screenshot,
// 2N+1 thermo, 2N+2 growth stop
constexpr int SP_SCREEN = 0, SP_THERMO = 1, SP_GROW = 2, NSPECIAL = 3;

// kinematic record of one disk: one 64-byte line half, so a candidate read
// during a prediction costs two 32-byte sectors and brings the list link and
// the collision counter along with the trajectory.
struct __align__(64) Disk {
  double x, y, vx, vy, tl, rad, m;
  int32_t nxt;     // next disk in the same cell (src/EDMD.h:48 nxt)
  uint32_t coll;   // collision counter (src/EDMD.h:52 coll)
};

// one event slot (src/EDMD.h:66-74 node) with its emulated queue key
struct __align__(32) Ev {
  double t;
  uint64_t tie;    // insertion-order class and counter, see schedule()
  uint32_t b;      // absolute calendar bucket the event enters the tree in
  int32_t j;       // crossing direction (1..4) or collision partner
  uint32_t ca;     // collActual: partner's counter at prediction time
  uint32_t st;     // ST_*
};

// tournament-tree node: the minimum key of its subtree and the leaf holding it;
// the time is held as its order-preserving integer image (time_key) so that
// tree comparisons run on the integer pipe
struct Node {
  uint64_t tk;
  uint64_t tie;
  uint32_t b;
  int32_t idx;
};

// order-preserving integer image of a double (non-NaN; -0 orders as +0)
__device__ __forceinline__ uint64_t time_key(double t) {
  uint64_t u = (uint64_t)__double_as_longlong(t);
  if (u == 0x8000000000000000ull) u = 0;
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// inverse of time_key (a zero comes back as +0)
__device__ __forceinline__ double key_time(uint64_t k) {
  uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

struct Box {
  double Lx, Ly, hLx, hLy;     // box and halves (boxConstantHelper src/EDMD.c:679)
  double cxs, cys, cxf, cyf;   // cell sizes and reciprocals
  double dtP, dtPN;            // calendar bucket width 5/N and width*N
  int32_t Nxc, Nyc, N;
  int32_t additive;            // contact distance r1 + r2 instead of 2 sqrt(r1 r2)
};

constexpr int MAXLEV = 8;

// scalar state of one system, kept in global memory between calls
struct SysState {
  double t, P;                 // current time, paulTime of the current bucket
  double collT[4];             // collTermX, Y, XY, YX
  double lastThermo;           // lastScreen of saveThermo (src/EDMD.c:5261)
  uint64_t C;                  // insertion counter
  uint64_t k, next_wrap;       // current absolute bucket, next overflow wrap
  uint64_t ncol, ncol_total, ncross, nstale, npair, npred, nevents, ntrace;
  int32_t ovf, grow, nrows, stop_reason;
  int32_t status, err_a, err_b, pad;
  uint64_t nlog;               // collision-geometry records written (EDMD_F_LOG)
  uint64_t nscreen;            // candidate pairs rejected by the FP32 screen (round engine)
};

struct SysDev {
  Box B;
  double res, Einit, dtime, dtimeTh, tmax;
  int32_t L, nlev;             // tree leaves (N + NSPECIAL) and levels
  int32_t lev_off[MAXLEV], lev_cnt[MAXLEV];
  Disk* d;
  double* vr;                  // growth rate per disk (src/EDMD.h:44 vr)
  int32_t *cx, *cy, *prv, *crossX, *crossY;
  int32_t* head;               // cell heads (cellList, src/EDMD.c:486)
  Ev* ev;                      // 2N + NSPECIAL slots
  int32_t *on, *op;            // overflow-bucket links (eventPaul[N])
  Node* tree;
  SysState* st;
  void* trace;                 // edmd_collision records
  int64_t trace_cap;
  void* log;                   // edmd_log_entry records (differentiation)
  int64_t log_cap;
  double* rows;                // thermo rows, 9 doubles each
  int32_t rows_cap, pad;
  // calendar of the thread-per-system engine (edmd_lane.cu)
  uint16_t* cal;               // N buckets x CAL_SUB lines of CAL_LINE u16, see edmd_lane.cu
  uint16_t* mask;              // per bucket: bit k set when sub-bucket k is non-empty
  double invw;                 // CAL_SUB / dtP
  double rdtP;                 // 1 / dtP
};

constexpr int CAL_SUB = 16;    // sub-buckets per calendar bucket (ordered by time)
constexpr int CAL_LINE = 32;   // u16 per sub-bucket line: count, 29 ids, spill-list head

struct RunArgs {
  int64_t max_coll;
  double t_stop;
  uint32_t flags;
  int64_t max_events;
  int32_t nsys;
  int32_t* work;               // persistent work counter (warp engine)
  const int32_t* order;        // warp engine: systems in the order they are taken (null: 0, 1, ...)
  uint32_t* cost;              // warp engine: each system's run time in this call (units of 1.024 us)
};

// ---------------------------------------------------------------- arithmetic

__device__ __forceinline__ void pbc(const Box& B, double& dx, double& dy) {  // PBC src/EDMD.c:5896
  if (dx >= B.hLx) dx -= B.Lx;
  else if (dx < -B.hLx) dx += B.Lx;
  if (dy >= B.hLy) dy -= B.Ly;
  else if (dy < -B.hLy) dy += B.Ly;
}
__device__ __forceinline__ double pbc_in_x(const Box& B, double d) {  // PBCinsideCellX 5922
  if (d >= B.hLx) return d - B.Lx;
  else if (d < -B.hLx) return d + B.Lx;
  return d;
}
__device__ __forceinline__ double pbc_in_y(const Box& B, double d) {  // PBCinsideCellY 5930
  if (d >= B.hLy) return d - B.Ly;
  else if (d < -B.hLy) return d + B.Ly;
  return d;
}
__device__ __forceinline__ int pbc_cx(const Box& B, int a) { return a < 0 ? a + B.Nxc : (a >= B.Nxc ? a - B.Nxc : a); }
__device__ __forceinline__ int pbc_cy(const Box& B, int a) { return a < 0 ? a + B.Nyc : (a >= B.Nyc ? a - B.Nyc : a); }


// 4 x exactly, on the integer pipe: x's exponent field + 2.  Equal to the
// FP64 product 4 * x for x = 0 and for normal |x| < 2^1021; disk radii are
// checked to be one of those when a system is created or loaded.
__device__ __forceinline__ double times4(double x) {
  const long long b = __double_as_longlong(x);
  return __longlong_as_double((b & 0x7ff0000000000000ll) ? b + (2ll << 52) : b);
}

// radii the engines accept: zero or normal, positive and below 2^1020 (so
// that times4 is exact)
__host__ __device__ __forceinline__ bool radius_ok(double r) {
  return r == 0.0 || (r >= 2.2250738585072014e-308 && r < 0x1p1020);
}

// Contact distance and its square, DIST / DIST2 (src/EDMD.c:35-43): the
// reference's default (NONADDITIVE 0) is 2 sqrt(r1 r2); additive contact
// (NONADDITIVE 1) is r1 + r2.  Same roundings as the macros (4 r1 r2 is
// (4 r1) r2 with 4 r1 exact).  The switch is per system, uniform over the
// lanes that work on one system.
// ADD = false compiles the reference's default rule only (a kernel
// specialised for contexts without additive systems).
template <bool ADD = true>
__device__ __forceinline__ double contact2(const Box& B, double r1, double r2) {
  if (ADD && B.additive) {
    const double s = r1 + r2;
    return s * s;
  }
  return times4(r1) * r2;
}
__device__ __forceinline__ double contact(const Box& B, double r1, double r2) {
  if (B.additive) return r1 + r2;
  return sqrt(times4(r1) * r2);
}

// collisionTimeNormal src/EDMD.c:2661-2723; p1 is current at t.
// *overlap is set when the pair overlaps by more than 0.01 (2708-2717).
__device__ __forceinline__ double coll_time_normal(const Box& B, const Disk& p1, const Disk& p2,
                                                   double t, bool* overlap) {
  double lat2 = t - p2.tl;
  double dvx = p2.vx - p1.vx;
  double dvy = p2.vy - p1.vy;
  double dx = (p2.x + lat2 * p2.vx) - p1.x;
  double dy = (p2.y + lat2 * p2.vy) - p1.y;
  pbc(B, dx, dy);
  double b = dx * dvx + dy * dvy;
  if (b > 0) return NEVER;
  double v2 = dvx * dvx + dvy * dvy;
  double d2 = dx * dx + dy * dy - contact2(B, p1.rad, p2.rad);
  double det = b * b - v2 * d2;
  if (d2 < -0.01) { *overlap = true; return NEVER; }
  if (det < 0) return NEVER;
  return (-b - sqrt(det)) / v2;
}

// collisionTimeGrow src/EDMD.c:2598-2659 (radii grow at vr)
__device__ __forceinline__ double coll_time_grow(const Box& B, const Disk& p1, double vr1,
                                                 const Disk& p2, double vr2, double t,
                                                 bool* overlap) {
  double lat2 = t - p2.tl;
  double dvx = p2.vx - p1.vx;
  double dvy = p2.vy - p1.vy;
  double dvr = vr1 + vr2;
  double dx = (p2.x + lat2 * p2.vx) - p1.x;
  double dy = (p2.y + lat2 * p2.vy) - p1.y;
  double dr = contact(B, p1.rad, p2.rad + lat2 * vr2);
  pbc(B, dx, dy);
  double b = dx * dvx + dy * dvy - dvr * dr;
  double v2 = dvx * dvx + dvy * dvy;
  double d2 = dx * dx + dy * dy;
  double det = b * b - (v2 - dvr * dvr) * (d2 - dr * dr);
  if (det < 0) return NEVER;
  double plus = (-b + sqrt(det)) / (v2 - dvr * dvr);
  double minus = (-b - sqrt(det)) / (v2 - dvr * dvr);
  if (((minus > 0) && (plus > 0) && (minus < plus)) || ((minus > 0) && (plus < 0))) return minus;
  else if (((minus > 0) && (plus > 0.000000001) && (plus < minus)) ||
           ((minus < 0) && (plus > 0.000000001)))
    return plus;
  if (d2 - dr * dr < -0.01) *overlap = true;
  return NEVER;
}

// crossingEventNormal src/EDMD.c:2405-2482 (the Grow variant 2343 is the same
// arithmetic); returns the absolute time and direction code 1..4.
__device__ __forceinline__ double crossing_time(const Box& B, const Disk& p, int cx, int cy,
                                                double t, int* dir) {
  double tx, ty;
  int xx, yy;
  if (p.vx < 0) { tx = pbc_in_x(B, cx * B.cxs - p.x) / p.vx; xx = 1; }
  else { tx = pbc_in_x(B, (1 + cx) * B.cxs - p.x) / p.vx; xx = 2; }
  if (p.vy < 0) { ty = pbc_in_y(B, cy * B.cys - p.y) / p.vy; yy = 3; }
  else { ty = pbc_in_y(B, (1 + cy) * B.cys - p.y) / p.vy; yy = 4; }
  if (tx < ty) { *dir = xx; return t + tx; }
  *dir = yy;
  return t + ty;
}

// Comparisons against a positive constant on the integer pipe.  For finite a
// and c > 0 these are exactly the IEEE comparisons (including -0 and +0):
//   ge_pos(a, c) == (a >= c),  lt_neg(a, c) == (a < -c),  is_neg(a) == (a < 0),
//   is_pos(a) == (a > 0).  FP64 compares issue on GB300's narrow FP64 pipe.
__device__ __forceinline__ bool ge_pos(double a, double c) {
  return __double_as_longlong(a) >= __double_as_longlong(c);
}
__device__ __forceinline__ bool lt_neg(double a, double c) {
  long long ia = __double_as_longlong(a);
  return ia < 0 && (ia & 0x7fffffffffffffffll) > __double_as_longlong(c);
}
__device__ __forceinline__ bool is_neg(double a) {
  long long ia = __double_as_longlong(a);
  return ia < 0 && (ia & 0x7fffffffffffffffll) != 0;
}
__device__ __forceinline__ bool is_pos(double a) { return __double_as_longlong(a) > 0; }

// -x when neg, else x: an exact sign flip on the integer pipe, so that
// a + flip(x, true) rounds exactly as a - x
__device__ __forceinline__ double flip(double x, bool neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ (neg ? (long long)0x8000000000000000ull : 0ll));
}

// general a < b and a <= b on the integer pipe: false when either is a NaN,
// and -0 equals +0, exactly as the FP64 comparisons
__device__ __forceinline__ bool nan_bits(double a) {
  return ((unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool lt_i(double a, double b) {
  return !nan_bits(a) && !nan_bits(b) && time_key(a) < time_key(b);
}
__device__ __forceinline__ bool le_i(double a, double b) {
  return !nan_bits(a) && !nan_bits(b) && time_key(a) <= time_key(b);
}

// pbc / pbc_in / free flight with integer-pipe comparisons (same results)
__device__ __forceinline__ void pbc_i(const Box& B, double& dx, double& dy) {
  if (ge_pos(dx, B.hLx)) dx -= B.Lx;
  else if (lt_neg(dx, B.hLx)) dx += B.Lx;
  if (ge_pos(dy, B.hLy)) dy -= B.Ly;
  else if (lt_neg(dy, B.hLy)) dy += B.Ly;
}
// freeFlyNormal src/EDMD.c:4954 / freeFlyGrow 4992 (rad advanced separately),
// the wrap tests on the integer pipe
__device__ __forceinline__ void free_fly_i(const Box& B, Disk& p, double t) {
  double dt = t - p.tl;
  p.tl = t;
  p.x += dt * p.vx;
  p.y += dt * p.vy;
  if (is_neg(p.x)) p.x += B.Lx;
  else if (ge_pos(p.x, B.Lx)) p.x -= B.Lx;
  if (is_neg(p.y)) p.y += B.Ly;
  else if (ge_pos(p.y, B.Ly)) p.y -= B.Ly;
}
// collisionTimeNormal (src/EDMD.c:2661-2723), same operations as
// coll_time_normal with the tests on the integer pipe
template <bool ADD = true>
__device__ __forceinline__ double coll_time_normal_i(const Box& B, const Disk& p1, const Disk& p2,
                                                     double t, bool* overlap) {
  double lat2 = t - p2.tl;
  double dvx = p2.vx - p1.vx;
  double dvy = p2.vy - p1.vy;
  double dx = (p2.x + lat2 * p2.vx) - p1.x;
  double dy = (p2.y + lat2 * p2.vy) - p1.y;
  pbc_i(B, dx, dy);
  double b = dx * dvx + dy * dvy;
  if (is_pos(b)) return NEVER;
  double v2 = dvx * dvx + dvy * dvy;
  double d2 = dx * dx + dy * dy - contact2<ADD>(B, p1.rad, p2.rad);
  double det = b * b - v2 * d2;
  if (lt_neg(d2, 0.01)) { *overlap = true; return NEVER; }
  if (is_neg(det)) return NEVER;
  return (-b - sqrt(det)) / v2;
}

__device__ __forceinline__ bool key_less(uint32_t b1, uint64_t t1, uint64_t k1, int32_t i1,
                                         uint32_t b2, uint64_t t2, uint64_t k2, int32_t i2) {
  if (b1 != b2) return b1 < b2;
  if (t1 != t2) return t1 < t2;
  if (k1 != k2) return k1 < k2;
  return i1 < i2;
}

// crossingEventNormal (src/EDMD.c:2405-2482) with the sign and periodic tests
// on the integer pipe; same operations and results as crossing_time
__device__ __forceinline__ double crossing_time_i(const Box& B, const Disk& p, int cx, int cy,
                                                  double t, int* dir) {
  double tx, ty, a;
  int xx, yy;
  if (is_neg(p.vx)) { a = cx * B.cxs - p.x; xx = 1; }
  else { a = (1 + cx) * B.cxs - p.x; xx = 2; }
  if (ge_pos(a, B.hLx)) a = a - B.Lx; else if (lt_neg(a, B.hLx)) a = a + B.Lx;
  tx = a / p.vx;
  if (is_neg(p.vy)) { a = cy * B.cys - p.y; yy = 3; }
  else { a = (1 + cy) * B.cys - p.y; yy = 4; }
  if (ge_pos(a, B.hLy)) a = a - B.Ly; else if (lt_neg(a, B.hLy)) a = a + B.Ly;
  ty = a / p.vy;
  if (lt_i(tx, ty)) { *dir = xx; return t + tx; }
  *dir = yy;
  return t + ty;
}

// One axis of crossingEventNormal (src/EDMD.c:2405-2482): the time to the
// wall of cell (cx, cy) the disk moves towards along x (ydim false) or y, and
// the direction code.  Branch-free over the axis, with the same operations
// as crossing_time_i, so lanes working on different axes share instructions.
__device__ __forceinline__ double axis_time(const Box& B, const Disk& p, int cx, int cy, bool ydim, int* dir) {
  const double pos = ydim ? p.y : p.x, v = ydim ? p.vy : p.vx;
  const double cs = ydim ? B.cys : B.cxs, hL = ydim ? B.hLy : B.hLx, L = ydim ? B.Ly : B.Lx;
  const int c = ydim ? cy : cx;
  const bool neg = is_neg(v);
  double a = (neg ? c : 1 + c) * cs - pos;
  *dir = (ydim ? 3 : 1) + (neg ? 0 : 1);
  if (ge_pos(a, hL)) a = a - L;
  else if (lt_neg(a, hL)) a = a + L;
  return a / v;
}

// crossing_time_i with the two divisions on two lanes of a full warp: the
// lane with (lane & xmask) == 0 takes the x axis of its disk, its partner
// lane ^ xmask the y axis; both lanes return the disk's crossing
__device__ __forceinline__ double crossing_time_lanes(const Box& B, const Disk& p, int cx, int cy, double t,
                                                      int lane, int xmask, int* dir) {
  const bool ydim = (lane & xmask) != 0;
  int d;
  const double ta = axis_time(B, p, cx, cy, ydim, &d);
  const double tb = __shfl_xor_sync(0xffffffffu, ta, xmask);
  const int db = __shfl_xor_sync(0xffffffffu, d, xmask);
  const double tx = ydim ? tb : ta, ty = ydim ? ta : tb;
  const bool ux = lt_i(tx, ty);
  *dir = ux ? (ydim ? db : d) : (ydim ? d : db);
  return t + (ux ? tx : ty);
}

// (int)(dt / dtP) of addEventToQueue without the FP64 division when provably
// equal: |dt*rdtP - fl(dt/dtP)| <= 3*q*2^-53 < 1e-9 for q < 2^22, so the floor
// is unchanged unless q is within 1e-9 of an integer (then divide exactly).
// floor(q) and the exact fraction q - floor(q) are read from the bits of q
// (integer pipe): with q = mant * 2^-shift, floor = mant >> shift and the
// fraction is frac * 2^-shift, frac = the low shift bits; fraction > 1e-9
// and fraction < 1 - 1e-9 become integer compares of frac with the
// constants' mantissas scaled by the same power of two.
__device__ __forceinline__ int bucket_offset(double dt, double dtP, double rdtP) {
  const double q = dt * rdtP;
  const unsigned long long u = (unsigned long long)__double_as_longlong(q);
  const unsigned long long c1 = (unsigned long long)__double_as_longlong(1e-9);
  const unsigned long long c2 = (unsigned long long)__double_as_longlong(1.0 - 1e-9);
  const int e = (int)((u >> 52) & 0x7ff) - 1023;
  if (e < 0) {                        // q < 1: floor 0, fraction q (q >= 0)
    if (u > c1 && u < c2) return 0;
  } else if (e <= 30) {
    const int shift = 52 - e;
    const unsigned long long M = 0xfffffffffffffull, H = 1ull << 52;
    const unsigned long long mant = (u & M) | H;
    const unsigned long long frac = mant & ((1ull << shift) - 1);
    // 1e-9 = M1 * 2^-82 and 1 - 1e-9 = M2 * 2^-53 (exponents -30 and -1)
    const unsigned long long M1 = (c1 & M) | H, M2 = (c2 & M) | H;
    const int k1 = 30 + e, k2 = 1 + e;
    if (frac > (M1 >> k1) && frac < ((M2 + (1ull << k2) - 1) >> k2)) return (int)(mant >> shift);
  }
  return (int)(dt / dtP);
}

}  // namespace edmd
