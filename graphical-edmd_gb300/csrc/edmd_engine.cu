// edmd_engine.cu -- serial-exact event engine (one warp per system) and the C ABI.
//
// Each system is advanced by one warp that pops events in exactly the order of
// the reference's queue (src/EDMD.c:2144-2327: a calendar of N buckets of
// width 5/N plus an overflow bucket, feeding an unbalanced BST whose in-order
// ties go to the later insertion).  That order is emulated by the key
//     (b, t, tie)
// b   = absolute calendar bucket in which the event enters the BST,
// t   = event time,
// tie = class and counter reproducing the BST insertion order inside a bucket:
//       class 0  re-added directly into the BST by an overflow wrap (inserted
//                before the bucket's own list is loaded), ascending counter;
//       class 1  pushed onto a bucket list (LIFO: loaded last-pushed-first),
//                descending counter;
//       class 2  inserted directly because it falls in the current bucket,
//                ascending counter.
// The keys live in a 32-ary tournament tree (level 0 = one leaf per disk, the
// minimum of its crossing and collision events, plus three special events);
// each tree level is fixed by one coalesced 32-wide load and a warp butterfly.
// Collision prediction packs the candidates of the 3x3 neighbour cells of the
// (up to two) disks that changed into the lanes of the warp.
#include "edmd_device.cuh"
#include "../../include/edmd_gpu.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <algorithm>
#include <memory>
#include <thread>
#include <vector>

using namespace edmd;

namespace edmd {
cudaError_t lane_build(const SysDev* ds, int nsys, cudaStream_t st);
cudaError_t lane_run_launch(const SysDev* ds, const RunArgs& A, int threads_per_block, cudaStream_t st);
}

#define FULL 0xffffffffu

namespace {

constexpr int MAXC = 8;          // candidates buffered per cell list per lane
constexpr int WARPS_PER_BLOCK = 4;

// scratch of one lane group (one system)
struct WarpSmem {
  int32_t reg[2 * 9 * MAXC];     // walk buffers, one per (disk, cell) task
  int32_t comp[2 * 9 * MAXC];    // packed candidates
  int16_t ord[2 * 9 * MAXC];     // their scan order
  long long msum[2];             // last two mass sums of the collision rule (bits) ...
  double inv[2];                 // ... and 1 / msum, the same division's result
};

// A group of GW lanes that runs one system: the whole warp (GW = 32) or one
// half of it (GW = 16, two systems per warp).  Every collective of the event
// loop goes through the group's mask and width, so the two halves of a warp
// are independent and may diverge.
template <int GW>
struct Grp {
  int lane;                      // 0 .. GW-1
  unsigned mask;                 // the group's lanes within the warp
  __device__ __forceinline__ explicit Grp(int tid)
      : lane(tid & (GW - 1)), mask(GW == 32 ? 0xffffffffu : (((1u << GW) - 1u) << ((tid & 31) & ~(GW - 1)))) {}
  template <class T> __device__ __forceinline__ T shfl(T v, int src) const { return __shfl_sync(mask, v, src, GW); }
  template <class T> __device__ __forceinline__ T shfl_xor(T v, int o) const {
    return __shfl_xor_sync(mask, v, o, GW);
  }
  template <class T> __device__ __forceinline__ T shfl_up(T v, int o) const {
    return __shfl_up_sync(mask, v, o, GW);
  }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  __device__ __forceinline__ bool any(bool p) const { return __any_sync(mask, p); }
  // group-relative index of the first lane where p holds, or -1
  __device__ __forceinline__ int first(bool p) const {
    const unsigned m = __ballot_sync(mask, p) & mask;
    return m ? ((__ffs(m) - 1) & (GW - 1)) : -1;
  }
};

__device__ __forceinline__ Node empty_node(int idx) {
  Node n; n.tk = ~0ull; n.tie = ~0ull; n.b = BINF; n.idx = idx;
  return n;
}

__device__ __forceinline__ bool node_less(const Node& a, const Node& b) {
  return key_less(a.b, a.tk, a.tie, a.idx, b.b, b.tk, b.tie, b.idx);
}

template <int GW>
__device__ __forceinline__ void grp_min(Node& n, const Grp<GW>& G) {
#pragma unroll
  for (int o = GW / 2; o > 0; o >>= 1) {
    Node m;
    m.tk = G.shfl_xor(n.tk, o);
    m.tie = G.shfl_xor(n.tie, o);
    m.b = G.shfl_xor(n.b, o);
    m.idx = G.shfl_xor(n.idx, o);
    if (node_less(m, n)) n = m;
  }
}

// the minimum of the 32 children of node `par` of level h-1, on every lane
template <int GW>
__device__ __forceinline__ Node children_min(const SysDev& S, int h, int par, const Grp<GW>& G) {
  const int ch = (par << 5) + G.lane;
  Node c = ch < S.lev_cnt[h - 1] ? S.tree[S.lev_off[h - 1] + ch] : empty_node(0x7fffffff);
  if (GW < 32) {
#pragma unroll
    for (int k = GW; k < 32; k += GW) {
      const int c2 = ch + k;
      if (c2 < S.lev_cnt[h - 1]) {
        const Node m = S.tree[S.lev_off[h - 1] + c2];
        if (node_less(m, c)) c = m;
      }
    }
  }
  grp_min(c, G);
  return c;
}

__device__ __forceinline__ Node ev_node(const Ev& e, int idx) {
  Node n; n.tk = time_key(e.t); n.tie = e.tie; n.b = e.b; n.idx = idx;
  return n;
}

// recompute the leaf of `leaf` from its events and fix its path to the root
template <int GW>
__device__ void leaf_update(const SysDev& S, int leaf, const Grp<GW>& G) {
  const int lane = G.lane;
  const int N = S.B.N;
  Node n = empty_node(leaf);
  if (leaf < N) {
    Ev e0 = S.ev[leaf], e1 = S.ev[N + leaf];
    if (e0.st == ST_QUEUED) n = ev_node(e0, leaf);
    if (e1.st == ST_QUEUED) { Node m = ev_node(e1, leaf); if (node_less(m, n)) n = m; }
  } else {
    Ev e = S.ev[2 * N + (leaf - N)];
    if (e.st == ST_QUEUED) n = ev_node(e, leaf);
  }
  if (lane == 0) S.tree[leaf] = n;
  G.sync();
  int idx = leaf;
  for (int h = 1; h < S.nlev; h++) {
    int par = idx >> 5;
    const Node c = children_min(S, h, par, G);
    if (lane == 0) S.tree[S.lev_off[h] + par] = c;
    G.sync();
    idx = par;
  }
}

// rebuild every level of the tree (after init or the growth stop)
template <int GW>
__device__ __noinline__ void tree_rebuild(const SysDev& S, const Grp<GW>& G) {
  const int lane = G.lane;
  const int N = S.B.N;
  for (int l = lane; l < S.L; l += GW) {
    Node n = empty_node(l);
    if (l < N) {
      Ev e0 = S.ev[l], e1 = S.ev[N + l];
      if (e0.st == ST_QUEUED) n = ev_node(e0, l);
      if (e1.st == ST_QUEUED) { Node m = ev_node(e1, l); if (node_less(m, n)) n = m; }
    } else {
      Ev e = S.ev[2 * N + (l - N)];
      if (e.st == ST_QUEUED) n = ev_node(e, l);
    }
    S.tree[l] = n;
  }
  G.sync();
#pragma unroll
  for (int h = 1; h < MAXLEV; h++) {
    if (h >= S.nlev) break;
    for (int par = 0; par < S.lev_cnt[h]; par++) {
      const Node c = children_min(S, h, par, G);
      if (lane == 0) S.tree[S.lev_off[h] + par] = c;
    }
    G.sync();
  }
}

// ---------------------------------------------------------------- queue

// addEventToQueue (src/EDMD.c:2144) in key form, in two parts: where the
// event goes (FP64: its offset from paulTime; -1 current bucket, -2
// overflow, else the bucket offset), and the insertion (integer work).
__device__ __forceinline__ int sched_place(const SysDev& S, const SysState& R, double T) {
  const Box& B = S.B;
  const double dt = T - R.P;
  if (!ge_pos(dt, B.dtP)) return -1;           // dt < dtPaul
  if (ge_pos(dt, B.dtPN)) return -2;           // dt >= dtPaul * N
  return bucket_offset(dt, B.dtP, S.rdtP);
}

// `cls_direct` is 2 for a schedule from an event handler and 0 for the
// re-add done by a wrap
template <int GW>
__device__ __forceinline__ void sched_insert(const SysDev& S, SysState& R, int e, double T, int32_t j,
                                             uint32_t ca, uint64_t cls_direct, int place, const Grp<GW>& G) {
  const int lane = G.lane;
  Ev ev;
  ev.t = T; ev.j = j; ev.ca = ca;
  if (place == -1) {
    ev.b = (uint32_t)R.k; ev.tie = (cls_direct << 62) | R.C; ev.st = ST_QUEUED;
  } else if (place == -2) {
    ev.b = BINF; ev.tie = R.C; ev.st = ST_OVF;
    if (lane == 0) {
      S.on[e] = R.ovf; S.op[e] = NIL;
      if (R.ovf != NIL) S.op[R.ovf] = e;
    }
    R.ovf = e;
  } else {
    ev.b = (uint32_t)(R.k + (uint64_t)place); ev.tie = (1ull << 62) | (TIE_MAX - R.C); ev.st = ST_QUEUED;
  }
  R.C++;
  if (lane == 0) S.ev[e] = ev;
  G.sync();
}

template <int GW>
__device__ void schedule(const SysDev& S, SysState& R, int e, double T, int32_t j, uint32_t ca,
                         uint64_t cls_direct, const Grp<GW>& G) {
  sched_insert(S, R, e, T, j, ca, cls_direct, sched_place(S, R, T), G);
}

// one or two handler schedules in a row (e0 first; e1 < 0: none): the FP64
// placement of e0 on even lanes and of e1 on odd lanes in shared
// instructions, then the insertions
template <int GW>
__device__ void schedule2(const SysDev& S, SysState& R, int e0, double T0, int32_t j0, uint32_t ca0,
                          int e1, double T1, int32_t j1, uint32_t ca1, const Grp<GW>& G) {
  const int lane = G.lane;
  const int pl = sched_place(S, R, (lane & 1) && e1 >= 0 ? T1 : T0);
  const int p0 = G.shfl(pl, 0), p1 = G.shfl(pl, 1);
  sched_insert(S, R, e0, T0, j0, ca0, 2ull, p0, G);
  if (e1 >= 0) sched_insert(S, R, e1, T1, j1, ca1, 2ull, p1, G);
}

// removeEventFromQueue (src/EDMD.c:2209) in key form
template <int GW>
__device__ void unqueue(const SysDev& S, SysState& R, int e, const Grp<GW>& G) {
  const int lane = G.lane;
  uint32_t st = S.ev[e].st;
  if (st == ST_OVF) {
    int p = S.op[e], n = S.on[e];
    if (lane == 0) {
      if (p != NIL) S.on[p] = n;
      if (n != NIL) S.op[n] = p;
    }
    if (p == NIL) R.ovf = n;
  }
  if (lane == 0) S.ev[e].st = ST_NONE;
  G.sync();
}

// the overflow bucket is redistributed when the calendar wraps
// (addNextPaulEvent src/EDMD.c:2287-2300)
// (false: the list is longer than it can be, i.e. corrupt)
template <int GW>
__device__ __noinline__ bool do_wrap(const SysDev& S, SysState& R, const Grp<GW>& G) {
  const int N = S.B.N;
  int e = R.ovf;
  R.ovf = NIL;
  G.sync();
  int guard = 0;                       // the overflow list holds at most 2N + 3 events
  while (e != NIL && guard++ <= 2 * N + NSPECIAL) {
    int n = S.on[e];
    double T = S.ev[e].t;
    int32_t j = S.ev[e].j;
    uint32_t ca = S.ev[e].ca;
    schedule(S, R, e, T, j, ca, 0ull, G);
    G.sync();
    int leaf = e < 2 * N ? (e < N ? e : e - N) : N + (e - 2 * N);
    leaf_update(S, leaf, G);
    e = n;
  }
  return e == NIL;
}

// ---------------------------------------------------------------- prediction

struct Pred { double dt; int32_t partner; uint32_t ca; };
constexpr int OVL_CORRUPT = -2;  // overlap marker: a cell list longer than N (EDMD_ERR_BUDGET)

__device__ __forceinline__ void grow_fly(const SysDev& S, Disk& p, int i, double t, bool grow) {
  double dt = t - p.tl;
  free_fly_i(S.B, p, t);
  if (grow) p.rad += dt * S.vr[i];
}

template <bool ADD>
__device__ __forceinline__ double pair_time(const SysDev& S, const Disk& A, int a, const Disk& P,
                                            int p, double t, bool grow, bool* ovl) {
  if (grow) return coll_time_grow(S.B, A, S.vr[a], P, S.vr[p], t, ovl);
  return coll_time_normal_i<ADD>(S.B, A, P, t, ovl);
}

// candidate times compared as their order-preserving integer images: the
// same order as FP64 '<' (both zeros share one image; a NaN, which '<' never
// selects, maps above every number), on the integer pipe
__device__ __forceinline__ uint64_t cand_key(double d) {
  const uint64_t u = (uint64_t)__double_as_longlong(d);
  return (u & 0x7fffffffffffffffull) > 0x7ff0000000000000ull ? ~0ull : time_key(d);
}

__device__ __forceinline__ void best_merge(uint64_t& bk, int& bo, int& bp, uint32_t& bc,
                                           uint64_t k, int o, int p, uint32_t c) {
  if (k < bk || (k == bk && o < bo)) { bk = k; bo = o; bp = p; bc = c; }
}

// collisionEventNormal / Grow (src/EDMD.c:2829 / 3104) for disks a0 and a1
// (a1 may be -1): scan the 3x3 neighbour cells, dy outer and dx inner, list
// order, keep the first strict minimum.  The (disk, cell) walks are tasks
// t = 0..8 (a0's cells in scan order) and 9..17 (a1's): task t runs on lane
// t % GW, a lane with two tasks walks both lists at once.  The candidates are
// then packed over the group in task order and solved GW at a time.
template <int GW, bool ADD>
__device__ void predict2(const SysDev& S, SysState& R, int a0, int a1, Pred& r0, Pred& r1,
                         const Grp<GW>& G, WarpSmem* sm, bool* ovl, int* ovl_a, int* ovl_b) {
  const Box& B = S.B;
  const int lane = G.lane;
  const bool grow = R.grow != 0;
  const double dinit = grow ? 10000000 : NEVER;
  const int ntask = a1 >= 0 ? 18 : 9;
  // the tasks of this lane: t = lane + k GW, k < NT (a warp: one task per
  // lane; 16 lanes: two; 8 lanes: three; 4 lanes: five)
  constexpr int NT = (18 + GW - 1) / GW;
  auto task_cell = [&](int own, int q) {
    return pbc_cy(B, S.cy[own] + q / 3 - 1) * B.Nxc + pbc_cx(B, S.cx[own] + q % 3 - 1);
  };
  int pt[NT], ct[NT], ot[NT], qt[NT];
#pragma unroll
  for (int k = 0; k < NT; k++) {
    const int t = lane + k * GW;
    ot[k] = t >= 9 ? a1 : a0;
    qt[k] = t >= 9 ? t - 9 : t;
    pt[k] = t < ntask ? S.head[task_cell(ot[k], qt[k])] : NIL;
    ct[k] = 0;
  }
  bool lcorrupt = false;
  {
    int guard = 0;                   // the lists hold N disks in all
    bool more = true;
    while (more && guard++ < 2 * B.N) {
      more = false;
#pragma unroll
      for (int k = 0; k < NT; k++) {
        if (pt[k] != NIL) {
          const int t = lane + k * GW;
          if (pt[k] != ot[k]) { if (ct[k] < MAXC) sm->reg[t * MAXC + ct[k]] = pt[k]; ct[k]++; }
          pt[k] = S.d[pt[k]].nxt;
          more |= pt[k] != NIL;
        }
      }
    }
    // a list longer than N is corrupt: reported like an overlap, with the
    // marker OVL_CORRUPT in place of the first disk (EDMD_ERR_BUDGET)
#pragma unroll
    for (int k = 0; k < NT; k++)
      if (pt[k] != NIL) lcorrupt = true;
  }
  bool over = false;
#pragma unroll
  for (int k = 0; k < NT; k++) over |= ct[k] > MAXC;
  const bool spill = G.any(over);
  Disk A0 = S.d[a0];
  Disk A1 = a1 >= 0 ? S.d[a1] : A0;
  uint64_t bd0 = cand_key(dinit), bd1 = bd0;
  int bo0 = -1, bo1 = -1, bp0 = 0, bp1 = 0;
  uint32_t bc0 = 0, bc1 = 0;
  bool lovl = false;
  int la = -1, lb = -1;
  int tot;
  if (!spill) {
    // exclusive prefix of the counts in task order: tasks 0..GW-1, then GW..
    int ex[NT];
    int base = 0;
#pragma unroll
    for (int k = 0; k < NT; k++) {
      int in = ct[k];
#pragma unroll
      for (int o = 1; o < GW; o <<= 1) {
        const int u = G.shfl_up(in, o);
        if (lane >= o) in += u;
      }
      ex[k] = base + in - ct[k];
      base += G.shfl(in, GW - 1);
    }
    // a0's candidates are tasks 0..8: their count is the prefix at task 9
    const int tot0 = G.shfl(ex[9 / GW], 9 % GW);
    tot = base;
#pragma unroll
    for (int k = 0; k < NT; k++) {
      const int t = lane + k * GW;
      for (int m = 0; m < ct[k]; m++) {
        sm->comp[ex[k] + m] = sm->reg[t * MAXC + m];
        sm->ord[ex[k] + m] = (int16_t)(qt[k] * MAXC + m);
      }
    }
    G.sync();
    for (int f = lane; f < tot; f += GW) {
      int p = sm->comp[f];
      int o = sm->ord[f];
      Disk P = S.d[p];
      bool g1 = f >= tot0;
      bool ov = false;
      double d = pair_time<ADD>(S, g1 ? A1 : A0, g1 ? a1 : a0, P, p, R.t, grow, &ov);
      if (ov) { lovl = true; la = g1 ? a1 : a0; lb = p; }
      if (g1) best_merge(bd1, bo1, bp1, bc1, cand_key(d), o, p, P.coll);
      else best_merge(bd0, bo0, bp0, bc0, cand_key(d), o, p, P.coll);
    }
    G.sync();
  } else {
    // a cell list longer than MAXC: every task walks its own list again,
    // solving as it goes
    tot = 0;
#pragma unroll
    for (int w = 0; w < NT; w++) {
      const int t = lane + w * GW;
      if (t >= ntask) continue;
      const int own = ot[w], q = qt[w];
      const bool g1 = t >= 9;
      const Disk& AA = g1 ? A1 : A0;
      int p = S.head[task_cell(own, q)];
      int k = 0, guard = 0;
      while (p != NIL && guard++ < B.N) {
        Disk P = S.d[p];
        if (p != own) {
          bool ov = false;
          double d = pair_time<ADD>(S, AA, own, P, p, R.t, grow, &ov);
          if (ov) { lovl = true; la = own; lb = p; }
          if (g1) best_merge(bd1, bo1, bp1, bc1, cand_key(d), q * 4096 + k, p, P.coll);
          else best_merge(bd0, bo0, bp0, bc0, cand_key(d), q * 4096 + k, p, P.coll);
          k++;
        }
        p = P.nxt;
      }
      if (p != NIL) lcorrupt = true;
      tot += k;
    }
    for (int o = GW / 2; o > 0; o >>= 1) tot += G.shfl_xor(tot, o);
  }
  // lexicographic (dt, scan order) minimum over the group
#pragma unroll
  for (int o = GW / 2; o > 0; o >>= 1) {
    uint64_t d = G.shfl_xor(bd0, o); int oo = G.shfl_xor(bo0, o);
    int pp = G.shfl_xor(bp0, o); uint32_t cc = G.shfl_xor(bc0, o);
    best_merge(bd0, bo0, bp0, bc0, d, oo, pp, cc);
    d = G.shfl_xor(bd1, o); oo = G.shfl_xor(bo1, o);
    pp = G.shfl_xor(bp1, o); cc = G.shfl_xor(bc1, o);
    best_merge(bd1, bo1, bp1, bc1, d, oo, pp, cc);
  }
  if (bo0 < 0) bc0 = S.d[0].coll;   // no partner: partner 0 (src/EDMD.c:2830)
  if (bo1 < 0) bc1 = S.d[0].coll;
  r0.dt = key_time(bd0); r0.partner = bp0; r0.ca = bc0;
  r1.dt = key_time(bd1); r1.partner = bp1; r1.ca = bc1;
  R.npair += (uint64_t)tot;
  R.npred += (a1 >= 0) ? 2 : 1;
  const int src = G.first(lovl);
  if (src >= 0) {
    *ovl = true;
    *ovl_a = G.shfl(la, src);
    *ovl_b = G.shfl(lb, src);
  }
  if (G.any(lcorrupt)) { *ovl = true; *ovl_a = OVL_CORRUPT; *ovl_b = a0; }
}

// ---------------------------------------------------------------- handlers


// sequential sum over disks, in index order, identical in all lanes
template <int GW, class F>
__device__ __forceinline__ void seq_sums(const SysDev& S, const Grp<GW>& G, int nval, double* out, F f) {
  const int lane = G.lane;
  const int N = S.B.N;
  for (int k = 0; k < nval; k++) out[k] = 0;
  for (int base = 0; base < N; base += GW) {
    double v[4] = {0, 0, 0, 0};
    int i = base + lane;
    if (i < N) f(i, v);
    int lim = min(GW, N - base);
    for (int s = 0; s < lim; s++)
      for (int k = 0; k < nval; k++) out[k] += G.shfl(v[k], s);
  }
}

// physicalQ (src/EDMD.c:5968-6013): px, py, E
template <int GW>
__device__ __noinline__ void physical_q(const SysDev& S, const Grp<GW>& G, double* E, double* px, double* py) {
  double o[3];
  seq_sums(S, G, 3, o, [&](int i, double* v) {
    Disk p = S.d[i];
    v[0] = p.vx * p.m;
    v[1] = p.vy * p.m;
    double vx = p.vx;
    v[2] = 0.5 * p.m * (vx * vx + p.vy * p.vy);
  });
  *px = o[0]; *py = o[1]; *E = o[2];
}

// takeAThermo + saveThermo (src/EDMD.c:4679, 5232-5697) with Nthermo = 1
template <int GW>
__device__ __noinline__ void do_thermo(const SysDev& S, SysState& R, const Grp<GW>& G) {
  const int lane = G.lane;
  const int N = S.B.N;
  double E, px, py;
  physical_q(S, G, &E, &px, &py);
  double area = S.B.Lx * S.B.Ly;
  double dT = R.t - R.lastThermo;
  R.lastThermo = R.t;
  double e4[4];
  seq_sums(S, G, 4, e4, [&](int i, double* v) {
    Disk p = S.d[i];
    v[0] = p.m * p.vx * p.vx; v[1] = p.m * p.vy * p.vy;
    v[2] = p.m * p.vx * p.vy; v[3] = p.m * p.vy * p.vx;
  });
  double row[9];
  row[0] = R.t; row[1] = (double)R.ncol; row[2] = E / N;
  row[4] = -1 * R.collT[0] / (area * dT) + e4[0] / area;
  row[5] = -1 * R.collT[1] / (area * dT) + e4[1] / area;
  row[6] = -1 * R.collT[2] / (area * dT) + e4[2] / area;
  row[7] = -1 * R.collT[3] / (area * dT) + e4[3] / area;
  row[3] = (-1 / (dT)) * (R.collT[0] + R.collT[1]) / (2 * area) + E / area;
  R.collT[0] = R.collT[1] = R.collT[2] = R.collT[3] = 0;
  double vxa;
  seq_sums(S, G, 1, &vxa, [&](int i, double* v) { v[0] = S.d[i].vx; });
  vxa /= N;
  double v24[2];
  seq_sums(S, G, 2, v24, [&](int i, double* v) {
    double d = S.d[i].vx - vxa; double d2 = d * d; v[0] = d2; v[1] = d2 * d2;
  });
  v24[0] /= N; v24[1] /= N;
  row[8] = (v24[0] > 0.0) ? v24[1] / (3.0 * v24[0] * v24[0]) - 1.0 : 0.0;
  if (R.t != 0) {
    if (R.nrows < S.rows_cap && lane == 0)
      for (int k = 0; k < 9; k++) S.rows[(int64_t)R.nrows * 9 + k] = row[k];
    R.nrows++;
  }
}

// stopGrow (src/EDMD.c:4740-4800)
template <int GW, bool ADD>
__device__ __noinline__ void do_growstop(const SysDev& S, SysState& R, const Grp<GW>& G, WarpSmem* sm,
                            bool* ovl, int* oa, int* ob) {
  const int lane = G.lane;
  const int N = S.B.N;
  for (int i = lane; i < N; i += GW) {
    Disk p = S.d[i];
    grow_fly(S, p, i, R.t, true);
    p.coll = 0;
    S.d[i] = p;
    S.crossX[i] = 0; S.crossY[i] = 0;
  }
  R.ncol = 0; R.ncross = 0;
  R.grow = 0;
  G.sync();
  // normalizePhysicalQ (src/EDMD.c:5723-5764)
  double E, px, py;
  physical_q(S, G, &E, &px, &py);
  for (int i = lane; i < N; i += GW) {
    Disk p = S.d[i];
    p.vx -= px / (N * p.m);
    p.vy -= py / (N * p.m);
    S.d[i] = p;
  }
  G.sync();
  physical_q(S, G, &E, &px, &py);
  for (int i = lane; i < N; i += GW) {
    Disk p = S.d[i];
    p.vx /= sqrt(E / N / S.Einit);
    p.vy /= sqrt(E / N / S.Einit);
    S.d[i] = p;
  }
  G.sync();
  for (int i = 0; i < N; i++) {
    uint32_t c = S.d[i].coll + 1;
    if (lane == 0) S.d[i].coll = c;
    G.sync();
    unqueue(S, R, N + i, G);
    Pred r0, r1;
    predict2<GW, ADD>(S, R, i, -1, r0, r1, G, sm, ovl, oa, ob);
    schedule(S, R, N + i, R.t + r0.dt, r0.partner, r0.ca, 2ull, G);
    unqueue(S, R, i, G);
    int dir;
    Disk p = S.d[i];
    double tc = crossing_time_i(S.B, p, S.cx[i], S.cy[i], R.t, &dir);
    schedule(S, R, i, tc, dir, 0, 2ull, G);
    G.sync();
  }
  tree_rebuild(S, G);
}

// crossing_time_i with the two divisions on two lanes of the group: the lane
// with (lane & xmask) == 0 takes the x axis of its disk, its partner lane ^
// xmask the y axis; both return the disk's crossing
template <int GW>
__device__ __forceinline__ double crossing_time_grp(const Box& B, const Disk& p, int cx, int cy, double t,
                                                    const Grp<GW>& G, int xmask, int* dir) {
  const bool ydim = (G.lane & xmask) != 0;
  int d;
  const double ta = axis_time(B, p, cx, cy, ydim, &d);
  const double tb = G.shfl_xor(ta, xmask);
  const int db = G.shfl_xor(d, xmask);
  const double tx = ydim ? tb : ta, ty = ydim ? ta : tb;
  const bool ux = lt_i(tx, ty);
  *dir = ux ? (ydim ? db : d) : (ydim ? d : db);
  return t + (ux ? tx : ty);
}

// ---------------------------------------------------------------- run loop

// the four virial sums live on lanes 0..3 (lane l accumulates term l % 4)
// during the event loop; every lane gets all four back here
template <int GW>
__device__ __forceinline__ void gather_virial(SysState& R, double ctl, const Grp<GW>& G) {
#pragma unroll
  for (int k = 0; k < 4; k++) R.collT[k] = G.shfl(ctl, k);
}

// ADD = false: a context without additive-contact systems (the rule's
// switch compiled out of the pair solves and the collision rule)
template <int GW, bool ADD = true>
__device__ void run_system(const SysDev& S, const RunArgs& A, int64_t max_coll, const Grp<GW>& G,
                           WarpSmem* sm) {
  const int lane = G.lane;
  const Box& B = S.B;
  const int N = B.N;
  SysState R = *S.st;
  if (R.status != EDMD_OK) return;
  double ctl = R.collT[lane & 3];      // this lane's virial term, see gather_virial
  if (lane == 0) { sm->msum[0] = sm->msum[1] = 0; }   // no mass sum is +0
  G.sync();
  const int root = S.lev_off[S.nlev - 1];
  int64_t logged = 0, nev = 0;
  int stop = 0, status = EDMD_OK;
  bool ovl = false;
  int oa = -1, ob = -1;
  for (;;) {
    if (!le_i(R.t, S.tmax)) { stop = EDMD_STOP_TMAX; break; }
    if (logged >= max_coll) { stop = EDMD_STOP_COLL; break; }
    if (nev >= A.max_events) { status = EDMD_ERR_BUDGET; break; }
    Node r;
    int guard = 0;
    for (;;) {
      r = S.tree[root];
      if (r.b == BINF || (uint64_t)r.b >= R.next_wrap) {
        if (r.b == BINF && R.ovf == NIL) { status = EDMD_ERR_BUDGET; break; }
        while (R.k < R.next_wrap) { R.P += B.dtP; R.k++; }
        if (!do_wrap(S, R, G)) { status = EDMD_ERR_BUDGET; break; }
        R.next_wrap += (uint64_t)N;
        if (++guard > (1 << 20)) { status = EDMD_ERR_BUDGET; break; }
        continue;
      }
      while (R.k < (uint64_t)r.b) { R.P += B.dtP; R.k++; }
      break;
    }
    if (status != EDMD_OK) break;
    int leaf = r.idx, e;
    if (leaf < N) {
      Ev e0 = S.ev[leaf];
      e = (e0.st == ST_QUEUED && e0.b == r.b && time_key(e0.t) == r.tk && e0.tie == r.tie) ? leaf : N + leaf;
    } else {
      e = 2 * N + (leaf - N);
    }
    Ev E = S.ev[e];
    if (le_i(A.t_stop, E.t)) { stop = EDMD_STOP_TIME; break; }
    R.t = E.t;
    nev++;
    R.nevents++;
    if (lane == 0) S.ev[e].st = ST_NONE;
    G.sync();
    const bool grow = R.grow != 0;
    int ka = -1, kb = -1, uq = -1;     // disks whose crossing events are scheduled below, event removed
    int pa = -1, pb = -1;              // disks whose collision events are predicted below
    int se0 = -1, se1 = -1;            // events inserted below, their times, partners, counters
    double sT0 = 0, sT1 = 0;
    int32_t sj0 = 0, sj1 = 0;
    uint32_t sca0 = 0, sca1 = 0;
    int la = -1, lb = -1;              // leaves whose tree paths are updated below
    if (e >= N && e < 2 * N) {
      // ---------------- collision (doTheCollisionNormal 3542 / Grow 3465)
      const int i = e - N, j = E.j;
      Disk di = S.d[i];
      Disk dj = S.d[j];
      const bool stale = E.ca != dj.coll;
      {
        // free flights of i (even lanes) and j (odd lanes) in shared
        // instructions; j's is used only when the event is not stale
        const bool odd = lane & 1;
        Disk M = odd ? dj : di;
        grow_fly(S, M, odd ? j : i, R.t, grow);
        di.x = G.shfl(M.x, 0); di.y = G.shfl(M.y, 0);
        di.tl = G.shfl(M.tl, 0); di.rad = G.shfl(M.rad, 0);
        dj.x = G.shfl(M.x, 1); dj.y = G.shfl(M.y, 1);
        dj.tl = G.shfl(M.tl, 1); dj.rad = G.shfl(M.rad, 1);
      }
      if (stale) {
        if (lane == 0) S.d[i] = di;
        G.sync();
        R.nstale++;
        pa = i;
      } else {
        const int ci = S.cy[i] * B.Nxc + S.cx[i];
        const int cj = S.cy[j] * B.Nxc + S.cx[j];
        if ((A.flags & EDMD_F_TRACE) && S.trace && (int64_t)R.ntrace < S.trace_cap && lane == 0) {
          edmd_collision* tr = (edmd_collision*)S.trace + R.ntrace;
          tr->i = i; tr->j = j; tr->cell_i = ci; tr->cell_j = cj; tr->t = R.t;
        }
        R.ntrace++;
        if (!(A.flags & EDMD_F_COUNT_NORMAL) || !grow) logged++;
        R.ncol++;
        R.ncol_total++;
        di.coll++;
        dj.coll++;
        // dx, dy, dvx, dvy on lanes 0..3 (mod 4) in one instruction
        const int q4 = lane & 3;
        double dx, dy, dvx, dvy;
        {
          const double d4 = (q4 == 0 ? dj.x : q4 == 1 ? dj.y : q4 == 2 ? dj.vx : dj.vy) -
                            (q4 == 0 ? di.x : q4 == 1 ? di.y : q4 == 2 ? di.vx : di.vy);
          dx = G.shfl(d4, 0); dy = G.shfl(d4, 1);
          dvx = G.shfl(d4, 2); dvy = G.shfl(d4, 3);
        }
        if (!grow) {   // elastic branch src/EDMD.c:3802-3827
          // 1/(1+1) and x/4 are exact, so these shortcuts round identically
          // (== 2.0 and == 4.0 as bit compares, on the integer pipe)
          // 1 / msum repeats for the few mass pairs of a system: the last two
          // results are kept (a bit-identical value, without the division)
          double msum = di.m + dj.m;
          const long long mk = __double_as_longlong(msum);
          double invMass;
          if (mk == 0x4000000000000000ll) invMass = 0.5;
          else if (mk == sm->msum[0]) invMass = sm->inv[0];
          else if (mk == sm->msum[1]) invMass = sm->inv[1];
          else {
            invMass = 1 / msum;
            G.sync();
            if (lane == 0) {
              sm->msum[1] = sm->msum[0]; sm->inv[1] = sm->inv[0];
              sm->msum[0] = mk; sm->inv[0] = invMass;
            }
            G.sync();
          }
          pbc_i(B, dx, dy);
          // dx*dvx on even lanes, dy*dvy on odd lanes, then their sum
          const double pm = ((q4 & 1) ? dy : dx) * ((q4 & 1) ? dvy : dvx);
          double collKernel = invMass * (1 + S.res) * (G.shfl(pm, 0) + G.shfl(pm, 1));
          double distSquared = contact2<ADD>(B, di.rad, dj.rad);
          double f = __double_as_longlong(distSquared) == 0x4010000000000000ll ? collKernel * 0.25
                                                                                : collKernel / distSquared;
          double ct = di.m * dj.m * f;
          // collTermX, Y, XY, YX: term lane % 4 on each lane, in shared instructions
          {
            const int q = lane & 3;
            ctl += ct * ((q & 1) ? dy : dx) * ((q == 0 || q == 3) ? dx : dy);
          }
          if ((A.flags & EDMD_F_LOG) && S.log && (int64_t)R.nlog < S.log_cap && lane == 0) {
            edmd_log_entry* lg = (edmd_log_entry*)S.log + R.nlog;
            lg->i = i; lg->j = j; lg->t = R.t; lg->dx = dx; lg->dy = dy;
            lg->dvx = dvx; lg->dvy = dvy; lg->f = f;
          }
          if (A.flags & EDMD_F_LOG) R.nlog++;
          // lanes 0..3 (mod 4) update i.vx, j.vx, i.vy, j.vy in shared
          // instructions (v - x computed as v + (-x), the same rounding)
          {
            const bool oj = q4 & 1, yax = q4 & 2;
            const double v = yax ? (oj ? dj.vy : di.vy) : (oj ? dj.vx : di.vx);
            const double inc = f * (oj ? di.m : dj.m) * (yax ? dy : dx);
            const double nv = v + flip(inc, oj);
            di.vx = G.shfl(nv, 0); dj.vx = G.shfl(nv, 1);
            di.vy = G.shfl(nv, 2); dj.vy = G.shfl(nv, 3);
          }
        } else {       // growth rule src/EDMD.c:3479-3520
          double delta = 0.1 * 0;
          double res = 0.75 * 0 + 1;
          double dvr = S.vr[i] + S.vr[j];
          pbc(B, dx, dy);
          double dist = sqrt(dx * dx + dy * dy);
          double dxr = dx / dist, dyr = dy / dist;
          double invMass = 1 / (di.m + dj.m);
          double collKernel = invMass * (1 + res) * (dxr * dvx + dyr * dvy - dvr);
          di.vx += collKernel * dj.m * dxr - 2 * dj.m * invMass * delta * dxr;
          di.vy += collKernel * dj.m * dyr - 2 * dj.m * invMass * delta * dyr;
          dj.vx -= collKernel * di.m * dxr - 2 * di.m * invMass * delta * dxr;
          dj.vy -= collKernel * di.m * dyr - 2 * di.m * invMass * delta * dyr;
        }
        if (lane == 0) { S.d[i] = di; S.d[j] = dj; }
        G.sync();
        unqueue(S, R, i, G);
        unqueue(S, R, j, G);
        ka = i; kb = j; uq = N + j;
        pa = i;
        pb = j;
      }
    } else if (e < N) {
      // ---------------- cell crossing (doTheCrossing 2501)
      const int i = e;
      R.ncross++;
      Disk di = S.d[i];
      grow_fly(S, di, i, R.t, grow);
      int cx = S.cx[i], cy = S.cy[i];
      if (lane == 0) {
        int pv = S.prv[i], nx = di.nxt;
        if (pv == NIL) S.head[cy * B.Nxc + cx] = nx;
        else S.d[pv].nxt = nx;
        if (nx != NIL) S.prv[nx] = pv;
      }
      int dx = 0, dy = 0;
      switch (E.j) {
        case 1: if (cx - 1 == -1) { cx = B.Nxc - 1; dx = -1; } else cx -= 1; break;
        case 2: if (cx + 1 == B.Nxc) { cx = 0; dx = 1; } else cx += 1; break;
        case 3: if (cy - 1 == -1) { cy = B.Nyc - 1; dy = -1; } else cy -= 1; break;
        case 4: if (cy + 1 == B.Nyc) { cy = 0; dy = 1; } else cy += 1; break;
      }
      G.sync();
      if (lane == 0) {
        int c = cy * B.Nxc + cx;
        int h = S.head[c];
        S.cx[i] = cx; S.cy[i] = cy;
        if (dx) S.crossX[i] += dx;
        if (dy) S.crossY[i] += dy;
        S.prv[i] = NIL;
        di.nxt = h;
        S.d[i] = di;
        S.head[c] = i;
        if (h != NIL) S.prv[h] = i;
      }
      G.sync();
      ka = i; uq = N + i;
      pa = i;
    } else if (e == 2 * N + SP_SCREEN) {
      // ---------------- screenshot (takeAScreenshot 4657): free-fly everything
      for (int i = lane; i < N; i += GW) {
        Disk p = S.d[i];
        grow_fly(S, p, i, R.t, grow);
        S.d[i] = p;
      }
      G.sync();
      se0 = e; sT0 = R.t + S.dtime;
      la = N + SP_SCREEN;
      if (A.flags & EDMD_F_STOP_AT_SCREEN) { stop = EDMD_STOP_SCREEN; }
    } else if (e == 2 * N + SP_THERMO) {
      gather_virial(R, ctl, G);
      do_thermo(S, R, G);
      ctl = R.collT[lane & 3];
      se0 = e; sT0 = R.t + S.dtimeTh;
      la = N + SP_THERMO;
    } else {
      do_growstop<GW, ADD>(S, R, G, sm, &ovl, &oa, &ob);
      if (A.flags & EDMD_F_STOP_AT_GROW) stop = EDMD_STOP_GROW;
    }
    // the tail shared by the handlers: new crossing events of the one or two
    // disks that changed (crossingEvent for i, then j; even lanes take i,
    // odd lanes j), the removal of the collision event they replace, new
    // collision events (collisionEvent for i, then j), the insertion of the
    // handler's new events, and the tree paths of the changed leaves
    if (ka >= 0) {
      const int k = (lane & 1) && kb >= 0 ? kb : ka;
      const Disk dk = S.d[k];
      int dir;
      const double tc = crossing_time_grp(B, dk, S.cx[k], S.cy[k], R.t, G, 2, &dir);
      schedule2(S, R, ka, G.shfl(tc, 0), G.shfl(dir, 0), 0,
                kb, G.shfl(tc, 1), G.shfl(dir, 1), 0, G);
      unqueue(S, R, uq, G);
    }
    if (pa >= 0) {
      Pred r0, r1;
      predict2<GW, ADD>(S, R, pa, pb, r0, r1, G, sm, &ovl, &oa, &ob);
      const double tn = R.t + ((lane & 1) ? r1.dt : r0.dt);
      se0 = N + pa; sT0 = G.shfl(tn, 0); sj0 = r0.partner; sca0 = r0.ca;
      if (pb >= 0) { se1 = N + pb; sT1 = G.shfl(tn, 1); sj1 = r1.partner; sca1 = r1.ca; }
      la = pa;
      lb = pb;
    }
    if (se0 >= 0) schedule2(S, R, se0, sT0, sj0, sca0, se1, sT1, sj1, sca1, G);
    G.sync();
    for (int q = 0; q < 2; q++) {
      const int lf = q ? lb : la;
      if (lf < 0) break;
      leaf_update(S, lf, G);
    }
    if (ovl) { status = oa == OVL_CORRUPT ? EDMD_ERR_BUDGET : EDMD_ERR_OVERLAP; break; }
    if (stop) break;
  }
  gather_virial(R, ctl, G);
  R.stop_reason = stop;
  R.status = status;
  if (ovl) { R.err_a = oa; R.err_b = ob; }
  if (lane == 0) *S.st = R;
  G.sync();
}

// Persistent launch: lane groups (GW lanes, one system each) pull systems
// from a counter, in A.order, and record each system's run time
// (globaltimer) for the next call's order.
template <int GW, bool ADD = true>
__global__ void __launch_bounds__(32 * WARPS_PER_BLOCK, 4)
k_run(const SysDev* __restrict__ sys, RunArgs A) {
  __shared__ WarpSmem smem[WARPS_PER_BLOCK * (32 / GW)];
  const Grp<GW> G(threadIdx.x);
  WarpSmem* sm = &smem[threadIdx.x / GW];
  for (;;) {
    int it = 0;
    if (G.lane == 0) it = atomicAdd(A.work, 1);
    it = G.shfl(it, 0);
    if (it >= A.nsys) break;
    const int s = A.order ? A.order[it] : it;
    unsigned long long t0 = 0, t1 = 0;
    if (A.cost) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    run_system<GW, ADD>(sys[s], A, A.max_coll, G, sm);
    if (A.cost && G.lane == 0) {
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
      const unsigned long long c = (t1 - t0) >> 10;
      A.cost[s] = c > 0xffffffffull ? 0xffffffffu : (uint32_t)c;
    }
  }
}

// ---------------------------------------------------------------- shared-memory kernel

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void record_cost(const RunArgs& A, int s, unsigned long long t0) {
  const unsigned long long c = (global_ns() - t0) >> 10;
  A.cost[s] = c > 0xffffffffull ? 0xffffffffu : (uint32_t)c;
}

// where one system's engine state sits in a block's dynamic shared memory:
// disk records, event slots, tree, cell coordinates and links, cell heads and
// overflow links; the scalar state, growth rates, trace, log and thermo rows
// stay in global memory
struct SmemLayout {
  size_t d, ev, tree, cx, cy, prv, crossX, crossY, head, on, op, total;
};

__host__ __device__ inline SmemLayout smem_layout(const SysDev& S) {
  const size_t N = (size_t)S.B.N, E = 2 * N + NSPECIAL, C = (size_t)S.B.Nxc * S.B.Nyc;
  size_t nodes = 0;
  for (int h = 0; h < S.nlev; h++) nodes += (size_t)S.lev_cnt[h];
  SmemLayout L;
  size_t o = 0;
  auto take = [&](size_t bytes) { const size_t r = o; o += (bytes + 63) & ~(size_t)63; return r; };
  L.d = take(N * sizeof(Disk));
  L.ev = take(E * sizeof(Ev));
  L.tree = take(nodes * sizeof(Node));
  L.cx = take(N * 4); L.cy = take(N * 4); L.prv = take(N * 4);
  L.crossX = take(N * 4); L.crossY = take(N * 4);
  L.head = take(C * 4);
  L.on = take(E * 4); L.op = take(E * 4);
  L.total = o;
  return L;
}

// words of one array between global and shared memory, over the warp
__device__ __forceinline__ void warp_copy(void* dst, const void* src, size_t bytes, int lane) {
  uint32_t* d = (uint32_t*)dst;
  const uint32_t* s = (const uint32_t*)src;
  for (size_t k = lane; k < bytes / 4; k += 32) d[k] = s[k];
}

// One warp per block: each system of `list` is copied into the block's
// shared memory, run by the same event loop as k_run through a descriptor
// whose arrays point there (every access in it is a generic-address access),
// and copied back.  Dependent accesses then cost shared-memory latency
// instead of L2/HBM latency, at the price of one resident system per ~100 KB.
__global__ void __launch_bounds__(32) k_run_smem(const SysDev* __restrict__ sys, RunArgs A,
                                                 const int32_t* __restrict__ list, int nlist,
                                                 int32_t* __restrict__ work) {
  extern __shared__ __align__(128) unsigned char dyn[];
  __shared__ WarpSmem wsm;
  const Grp<32> G(threadIdx.x);
  const int lane = G.lane;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(work, 1);
    it = G.shfl(it, 0);
    if (it >= nlist) break;
    const int s = list[it];
    const unsigned long long t0 = A.cost ? global_ns() : 0;
    const SysDev& S = sys[s];
    const SmemLayout Y = smem_layout(S);
    const size_t N = (size_t)S.B.N, E = 2 * N + NSPECIAL, C = (size_t)S.B.Nxc * S.B.Nyc;
    size_t nodes = 0;
    for (int h = 0; h < S.nlev; h++) nodes += (size_t)S.lev_cnt[h];
    SysDev L = S;
    L.d = (Disk*)(dyn + Y.d); L.ev = (Ev*)(dyn + Y.ev); L.tree = (Node*)(dyn + Y.tree);
    L.cx = (int32_t*)(dyn + Y.cx); L.cy = (int32_t*)(dyn + Y.cy); L.prv = (int32_t*)(dyn + Y.prv);
    L.crossX = (int32_t*)(dyn + Y.crossX); L.crossY = (int32_t*)(dyn + Y.crossY);
    L.head = (int32_t*)(dyn + Y.head); L.on = (int32_t*)(dyn + Y.on); L.op = (int32_t*)(dyn + Y.op);
    warp_copy(L.d, S.d, N * sizeof(Disk), lane);
    warp_copy(L.ev, S.ev, E * sizeof(Ev), lane);
    warp_copy(L.tree, S.tree, nodes * sizeof(Node), lane);
    warp_copy(L.cx, S.cx, N * 4, lane); warp_copy(L.cy, S.cy, N * 4, lane);
    warp_copy(L.prv, S.prv, N * 4, lane);
    warp_copy(L.crossX, S.crossX, N * 4, lane); warp_copy(L.crossY, S.crossY, N * 4, lane);
    warp_copy(L.head, S.head, C * 4, lane);
    warp_copy(L.on, S.on, E * 4, lane); warp_copy(L.op, S.op, E * 4, lane);
    G.sync();
    run_system(L, A, A.max_coll, G, &wsm);
    G.sync();
    warp_copy(S.d, L.d, N * sizeof(Disk), lane);
    warp_copy(S.ev, L.ev, E * sizeof(Ev), lane);
    warp_copy(S.tree, L.tree, nodes * sizeof(Node), lane);
    warp_copy(S.cx, L.cx, N * 4, lane); warp_copy(S.cy, L.cy, N * 4, lane);
    warp_copy(S.prv, L.prv, N * 4, lane);
    warp_copy(S.crossX, L.crossX, N * 4, lane); warp_copy(S.crossY, L.crossY, N * 4, lane);
    warp_copy(S.head, L.head, C * 4, lane);
    warp_copy(S.on, L.on, E * 4, lane); warp_copy(S.op, L.op, E * 4, lane);
    G.sync();
    if (A.cost && lane == 0) record_cost(A, s, t0);
  }
}

// ---------------------------------------------------------------- init kernels

// initial predictions of eventListInit (src/EDMD.c:2007-2012): all disks are
// current at t = 0 and the calendar sits at bucket 0, so every key is known
// without serialising: the k-th scheduled event has counter k.
// grid.y = system, grid.x covers the disks of the largest system + 1.
__global__ void k_init_events(const SysDev* __restrict__ sys) {
  const SysDev& S = sys[blockIdx.y];
  const Box& B = S.B;
  const int N = B.N;
  const bool grow = S.st->grow != 0;
  const int nspec = grow ? 3 : 2;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  auto key = [&](Ev& ev, double T, uint64_t C) {
    double dt = T - 0.0;
    if (dt < B.dtP) { ev.b = 0; ev.tie = (2ull << 62) | C; ev.st = ST_QUEUED; }
    else if (dt >= B.dtPN) { ev.b = BINF; ev.tie = C; ev.st = ST_OVF; }
    else { int d = (int)(dt / B.dtP); ev.b = (uint32_t)d; ev.tie = (1ull << 62) | (TIE_MAX - C); ev.st = ST_QUEUED; }
  };
  if (i < N) {
    Disk A = S.d[i];
    int dir;
    Ev ec; ec.t = crossing_time(B, A, S.cx[i], S.cy[i], 0.0, &dir); ec.j = dir; ec.ca = 0;
    key(ec, ec.t, (uint64_t)nspec + 2ull * i);
    S.ev[i] = ec;
    double bd = grow ? 10000000 : NEVER;
    int bp = 0;
    bool ov = false;
    int ovp = -1;                     // first partner found overlapping
    int X = S.cx[i], Y = S.cy[i];
    uint64_t np = 0;
    for (int q = 0; q < 9; q++) {
      int cell = pbc_cy(B, Y + q / 3 - 1) * B.Nxc + pbc_cx(B, X + q % 3 - 1);
      for (int p = S.head[cell]; p != NIL; p = S.d[p].nxt) {
        if (p == i) continue;
        Disk P = S.d[p];
        bool o2 = false;
        double d = grow ? coll_time_grow(B, A, S.vr[i], P, S.vr[p], 0.0, &o2)
                        : coll_time_normal(B, A, P, 0.0, &o2);
        if (o2 && ovp < 0) ovp = p;
        ov |= o2;
        np++;
        if (bd > d) { bd = d; bp = p; }
      }
    }
    Ev el; el.t = 0.0 + bd; el.j = bp; el.ca = 0;
    key(el, el.t, (uint64_t)nspec + 2ull * i + 1);
    S.ev[N + i] = el;
    atomicAdd((unsigned long long*)&S.st->npair, (unsigned long long)np);
    // one thread (the first to claim the status) names the pair
    if (ov && atomicCAS(&S.st->status, EDMD_OK, EDMD_ERR_OVERLAP) == EDMD_OK) {
      S.st->err_a = i;
      S.st->err_b = ovp;
    }
  } else if (i == N) {
    // thermo, [growth stop], screenshot in eventListInit order
    Ev e; e.j = 0; e.ca = 0;
    e.t = S.st->lastThermo;   // holds first_thermo + 1e-9 on entry
    key(e, e.t, 0);
    S.ev[2 * N + SP_THERMO] = e;
    uint64_t C = 1;
    Ev g; g.j = 0; g.ca = 0; g.t = S.st->collT[0];  // holds t_growstop on entry
    if (grow) { key(g, g.t, C); C++; } else { g.st = ST_NONE; g.b = BINF; g.tie = 0; }
    S.ev[2 * N + SP_GROW] = g;
    Ev sc; sc.j = 0; sc.ca = 0; sc.t = S.st->collT[1];  // holds first_screen on entry
    key(sc, sc.t, C);
    S.ev[2 * N + SP_SCREEN] = sc;
  }
}

// link the initial overflow bucket in LIFO order and finish the scalar state;
// one block per system.  The reference pushes the initial events in the order
// thermo, [growth stop], screenshot, then crossing i and collision i for
// i = 0..N-1 (eventListInit, src/EDMD.c:1935-2019); an overflow event's `on`
// link is the previous overflow event in that order and `op` the next one, so
// both follow from a running maximum over the push positions.
__device__ __forceinline__ int init_slot(int p, int N, bool grow) {
  const int nspec = grow ? 3 : 2;
  if (p < nspec) {
    if (p == 0) return 2 * N + SP_THERMO;
    if (grow && p == 1) return 2 * N + SP_GROW;
    return 2 * N + SP_SCREEN;
  }
  const int k = p - nspec;
  return (k & 1) ? N + (k >> 1) : (k >> 1);
}

__global__ void __launch_bounds__(256) k_init_finish(const SysDev* __restrict__ sys, int nsys) {
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const SysDev& S = sys[s];
  const int N = S.B.N;
  const bool grow = S.st->grow != 0;
  const int P = (grow ? 3 : 2) + 2 * N;
  __shared__ int wmax[8];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = -1;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base = 0; base < P; base += blockDim.x) {
    const int p = base + threadIdx.x;
    const int e = p < P ? init_slot(p, N, grow) : -1;
    const bool ovf = e >= 0 && S.ev[e].st == ST_OVF;
    // exclusive running maximum of the overflow positions: the previous one
    int v = ovf ? p : -1;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(FULL, incl, o);
      if (lane >= o && u > incl) incl = u;
    }
    if (lane == 31) wmax[w] = incl;
    __syncthreads();
    int before = carry;
    for (int k = 0; k < w; k++) before = wmax[k] > before ? wmax[k] : before;
    int excl = __shfl_up_sync(FULL, incl, 1);
    if (lane == 0) excl = -1;
    const int prev = excl > before ? excl : before;
    if (ovf) {
      // every overflow event but the last gets its `op` from its successor
      const int pe = prev >= 0 ? init_slot(prev, N, grow) : NIL;
      S.on[e] = pe;
      if (pe != NIL) S.op[pe] = e;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) {
      const int last = incl > before ? incl : before;
      carry = last;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    SysState& R = *S.st;
    R.ovf = carry >= 0 ? init_slot(carry, N, grow) : NIL;
    if (R.ovf != NIL) S.op[R.ovf] = NIL;
    R.C = (uint64_t)(grow ? 3 : 2) + 2ull * N;
    R.npred = (uint64_t)N;
    R.lastThermo = 0;
    R.collT[0] = R.collT[1] = 0;
  }
}

// one block per system: the leaves in parallel, then one level at a time
// with a warp per parent node
__global__ void __launch_bounds__(256) k_tree_build(const SysDev* __restrict__ sys, int nsys) {
  const int s = blockIdx.x;
  if (s >= nsys) return;
  const SysDev& S = sys[s];
  const int N = S.B.N;
  for (int l = threadIdx.x; l < S.L; l += blockDim.x) {
    Node n = empty_node(l);
    if (l < N) {
      Ev e0 = S.ev[l], e1 = S.ev[N + l];
      if (e0.st == ST_QUEUED) n = ev_node(e0, l);
      if (e1.st == ST_QUEUED) { Node m = ev_node(e1, l); if (node_less(m, n)) n = m; }
    } else {
      Ev e = S.ev[2 * N + (l - N)];
      if (e.st == ST_QUEUED) n = ev_node(e, l);
    }
    S.tree[l] = n;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int h = 1; h < S.nlev; h++) {
    for (int par = w; par < S.lev_cnt[h]; par += nw) {
      const int ch = (par << 5) + lane;
      Node c = ch < S.lev_cnt[h - 1] ? S.tree[S.lev_off[h - 1] + ch] : empty_node(0x7fffffff);
      grp_min(c, Grp<32>(threadIdx.x));
      if (lane == 0) S.tree[S.lev_off[h] + par] = c;
    }
    __syncthreads();
  }
}

__global__ void k_sync(const SysDev* __restrict__ sys, int nsys) {
  int s = blockIdx.x;
  if (s >= nsys) return;
  const SysDev& S = sys[s];
  const double t = S.st->t;
  const bool grow = S.st->grow != 0;
  for (int i = threadIdx.x; i < S.B.N; i += blockDim.x) {
    Disk p = S.d[i];
    grow_fly(S, p, i, t, grow);
    S.d[i] = p;
  }
}

// disk records of every system -> concatenated SoA staging (x y vx vy rad m)
__global__ void k_gather(const Disk* __restrict__ d, int64_t total, double* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  Disk p = d[i];
  out[i] = p.x; out[total + i] = p.y; out[2 * total + i] = p.vx;
  out[3 * total + i] = p.vy; out[4 * total + i] = p.rad; out[5 * total + i] = p.m;
}

}  // namespace

// ==================================================================== C ABI

#include "edmd_ctx.h"

static int g_engine = EDMD_ENGINE_AUTO;
static int g_lane_threads = 32;
static int g_group = 32;                        // warp engine: lanes per system

extern "C" int edmd_set_engine(int32_t kind) {
  if (kind < EDMD_ENGINE_AUTO || kind > EDMD_ENGINE_LANE) return EDMD_ERR_ARG;
  g_engine = kind;
  return EDMD_OK;
}

extern "C" int edmd_set_lane_threads(int32_t threads_per_block) {
  if (threads_per_block < 1 || threads_per_block > 1024) return EDMD_ERR_ARG;
  g_lane_threads = threads_per_block;
  return EDMD_OK;
}

extern "C" int edmd_set_warp_group(int32_t lanes) {
  if (lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32) return EDMD_ERR_ARG;
  g_group = lanes;
  return EDMD_OK;
}

extern "C" int edmd_device_info(char* name, int32_t cap, int32_t* sm_count) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return EDMD_ERR_NODEV;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) return EDMD_ERR_CUDA;
  if (name && cap > 0) { strncpy(name, p.name, cap - 1); name[cap - 1] = 0; }
  if (sm_count) *sm_count = p.multiProcessorCount;
  return EDMD_OK;
}



// host threads for staging n disks: one below 2^16 disks, else up to 16
static int staging_threads(int64_t n) {
  if (n < ((int64_t)1 << 16)) return 1;
  const unsigned hc = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(hc, 16u));
}

// run f(0) .. f(n-1), on n threads where they can be had (inline otherwise)
template <class F>
static void run_threads(int n, F&& f) {
  std::vector<std::thread> pool;
  for (int k = 1; k < n; k++) {
    try {
      pool.emplace_back(f, k);
    } catch (...) {
      f(k);
    }
  }
  f(0);
  for (auto& th : pool) th.join();
}

// (Re)initialise every system from host arrays: the cell lists are built on
// the host in index order (cellListInit src/EDMD.c:1906 -> addToCell 2053,
// push-front), the event set on the device (eventListInit 1935).
// first_screen/first_thermo/t_growstop per system come from `desc` unless
// `restart`, which follows the -l load path: normal phase, firstScreen 1,
// firstThermo 1000 (src/EDMD.c:244-247; eventListInit 1958 skips the growth
// shift when load != 0).
static int stage_all(edmd_ctx* ctx, const double* x, const double* y, const double* vx,
                     const double* vy, const double* rad, const double* m, const double* vr,
                     bool restart) {
  ctx->round_dirty = false;
  const int64_t TN = ctx->total_N;
  const int nsys = ctx->nsys;
  // every field of every staged record is written below
  std::unique_ptr<Disk[]> hd(new Disk[TN]);
  std::unique_ptr<int32_t[]> hcx(new int32_t[TN]), hcy(new int32_t[TN]), hprv(new int32_t[TN]);
  std::vector<int32_t> hhead(ctx->total_C, NIL);
  std::vector<SysState> hst(nsys);
  const int nth = staging_threads(TN);
  // records and cells, disk by disk, in contiguous slices of the concatenated
  // disks; each slice stops at its first bad disk, so the smallest of those is
  // the first bad disk in index order (2 g: position, 2 g + 1: radius)
  std::vector<int64_t> bad(nth, INT64_MAX);
  run_threads(nth, [&](int k) {
    const int64_t lo = TN * k / nth, hi = TN * (k + 1) / nth;
    int s = (int)(std::upper_bound(ctx->disk_off.begin(), ctx->disk_off.end(), lo) - ctx->disk_off.begin()) - 1;
    for (int64_t g = lo; g < hi; g++) {
      while (s + 1 < nsys && g >= ctx->disk_off[s + 1]) s++;
      const Box& B = ctx->hs[s].B;
      const edmd_system_desc& D = ctx->desc[s];
      double px = x[g], py = y[g];
      if (restart) {                     // PBCpostX/Y on loaded positions (src/EDMD.c:1405-1406)
        if (px < 0) px += D.Lx; else if (px >= D.Lx) px -= D.Lx;
        if (py < 0) py += D.Ly; else if (py >= D.Ly) py -= D.Ly;
      }
      if (!(px >= 0 && px < D.Lx && py >= 0 && py < D.Ly)) { bad[k] = 2 * g; return; }
      if (!radius_ok(rad[g])) { bad[k] = 2 * g + 1; return; }
      Disk& q = hd[g];
      q.x = px; q.y = py; q.vx = vx[g]; q.vy = vy[g]; q.tl = 0; q.rad = rad[g]; q.m = m[g];
      q.coll = 0;
      int X = (int)(q.x * B.cxf), Y = (int)(q.y * B.cyf);
      if (X >= B.Nxc) X = B.Nxc - 1;
      if (Y >= B.Nyc) Y = B.Nyc - 1;
      hcx[g] = X; hcy[g] = Y;
    }
  });
  const int64_t first_bad = *std::min_element(bad.begin(), bad.end());
  if (first_bad != INT64_MAX) {
    const int64_t g = first_bad / 2;
    const int s = (int)(std::upper_bound(ctx->disk_off.begin(), ctx->disk_off.end(), g) - ctx->disk_off.begin()) - 1;
    return set_err(ctx, EDMD_ERR_ARG, std::string(first_bad % 2 ? "radius not zero or normal positive"
                                                                  : "position outside the box") +
                                          " (system " + std::to_string(s) + ")");
  }
  // cell lists, system by system: push-front in index order (cellListInit
  // src/EDMD.c:1906 -> addToCell 2053)
  run_threads(std::min(nth, nsys), [&](int k) {
    for (int s = k; s < nsys; s += std::min(nth, nsys)) {
      const Box& B = ctx->hs[s].B;
      const int64_t o = ctx->disk_off[s];
      int32_t* head = hhead.data() + ctx->cell_off[s];
      for (int64_t i = 0; i < B.N; i++) {
        const int64_t g = o + i;
        const int c = hcy[g] * B.Nxc + hcx[g];
        hprv[g] = NIL;
        hd[g].nxt = head[c];
        head[c] = (int32_t)i;
        if (hd[g].nxt != NIL) hprv[o + hd[g].nxt] = (int32_t)i;
      }
    }
  });
  for (int s = 0; s < nsys; s++) {
    const SysDev& S = ctx->hs[s];
    const Box& B = S.B;
    const edmd_system_desc& D = ctx->desc[s];
    SysState& st = hst[s];
    memset(&st, 0, sizeof(st));
    st.k = 0; st.next_wrap = (uint64_t)B.N; st.ovf = NIL;
    st.grow = (!restart && D.t_growstop > 0) ? 1 : 0;
    double fs = restart ? 1.0 : D.first_screen, ft = restart ? 1000.0 : D.first_thermo;
    st.lastThermo = ft + 0.000000001;   // addEventThermo(firstThermo + 1e-9), read by k_init_events
    st.collT[0] = st.grow ? D.t_growstop : -1;
    st.collT[1] = fs;
  }
  cudaStream_t sm = ctx->stream;
  CK(cudaMemcpyAsync(ctx->st, hst.data(), ctx->nsys * sizeof(SysState), cudaMemcpyHostToDevice, sm));
  CK(cudaMemcpyAsync(ctx->d, hd.get(), TN * sizeof(Disk), cudaMemcpyHostToDevice, sm));
  if (vr && !restart) CK(cudaMemcpyAsync(ctx->vr, vr, TN * 8, cudaMemcpyHostToDevice, sm));
  else if (!vr && !restart) CK(cudaMemsetAsync(ctx->vr, 0, TN * 8, sm));
  CK(cudaMemcpyAsync(ctx->cx, hcx.get(), TN * 4, cudaMemcpyHostToDevice, sm));
  CK(cudaMemcpyAsync(ctx->cy, hcy.get(), TN * 4, cudaMemcpyHostToDevice, sm));
  CK(cudaMemcpyAsync(ctx->prv, hprv.get(), TN * 4, cudaMemcpyHostToDevice, sm));
  CK(cudaMemsetAsync(ctx->crossX, 0, TN * 4, sm));
  CK(cudaMemsetAsync(ctx->crossY, 0, TN * 4, sm));
  CK(cudaMemcpyAsync(ctx->head, hhead.data(), ctx->total_C * 4, cudaMemcpyHostToDevice, sm));
  dim3 g((ctx->maxN + 1 + 127) / 128, ctx->nsys);
  k_init_events<<<g, 128, 0, sm>>>(ctx->ds);
  k_init_finish<<<ctx->nsys, 256, 0, sm>>>(ctx->ds, ctx->nsys);
  if (ctx->engine == EDMD_ENGINE_LANE) CK(lane_build(ctx->ds, ctx->nsys, sm));
  else k_tree_build<<<ctx->nsys, 256, 0, sm>>>(ctx->ds, ctx->nsys);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(sm));   // host staging vectors go out of scope
  return report_status(ctx, "initial configuration");
}

extern "C" int edmd_create(int32_t nsys, const edmd_system_desc* desc, const double* x,
                           const double* y, const double* vx, const double* vy,
                           const double* rad, const double* m, const double* vr,
                           int64_t trace_cap, edmd_ctx** out) {
  if (!out || nsys <= 0 || !desc || !x || !y || !vx || !vy || !rad || !m || trace_cap < 0)
    return EDMD_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return EDMD_ERR_NODEV;
  edmd_ctx* ctx = new edmd_ctx();
  *out = ctx;
  ctx->nsys = nsys;
  ctx->hs.resize(nsys);
  ctx->desc.assign(desc, desc + nsys);
  ctx->disk_off.resize(nsys);
  ctx->cell_off.resize(nsys);
  const int rows_cap = 1024;
  std::vector<int64_t> ev_off(nsys), node_off(nsys);
  int64_t TN = 0, TC = 0, TE = 0, TT = 0;
  for (int s = 0; s < nsys; s++) {
    const edmd_system_desc& D = desc[s];
    if (D.N < 2 || !(D.Lx > 0) || !(D.Ly > 0) || (D.contact != EDMD_CONTACT_NONADDITIVE &&
                                                     D.contact != EDMD_CONTACT_ADDITIVE))
      return set_err(ctx, EDMD_ERR_ARG, "bad system descriptor");
    SysDev& S = ctx->hs[s];
    memset(&S, 0, sizeof(S));
    Box& B = S.B;
    B.N = D.N; B.Lx = D.Lx; B.Ly = D.Ly;
    B.additive = D.contact == EDMD_CONTACT_ADDITIVE;
    if (B.additive) ctx->any_additive = true;
    B.hLx = D.Lx / 2; B.hLy = D.Ly / 2;                      // boxConstantHelper 679-714
    B.Nyc = (int)(B.hLy); B.Nxc = (int)(B.hLx);
    if (B.Nxc < 1 || B.Nyc < 1) return set_err(ctx, EDMD_ERR_ARG, "box smaller than one cell");
    B.cxs = D.Lx / B.Nxc; B.cys = D.Ly / B.Nyc;
    B.cxf = 1 / B.cxs; B.cyf = 1 / B.cys;
    B.dtP = 5.0 / (double)D.N;
    B.dtPN = B.dtP * D.N;
    S.rdtP = 1.0 / B.dtP;
    S.res = D.res; S.Einit = D.Einit; S.dtime = D.dtime; S.dtimeTh = D.dtime_thermo; S.tmax = D.tmax;
    S.L = D.N + NSPECIAL;
    int c = S.L;
    S.nlev = 0;
    int64_t nodes = 0;
    for (;;) {
      if (S.nlev >= MAXLEV) return set_err(ctx, EDMD_ERR_ARG, "system too large");
      S.lev_off[S.nlev] = (int32_t)nodes; S.lev_cnt[S.nlev] = c; nodes += c; S.nlev++;
      if (c == 1) break;
      c = (c + 31) / 32;
    }
    ctx->disk_off[s] = TN; ctx->cell_off[s] = TC; ev_off[s] = TE; node_off[s] = TT;
    TN += D.N; TC += (int64_t)B.Nxc * B.Nyc; TE += 2 * (int64_t)D.N + NSPECIAL; TT += nodes;
    if (D.N > ctx->maxN) ctx->maxN = D.N;
  }
  ctx->total_N = TN; ctx->total_C = TC;
  ctx->engine = g_engine;
  if (ctx->engine == EDMD_ENGINE_AUTO) {
    // One thread per system issues each FP64 instruction for up to 32
    // systems, but needs enough systems to hide its dependent loads: measured
    // on GB300 (Hex starts at phi 0.55, 2000 collisions a call), the lane
    // engine runs 2.9e7 / 5.2e7 / 9.3e7 / 1.6e8 coll/s at 4096 / 8192 /
    // 16384 / 32768 systems of 256 disks against 7.5e7 / 7.5e7 / 8.4e7 /
    // 8.5e7 for one warp per system (16384 systems of 1024 disks: 9.4e7
    // against 7.6e7).  Its calendar costs ~2 KB per disk.
    const bool many = nsys >= 16384 && 2 * (int64_t)ctx->maxN + NSPECIAL <= 65535 &&
                      TN * (int64_t)(CAL_SUB * CAL_LINE * 2 + 2) <= ((int64_t)32 << 30);
    ctx->engine = many ? EDMD_ENGINE_LANE : EDMD_ENGINE_WARP;
  }
  if (ctx->engine == EDMD_ENGINE_LANE && 2 * (int64_t)ctx->maxN + NSPECIAL > 65535)
    return set_err(ctx, EDMD_ERR_ARG, "thread-per-system engine supports N <= 32766");
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&ctx->e0));
  CK(cudaEventCreate(&ctx->e1));
  CK(dalloc(&ctx->d, TN)); CK(dalloc(&ctx->vr, TN));
  CK(dalloc(&ctx->cx, TN)); CK(dalloc(&ctx->cy, TN)); CK(dalloc(&ctx->prv, TN));
  CK(dalloc(&ctx->crossX, TN)); CK(dalloc(&ctx->crossY, TN));
  CK(dalloc(&ctx->head, TC));
  CK(dalloc(&ctx->ev, TE)); CK(dalloc(&ctx->on, TE)); CK(dalloc(&ctx->op, TE));
  CK(dalloc(&ctx->tree, TT));
  CK(dalloc(&ctx->st, nsys));
  CK(dalloc(&ctx->trace, (size_t)nsys * trace_cap));
  CK(dalloc(&ctx->rows, (size_t)nsys * rows_cap * 9));
  CK(dalloc(&ctx->work, 1));
  CK(dalloc(&ctx->order, nsys));
  CK(dalloc(&ctx->cost, nsys));
  CK(cudaMemsetAsync(ctx->cost, 0, nsys * sizeof(uint32_t), ctx->stream));
  CK(dalloc(&ctx->ds, nsys));
  if (ctx->engine == EDMD_ENGINE_LANE) {
    CK(dalloc(&ctx->cal, (size_t)TN * CAL_SUB * CAL_LINE));
    CK(dalloc(&ctx->mask, (size_t)TN));
  }
  for (int s = 0; s < nsys; s++) {
    SysDev& S = ctx->hs[s];
    int64_t o = ctx->disk_off[s];
    S.d = ctx->d + o; S.vr = ctx->vr + o;
    S.cx = ctx->cx + o; S.cy = ctx->cy + o; S.prv = ctx->prv + o;
    S.crossX = ctx->crossX + o; S.crossY = ctx->crossY + o;
    S.head = ctx->head + ctx->cell_off[s];
    S.ev = ctx->ev + ev_off[s]; S.on = ctx->on + ev_off[s]; S.op = ctx->op + ev_off[s];
    S.tree = ctx->tree + node_off[s];
    S.st = ctx->st + s;
    S.trace = trace_cap > 0 ? (void*)(ctx->trace + (size_t)s * trace_cap) : nullptr;
    S.trace_cap = trace_cap;
    S.rows = ctx->rows + (size_t)s * rows_cap * 9;
    S.rows_cap = rows_cap;
    if (ctx->engine == EDMD_ENGINE_LANE) {
      S.cal = ctx->cal + (size_t)o * CAL_SUB * CAL_LINE;
      S.mask = ctx->mask + o;
      S.invw = CAL_SUB / S.B.dtP;
    }
  }
  CK(cudaMemcpyAsync(ctx->ds, ctx->hs.data(), nsys * sizeof(SysDev), cudaMemcpyHostToDevice, ctx->stream));
  return stage_all(ctx, x, y, vx, vy, rad, m, vr, false);
}

extern "C" int edmd_load_state(edmd_ctx* ctx, const double* x, const double* y, const double* vx,
                               const double* vy, const double* rad, const double* m) {
  if (!ctx || !x || !y || !vx || !vy || !rad || !m) return EDMD_ERR_ARG;
  return stage_all(ctx, x, y, vx, vy, rad, m, nullptr, true);
}

// EDMD_F_SMEM: the systems whose engine state fits one block's shared memory
// go to k_run_smem on a second stream, the others to k_run on the context's
// stream (longest first by the previous call's run times, as without the
// flag); both start after e0 and the context's stream waits for the second
// one before e1.
static int advance_smem_split(edmd_ctx* ctx, RunArgs A, int kgrid_max, int nsm) {
  int dev = 0, optin = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t limit = (size_t)optin - sizeof(WarpSmem) - 1024;
  std::vector<uint32_t> cost(ctx->nsys);
  CK(sync_copy(ctx, cost.data(), ctx->cost, ctx->nsys * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  std::vector<int32_t> fit, rest;
  size_t need = 0;
  for (int s = 0; s < ctx->nsys; s++) {
    const size_t b = smem_layout(ctx->hs[s]).total;
    if (b <= limit) { fit.push_back(s); need = b > need ? b : need; }
    else rest.push_back(s);
  }
  auto longest_first = [&](std::vector<int32_t>& v) {
    std::stable_sort(v.begin(), v.end(), [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
  };
  longest_first(fit);
  longest_first(rest);
  if (!ctx->smem_list) {
    CK(dalloc(&ctx->smem_list, ctx->nsys));
    CK(dalloc(&ctx->smem_work, 1));
    CK(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->e2, cudaEventDisableTiming));
  }
  if (!rest.empty())
    CK(cudaMemcpyAsync(ctx->order, rest.data(), rest.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                       ctx->stream));
  if (!fit.empty())
    CK(cudaMemcpyAsync(ctx->smem_list, fit.data(), fit.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                       ctx->stream));
  CK(cudaMemsetAsync(ctx->smem_work, 0, sizeof(int32_t), ctx->stream));
  CK(cudaEventRecord(ctx->e0, ctx->stream));
  if (!fit.empty()) {
    CK(cudaFuncSetAttribute(k_run_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
    int per = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_run_smem, 32, need));
    int g = per * nsm;
    if (g > (int)fit.size()) g = (int)fit.size();
    if (g < 1) g = 1;
    CK(cudaStreamWaitEvent(ctx->stream2, ctx->e0, 0));
    k_run_smem<<<g, 32, need, ctx->stream2>>>(ctx->ds, A, ctx->smem_list, (int)fit.size(), ctx->smem_work);
    CK(cudaGetLastError());
    ctx->last_launches++;
    CK(cudaEventRecord(ctx->e2, ctx->stream2));
  }
  if (!rest.empty()) {
    RunArgs B = A;
    B.nsys = (int32_t)rest.size();
    B.order = ctx->order;
    const int per_block = WARPS_PER_BLOCK;
    int grid = ((int)rest.size() + per_block - 1) / per_block;
    if (grid > kgrid_max) grid = kgrid_max;
    if (ctx->any_additive) k_run<32><<<grid, 32 * WARPS_PER_BLOCK, 0, ctx->stream>>>(ctx->ds, B);
    else k_run<32, false><<<grid, 32 * WARPS_PER_BLOCK, 0, ctx->stream>>>(ctx->ds, B);
    CK(cudaGetLastError());
    ctx->last_launches++;
  }
  if (!fit.empty()) CK(cudaStreamWaitEvent(ctx->stream, ctx->e2, 0));
  return EDMD_OK;
}

extern "C" int edmd_advance(edmd_ctx* ctx, int64_t max_coll, double t_stop, uint32_t flags,
                            int64_t max_events, float* elapsed_ms) {
  if (!ctx) return EDMD_ERR_ARG;
  if (max_coll < 0 || max_events <= 0) return set_err(ctx, EDMD_ERR_ARG, "bad advance limits");
  if (ctx->round_dirty)
    return set_err(ctx, EDMD_ERR_ARG, "advanced by the round engine: reload the state with edmd_load_state");
  RunArgs A;
  A.max_coll = max_coll; A.t_stop = t_stop; A.flags = flags; A.max_events = max_events;
  A.nsys = ctx->nsys; A.work = ctx->work;
  A.order = nullptr; A.cost = ctx->cost;
  if (ctx->engine == EDMD_ENGINE_LANE) {
    CK(cudaEventRecord(ctx->e0, ctx->stream));
    CK(lane_run_launch(ctx->ds, A, g_lane_threads, ctx->stream));
    ctx->last_launches = 1;
  } else {
    CK(cudaMemsetAsync(ctx->work, 0, sizeof(int32_t), ctx->stream));
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int per_sm = 0;
    const int gw = g_group;                     // lanes per system: 4, 8, 16 or 32
    const int per_block = WARPS_PER_BLOCK * (32 / gw);
    if (gw == 4) CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_run<4>, 32 * WARPS_PER_BLOCK, 0));
    else if (gw == 8) CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_run<8>, 32 * WARPS_PER_BLOCK, 0));
    else if (gw == 16) CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_run<16>, 32 * WARPS_PER_BLOCK, 0));
    else CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_run<32>, 32 * WARPS_PER_BLOCK, 0));
    int want = (ctx->nsys + per_block - 1) / per_block;
    int grid = per_sm * nsm;
    if (grid > want) grid = want;
    if (grid < 1) grid = 1;
    // more systems than resident warps: with one item per system the last
    // wave runs on part of the GPU; chunks of the collision budget let the
    // warps share the remaining work evenly (same events, same results)
    const int64_t resident = (int64_t)grid * per_block;
    if (ctx->nsys > resident) {
      // more systems than resident warps: the systems that took longest in
      // the previous call start first (longest processing time first), so the
      // last wave holds the short ones and the launch ends with fewer idle
      // warps; ties keep index order, and the first call runs in index order
      std::vector<uint32_t> cost(ctx->nsys);
      CK(sync_copy(ctx, cost.data(), ctx->cost, ctx->nsys * sizeof(uint32_t), cudaMemcpyDeviceToHost));
      std::vector<int32_t>& ord = ctx->order_h;
      ord.resize(ctx->nsys);
      for (int s = 0; s < ctx->nsys; s++) ord[s] = s;
      std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
      CK(cudaMemcpyAsync(ctx->order, ord.data(), ctx->nsys * sizeof(int32_t), cudaMemcpyHostToDevice,
                         ctx->stream));
      A.order = ctx->order;
    }
    ctx->last_launches = 0;
    if ((flags & EDMD_F_SMEM) && gw == 32) {
      int rc = advance_smem_split(ctx, A, per_sm * nsm, nsm);
      if (rc) return rc;
    } else {
    ctx->last_launches = 1;
    CK(cudaEventRecord(ctx->e0, ctx->stream));
    if (gw == 4) k_run<4><<<grid, 32 * WARPS_PER_BLOCK, 0, ctx->stream>>>(ctx->ds, A);
    else if (gw == 8) k_run<8><<<grid, 32 * WARPS_PER_BLOCK, 0, ctx->stream>>>(ctx->ds, A);
    else if (gw == 16) k_run<16><<<grid, 32 * WARPS_PER_BLOCK, 0, ctx->stream>>>(ctx->ds, A);
    else if (ctx->any_additive) k_run<32><<<grid, 32 * WARPS_PER_BLOCK, 0, ctx->stream>>>(ctx->ds, A);
    else k_run<32, false><<<grid, 32 * WARPS_PER_BLOCK, 0, ctx->stream>>>(ctx->ds, A);
    }
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->e1, ctx->stream));
  CK(cudaEventSynchronize(ctx->e1));
  CK(cudaEventElapsedTime(&ctx->last_ms, ctx->e0, ctx->e1));
  if (elapsed_ms) *elapsed_ms = ctx->last_ms;
  return report_status(ctx, "advance");
}

extern "C" int edmd_sync(edmd_ctx* ctx) {
  if (!ctx) return EDMD_ERR_ARG;
  k_sync<<<ctx->nsys, 256, 0, ctx->stream>>>(ctx->ds, ctx->nsys);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return EDMD_OK;
}

extern "C" int edmd_get_state(edmd_ctx* ctx, int32_t s, double* x, double* y, double* vx,
                              double* vy, double* rad, double* m, int32_t* cell, uint32_t* coll) {
  if (!ctx || s < 0 || s >= ctx->nsys) return EDMD_ERR_ARG;
  const SysDev& S = ctx->hs[s];
  int N = S.B.N;
  std::vector<Disk> hd(N);
  std::vector<int32_t> hcx(N), hcy(N);
  CK(sync_copy(ctx, hd.data(), S.d, N * sizeof(Disk), cudaMemcpyDeviceToHost));
  CK(sync_copy(ctx, hcx.data(), S.cx, N * 4, cudaMemcpyDeviceToHost));
  CK(sync_copy(ctx, hcy.data(), S.cy, N * 4, cudaMemcpyDeviceToHost));
  for (int i = 0; i < N; i++) {
    if (x) x[i] = hd[i].x;
    if (y) y[i] = hd[i].y;
    if (vx) vx[i] = hd[i].vx;
    if (vy) vy[i] = hd[i].vy;
    if (rad) rad[i] = hd[i].rad;
    if (m) m[i] = hd[i].m;
    if (cell) cell[i] = hcy[i] * S.B.Nxc + hcx[i];
    if (coll) coll[i] = hd[i].coll;
  }
  return EDMD_OK;
}

extern "C" int edmd_get_states(edmd_ctx* ctx, double* x, double* y, double* vx, double* vy,
                               double* rad, double* m) {
  if (!ctx) return EDMD_ERR_ARG;
  const int64_t TN = ctx->total_N;
  if (!ctx->stage) CK(dalloc(&ctx->stage, 6 * TN));
  k_gather<<<(unsigned)((TN + 255) / 256), 256, 0, ctx->stream>>>(ctx->d, TN, ctx->stage);
  CK(cudaGetLastError());
  double* outs[6] = {x, y, vx, vy, rad, m};
  for (int k = 0; k < 6; k++)
    if (outs[k]) CK(cudaMemcpyAsync(outs[k], ctx->stage + k * TN, TN * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return EDMD_OK;
}

extern "C" int edmd_get_counters(edmd_ctx* ctx, int32_t s, edmd_counters* out) {
  if (!ctx || s < 0 || s >= ctx->nsys || !out) return EDMD_ERR_ARG;
  SysState R;
  CK(sync_copy(ctx, &R, ctx->hs[s].st, sizeof(R), cudaMemcpyDeviceToHost));
  out->ncol = R.ncol; out->ncol_total = R.ncol_total; out->ncross = R.ncross;
  out->nstale = R.nstale; out->npair = R.npair; out->npred = R.npred; out->nevents = R.nevents;
  out->nscreen = R.nscreen;
  out->t = R.t; out->growing = R.grow; out->stop_reason = R.stop_reason;
  return EDMD_OK;
}

extern "C" int edmd_get_all_counters(edmd_ctx* ctx, edmd_counters* out) {
  if (!ctx || !out) return EDMD_ERR_ARG;
  std::vector<SysState> R(ctx->nsys);
  CK(sync_copy(ctx, R.data(), ctx->st, ctx->nsys * sizeof(SysState), cudaMemcpyDeviceToHost));
  for (int s = 0; s < ctx->nsys; s++) {
    edmd_counters& o = out[s];
    o.ncol = R[s].ncol; o.ncol_total = R[s].ncol_total; o.ncross = R[s].ncross;
    o.nstale = R[s].nstale; o.npair = R[s].npair; o.npred = R[s].npred; o.nevents = R[s].nevents;
    o.nscreen = R[s].nscreen;
    o.t = R[s].t; o.growing = R[s].grow; o.stop_reason = R[s].stop_reason;
  }
  return EDMD_OK;
}

extern "C" int edmd_get_virial(edmd_ctx* ctx, int32_t s, double out[4], int32_t reset) {
  if (!ctx || s < 0 || s >= ctx->nsys || !out) return EDMD_ERR_ARG;
  SysState* p = ctx->hs[s].st;
  CK(sync_copy(ctx, out, p->collT, 4 * sizeof(double), cudaMemcpyDeviceToHost));
  if (reset) CK(sync_set(ctx, p->collT, 0, 4 * sizeof(double)));
  return EDMD_OK;
}

extern "C" int edmd_get_thermo(edmd_ctx* ctx, int32_t s, double* rows, int32_t cap, int32_t* n) {
  if (!ctx || s < 0 || s >= ctx->nsys || !n) return EDMD_ERR_ARG;
  const SysDev& S = ctx->hs[s];
  int32_t nr = 0;
  CK(sync_copy(ctx, &nr, &S.st->nrows, 4, cudaMemcpyDeviceToHost));
  *n = nr;
  int k = nr < cap ? nr : cap;
  if (k > S.rows_cap) k = S.rows_cap;
  if (rows && k > 0) CK(sync_copy(ctx, rows, S.rows, (size_t)k * 9 * 8, cudaMemcpyDeviceToHost));
  return nr > S.rows_cap ? EDMD_ERR_CAPACITY : EDMD_OK;
}

extern "C" int edmd_take_thermo(edmd_ctx* ctx, int32_t s, double* rows, int32_t cap, int32_t* n) {
  const int rc = edmd_get_thermo(ctx, s, rows, cap, n);
  if (rc != EDMD_OK && rc != EDMD_ERR_CAPACITY) return rc;
  const int32_t zero = 0;
  CK(sync_copy(ctx, &ctx->hs[s].st->nrows, &zero, 4, cudaMemcpyHostToDevice));
  return rc;
}

extern "C" int edmd_get_trace(edmd_ctx* ctx, int32_t s, edmd_collision* out, int64_t cap, int64_t* n) {
  if (!ctx || s < 0 || s >= ctx->nsys || !n) return EDMD_ERR_ARG;
  const SysDev& S = ctx->hs[s];
  uint64_t nt = 0;
  CK(sync_copy(ctx, &nt, &S.st->ntrace, 8, cudaMemcpyDeviceToHost));
  *n = (int64_t)nt;
  int64_t k = (int64_t)nt < cap ? (int64_t)nt : cap;
  if (k > S.trace_cap) k = S.trace_cap;
  if (out && k > 0) CK(sync_copy(ctx, out, S.trace, k * sizeof(edmd_collision), cudaMemcpyDeviceToHost));
  return (int64_t)nt > S.trace_cap ? EDMD_ERR_CAPACITY : EDMD_OK;
}

extern "C" int edmd_set_device(int32_t dev) {
  return cudaSetDevice(dev) == cudaSuccess ? EDMD_OK : EDMD_ERR_CUDA;
}

extern "C" int edmd_host_alloc(void** p, int64_t bytes) {
  if (!p || bytes <= 0) return EDMD_ERR_ARG;
  return cudaMallocHost(p, (size_t)bytes) == cudaSuccess ? EDMD_OK : EDMD_ERR_CUDA;
}

extern "C" int edmd_host_free(void* p) {
  return cudaFreeHost(p) == cudaSuccess ? EDMD_OK : EDMD_ERR_CUDA;
}

extern "C" int edmd_destroy(edmd_ctx* ctx) {
  if (!ctx) return EDMD_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  round_free(ctx);
  void* ptrs[] = {ctx->d, ctx->vr, ctx->cx, ctx->cy, ctx->prv, ctx->crossX, ctx->crossY, ctx->head,
                  ctx->ev, ctx->on, ctx->op, ctx->tree, ctx->st, ctx->trace, ctx->rows, ctx->stage,
                  ctx->work, ctx->order, ctx->cost, ctx->ds, ctx->cal, ctx->mask};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (void* p : ctx->ckpt)
    if (p) cudaFree(p);
  if (ctx->logbuf) cudaFree(ctx->logbuf);
  if (ctx->e0) cudaEventDestroy(ctx->e0);
  if (ctx->e1) cudaEventDestroy(ctx->e1);
  if (ctx->c0) cudaEventDestroy(ctx->c0);
  if (ctx->e2) cudaEventDestroy(ctx->e2);
  if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
  if (ctx->smem_list) cudaFree(ctx->smem_list);
  if (ctx->smem_work) cudaFree(ctx->smem_work);
  if (ctx->c1) cudaEventDestroy(ctx->c1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return EDMD_OK;
}

extern "C" int edmd_get_engine(const edmd_ctx* ctx) {
  return ctx ? ctx->engine : -1;
}

extern "C" int edmd_get_last_ms(const edmd_ctx* ctx, float* ms) {
  if (!ctx || !ms) return EDMD_ERR_ARG;
  *ms = ctx->last_ms;
  return EDMD_OK;
}

extern "C" int edmd_get_last_launches(const edmd_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return EDMD_ERR_ARG;
  *n = ctx->last_launches;
  return EDMD_OK;
}

// ==================================================================== allocation-free entry point
//
// edmd_run_noalloc serves callers that must not allocate device memory, for
// example code that runs inside a latency-critical loop or a host framework
// that owns every device buffer and forbids cudaMalloc/cudaFree after start-up.
// The caller passes its own device arrays (the state in and out); everything
// the engine needs besides them -- the system descriptor, cell lists, event
// records, the tournament tree, the scalar state and the work counter -- lives
// in the file-scope array below, which every GPU that loads this library keeps
// until the process exits.
namespace {
constexpr int64_t NOALLOC_MAX_N = 8192;        // disks per call
constexpr int64_t NOALLOC_MAX_CELLS = 65536;   // Nxcells * Nycells per call
constexpr size_t NOALLOC_BYTES = (size_t)4 << 20;
constexpr int NOALLOC_MAX_DEVICES = 64;
// event budget of one call (see edmd_run_noalloc)
constexpr int64_t NOALLOC_EVENTS_PER_COLL = 256, NOALLOC_EVENTS_PER_DISK = 256, NOALLOC_EVENTS_BASE = 1 << 20;
}

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];
static unsigned char* g_noalloc_addr[NOALLOC_MAX_DEVICES];   // device address, per device
static thread_local std::string g_noalloc_err;

namespace {

__global__ void k_noalloc_put(SysDev s, SysDev* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = s;
}

// disk records, cell lists (index order, push-front as addToCell) and the
// scalar state from the caller's device arrays; one thread, N <= 8192.
// A position outside [0, Lx) x [0, Ly) (or a NaN), or a radius that is not
// zero or normal positive, is an argument error, as in edmd_create: the
// scalar state gets status EDMD_ERR_ARG with the first such
// disk in err_a, the event loop then does nothing, and the host reports it.
// The cell index is still clamped into the grid so that the initial
// predictions that run before the loop stay inside the arrays.
__global__ void k_noalloc_stage(const SysDev* __restrict__ sys, const double* x, const double* y,
                                const double* vx, const double* vy, const double* rad,
                                const double* m, double first_screen, double first_thermo) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const SysDev& S = sys[0];
  const Box& B = S.B;
  const int N = B.N;
  int bad = -1;
  for (int c = 0; c < B.Nxc * B.Nyc; c++) S.head[c] = NIL;
  for (int i = 0; i < N; i++) {
    Disk q;
    q.x = x[i]; q.y = y[i]; q.vx = vx[i]; q.vy = vy[i]; q.tl = 0; q.rad = rad[i]; q.m = m[i];
    q.coll = 0;
    if (bad < 0 && !(q.x >= 0 && q.x < B.Lx && q.y >= 0 && q.y < B.Ly && radius_ok(q.rad))) bad = i;
    int X = (int)(q.x * B.cxf), Y = (int)(q.y * B.cyf);
    if (!(X < B.Nxc)) X = B.Nxc - 1;
    if (!(Y < B.Nyc)) Y = B.Nyc - 1;
    if (!(X >= 0)) X = 0;
    if (!(Y >= 0)) Y = 0;
    S.cx[i] = X; S.cy[i] = Y; S.prv[i] = NIL;
    S.crossX[i] = 0; S.crossY[i] = 0;
    S.vr[i] = 0;
    q.nxt = S.head[Y * B.Nxc + X];
    S.head[Y * B.Nxc + X] = i;
    if (q.nxt != NIL) S.prv[q.nxt] = i;
    S.d[i] = q;
  }
  SysState st;
  memset(&st, 0, sizeof(st));
  st.k = 0; st.next_wrap = (uint64_t)N; st.ovf = NIL; st.grow = 0;
  st.lastThermo = first_thermo + 0.000000001;   // read by k_init_events
  st.collT[0] = -1;
  st.collT[1] = first_screen;
  if (bad >= 0) { st.status = EDMD_ERR_ARG; st.err_a = bad; }
  *S.st = st;
}

__global__ void k_noalloc_out(const SysDev* __restrict__ sys, double* x, double* y, double* vx,
                              double* vy) {
  const SysDev& S = sys[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.B.N; i += gridDim.x * blockDim.x) {
    Disk p = S.d[i];
    x[i] = p.x; y[i] = p.y; vx[i] = p.vx; vy[i] = p.vy;
  }
}

int noalloc_fail(int code, const char* m) {
  g_noalloc_err = m;
  return code;
}

}  // namespace

extern "C" int edmd_run_noalloc(const edmd_system_desc* desc, double* x, double* y, double* vx,
                                double* vy, const double* rad, const double* m, int64_t max_coll,
                                double t_stop, int64_t* ncol_out, double* t_out, void* stream) {
  if (!desc || !x || !y || !vx || !vy || !rad || !m || max_coll < 0)
    return noalloc_fail(EDMD_ERR_ARG, "edmd_run_noalloc: null argument or negative max_coll");
  const edmd_system_desc& D = *desc;
  if (D.t_growstop > 0)
    return noalloc_fail(EDMD_ERR_ARG, "edmd_run_noalloc: growth starts are not supported");
  if (D.N < 2 || D.N > NOALLOC_MAX_N)
    return noalloc_fail(EDMD_ERR_CAPACITY, "edmd_run_noalloc: N must be in [2, 8192]");
  if (D.contact != EDMD_CONTACT_NONADDITIVE && D.contact != EDMD_CONTACT_ADDITIVE)
    return noalloc_fail(EDMD_ERR_ARG, "edmd_run_noalloc: bad contact rule");
  SysDev S;
  memset(&S, 0, sizeof(S));
  Box& B = S.B;
  B.N = D.N; B.Lx = D.Lx; B.Ly = D.Ly;
  B.additive = D.contact == EDMD_CONTACT_ADDITIVE;
  B.hLx = D.Lx / 2; B.hLy = D.Ly / 2;                      // boxConstantHelper 679-714
  B.Nyc = (int)(B.hLy); B.Nxc = (int)(B.hLx);
  if (!(D.Lx > 0) || !(D.Ly > 0) || B.Nxc < 1 || B.Nyc < 1)
    return noalloc_fail(EDMD_ERR_ARG, "edmd_run_noalloc: box smaller than one cell");
  if ((int64_t)B.Nxc * B.Nyc > NOALLOC_MAX_CELLS)
    return noalloc_fail(EDMD_ERR_CAPACITY, "edmd_run_noalloc: more than 65536 cells");
  B.cxs = D.Lx / B.Nxc; B.cys = D.Ly / B.Nyc;
  B.cxf = 1 / B.cxs; B.cyf = 1 / B.cys;
  B.dtP = 5.0 / (double)D.N;
  B.dtPN = B.dtP * D.N;
  S.rdtP = 1.0 / B.dtP;
  S.res = D.res; S.Einit = D.Einit; S.dtime = D.dtime; S.dtimeTh = D.dtime_thermo; S.tmax = D.tmax;
  S.L = D.N + NSPECIAL;
  int c = S.L;
  size_t nodes = 0;
  for (;;) {
    S.lev_off[S.nlev] = (int32_t)nodes; S.lev_cnt[S.nlev] = c; nodes += c; S.nlev++;
    if (c == 1) break;
    c = (c + 31) / 32;
  }
  // once per device, with that device current: the device address of the array
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return noalloc_fail(EDMD_ERR_CUDA, "edmd_run_noalloc: no current CUDA device");
  if (!g_noalloc_addr[dev]) {
    void* a = nullptr;
    cudaError_t ce = cudaGetSymbolAddress(&a, g_noalloc_scratch);
    if (ce != cudaSuccess || !a) return noalloc_fail(EDMD_ERR_CUDA, cudaGetErrorString(ce));
    g_noalloc_addr[dev] = (unsigned char*)a;
  }
  unsigned char* base = g_noalloc_addr[dev];
  size_t off = 0;
  auto take = [&](size_t bytes) { unsigned char* r = base + off; off += align_up(bytes, 256); return r; };
  size_t N = D.N, E = 2 * N + NSPECIAL, C = (size_t)B.Nxc * B.Nyc;
  SysDev* dsys = (SysDev*)take(sizeof(SysDev));
  int32_t* work = (int32_t*)take(sizeof(int32_t));
  S.st = (SysState*)take(sizeof(SysState));
  S.d = (Disk*)take(N * sizeof(Disk));
  S.vr = (double*)take(N * 8);
  S.cx = (int32_t*)take(N * 4); S.cy = (int32_t*)take(N * 4); S.prv = (int32_t*)take(N * 4);
  S.crossX = (int32_t*)take(N * 4); S.crossY = (int32_t*)take(N * 4);
  S.head = (int32_t*)take(C * 4);
  S.ev = (Ev*)take(E * sizeof(Ev));
  S.on = (int32_t*)take(E * 4); S.op = (int32_t*)take(E * 4);
  S.tree = (Node*)take(nodes * sizeof(Node));
  S.rows = (double*)take(64 * 9 * 8);
  S.rows_cap = 64;
  S.trace = nullptr; S.trace_cap = 0;
  if (off > NOALLOC_BYTES)
    return noalloc_fail(EDMD_ERR_CAPACITY, "edmd_run_noalloc: system does not fit the 4 MiB scratch array");
  cudaStream_t st = (cudaStream_t)stream;
  RunArgs A;
  // a finite event budget: NOALLOC_EVENTS_PER_COLL events per requested
  // collision plus NOALLOC_EVENTS_PER_DISK per disk (saturating), so that a
  // loop whose clock stops advancing ends with EDMD_ERR_BUDGET
  const int64_t cap = (int64_t)1 << 60;
  const int64_t per_coll = max_coll > cap / NOALLOC_EVENTS_PER_COLL ? cap : max_coll * NOALLOC_EVENTS_PER_COLL;
  const int64_t budget = std::min(cap, per_coll + (int64_t)N * NOALLOC_EVENTS_PER_DISK + NOALLOC_EVENTS_BASE);
  A.max_coll = max_coll; A.t_stop = t_stop; A.flags = 0; A.max_events = budget;
  A.nsys = 1; A.work = work; A.order = nullptr; A.cost = nullptr;
  k_noalloc_put<<<1, 1, 0, st>>>(S, dsys);
  k_noalloc_stage<<<1, 32, 0, st>>>(dsys, x, y, vx, vy, rad, m, D.first_screen, D.first_thermo);
  k_init_events<<<dim3((unsigned)((N + 1 + 127) / 128), 1), 128, 0, st>>>(dsys);
  k_init_finish<<<1, 256, 0, st>>>(dsys, 1);
  k_tree_build<<<1, 256, 0, st>>>(dsys, 1);
  if (cudaMemsetAsync(work, 0, sizeof(int32_t), st) != cudaSuccess)
    return noalloc_fail(EDMD_ERR_CUDA, "edmd_run_noalloc: memset failed");
  if (B.additive) k_run<32><<<1, 32 * WARPS_PER_BLOCK, 0, st>>>(dsys, A);
  else k_run<32, false><<<1, 32 * WARPS_PER_BLOCK, 0, st>>>(dsys, A);
  k_sync<<<1, 256, 0, st>>>(dsys, 1);
  k_noalloc_out<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(dsys, x, y, vx, vy);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return noalloc_fail(EDMD_ERR_CUDA, cudaGetErrorString(ce));
  SysState R;
  ce = cudaMemcpyAsync(&R, S.st, sizeof(R), cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) return noalloc_fail(EDMD_ERR_CUDA, cudaGetErrorString(ce));
  if (ncol_out) *ncol_out = (int64_t)R.ncol;
  if (t_out) *t_out = R.t;
  if (R.status == EDMD_ERR_ARG)
    return noalloc_fail(R.status, ("edmd_run_noalloc: position of disk " + std::to_string(R.err_a) +
                                   " outside the box").c_str());
  if (R.status == EDMD_ERR_OVERLAP)
    return noalloc_fail(R.status, ("edmd_run_noalloc: overlapping disks " + std::to_string(R.err_a) + " and " +
                                   std::to_string(R.err_b)).c_str());
  if (R.status == EDMD_ERR_BUDGET)
    return noalloc_fail(R.status, "edmd_run_noalloc: event budget exhausted (the state at the stop is written back)");
  if (R.status != EDMD_OK) return noalloc_fail(R.status, "edmd_run_noalloc: event loop stopped");
  g_noalloc_err.clear();
  return EDMD_OK;
}

extern "C" const char* edmd_last_error(const edmd_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_noalloc_err.c_str();
}
