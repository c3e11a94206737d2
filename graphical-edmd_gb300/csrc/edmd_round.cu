// edmd_round.cu -- round-parallel event engine: the causally independent events
// of one large system, or of a whole batch, processed at once, one warp or one
// thread per event.
//
// Every disk has one pending event: the earlier of its crossing event
// (crossingEventNormal, src/EDMD.c:2405) and its collision event
// (collisionEventNormal, src/EDMD.c:2829).  The event's footprint is the
// owner's cell plus the target cell (crossing) or the partner's cell at
// prediction time (collision; the partner stays in the owner's 3x3 block until
// the contact unless it collides first, which makes the event stale).
// Processing writes disks, lists and events of the owner's cell and the
// partner's current cell (a neighbour of the owner's), and reads the 3x3
// cells around them: everything lies within two cells of the owner's cell and
// the writes within one, so events whose footprints are more than three cells
// apart never touch the same data (window radius r >= 3).  Each round:
//   1. per cell, the minimum (time key, owner) of the events attributed to it
//      is kept up to date incrementally;
//   2. a tile kernel reduces those minima over square windows of radius r in
//      shared memory and selects every eligible event (before the system's
//      next screenshot, t_stop and its collision budget) that is the window
//      minimum at both of its footprint cells: no earlier pending event lies
//      within r cells, and selected events are more than r cells apart;
//   3. the selected events are processed, one warp each or (rounds of many
//      events) one thread each, with the arithmetic of the serial engines;
//   4. the cell minima around them are recomputed, and systems with nothing
//      left before their screenshot pass it (every disk free-flown to it).
// Events created inside a round can still precede a processed event (a chain
// of new events crossing r cells faster than the time gap).  That is detected,
// never silently accepted: each event carries the serial engine's pop clock
// at its processing (max of its time and its creator's clock), every cell
// keeps the largest clock of the events that wrote it (lw) and read it (lr),
// and an event that writes a cell with a later lw or lr, or reads one with a
// later lw, is counted as a causality violation.  With none, every disk sees
// the serial sequence of events, so the state is the reference's; only the
// summation order of the virial and the order of the trace differ.  Equal
// keys are ordered like the serial queue orders them: mutual equal-time
// predictions inherited from a serial engine carry the rank of their queue
// keys (k_rank) in the event id; a new event that ties with the inherited
// event of its partner for the same pair ranks by the serial key it would
// have been given (new_rank), other new ones rank after inherited ones; two
// valid mutual events give bit-identical velocities in either order since
// the collision rule is odd in (dx, dy) and in (dvx, dvy).
#include <cstdio>
#include <cstdint>
#include <cstring>
#include "edmd_ctx.h"

namespace {

constexpr uint64_t KINF = ~0ull;
constexpr int32_t IINF = 0x7fffffff;
constexpr int32_t GMASK = 0xffffff;   // disk index inside an event id (rank in the top byte)
constexpr unsigned FULLM = 0xffffffffu;
constexpr int TX = 16, TY = 32;       // selection tile (cells): 2.1 cells loaded per cell at radius 4;
                                      // measured against 32x16, 32x8 and 64x8 (best by ~1%)
constexpr int RTILE = 12;             // largest window radius of the tile kernel
constexpr int MAXDIRTY = 8;           // cells whose minimum one event can change
constexpr int MAXC = 8;               // candidates buffered per cell list per lane
constexpr int OB_CORRUPT = -2;        // overlap partner marker: a cell list longer than N (EDMD_ERR_BUDGET)
// tie ranks of collision events (the top byte of an event id, see event_id):
// inherited mutual pairs are 1 (pops first) and 2, events this engine makes
// are R_NEW, or R_FIRST when the serial queue would pop them before the
// inherited event of equal time they tie with (new_rank)
constexpr uint8_t R_FIRST = 0, R_NEW = 3;
constexpr int WPB = 1;                // warps per block of the processing kernel (measured best:
                                      // one-warp blocks, 20 per SM, 96 registers)
constexpr int NSTRIPE = 32;           // copies of each system's counters
// counters of the round engine, per system and stripe (u64 slots)
enum { C_CT0, C_CT1, C_CT2, C_CT3, C_NCOL, C_NCROSS, C_NSTALE, C_NPAIR, C_NPRED, C_NEV, C_NSCREEN, C_TLAST, NCNT };

struct RoundArgs {
  int32_t nsys;
  int32_t radius;
  int64_t TN;
  int32_t ntiles;
  uint32_t flags;
  uint64_t tstop_key;
  const int32_t* dsys;           // system of each disk
  const int64_t* doff;           // disk offset of each system
  const int64_t* coff;           // cell offset of each system
  uint64_t* dkey;                // time key of each disk's next event (KINF: none)
  int32_t* dpk;                  // its id: serial tie rank << 24 | disk
  uint8_t* drank;                // tie rank of each disk's collision event (R_FIRST .. R_NEW)
  uint32_t* ikb;                 // serial queue key (bucket, tie) of each disk's collision event
  uint64_t* iktie;               // as inherited from a serial engine (k_rank)
  int32_t* fc;                   // its two footprint cells (local), 2 per disk
  uint64_t* cmt; int32_t* cmi;   // attributed minimum (key, id) per cell
  uint64_t* lw; uint64_t* lr;    // causality stamps per cell
  int32_t* safe; int32_t* nsafe; // selected events of the round
  int32_t* nsafe_next;           // the next round's count (two alternate), emptied in this round
  int32_t* pnext;                // events taken past the first wave of the event kernel, emptied after the round
  int32_t* dcell;                // cells to recompute, MAXDIRTY per selected event
  int32_t* selflag;              // some event of the system was selected
  int32_t* active;               // systems still running after the round
  uint64_t* lim;                 // per-system bound on eligible keys for the round
  const uint64_t* target;        // per-system ncol at which the budget is met
  uint64_t* freeze;              // per-system key bound once the budget is met
  uint64_t* tlast;               // per-system largest screenshot key passed
  uint64_t* cnt;                 // [nsys][NSTRIPE][NCNT] counters of this call
  int32_t thr_min;               // rounds of at least this many events run one thread per event
  int32_t thread_kernel;         // k_process_thread is in this round's graph
  int32_t* maxsafe;              // largest selection count of the graph launch
  float4* shp;                   // FP32 shadow of each disk: cell-relative x, y and vx, vy
  float* sht;                    // ... and its time relative to the system's epoch
  double* epoch;                 // per-system time origin of the shadows (the call's start)
  const int32_t* tsys;           // tiles: system, first cell x, first cell y
  const int32_t* tx0;
  const int32_t* ty0;
  unsigned long long* violations;
};

__device__ __forceinline__ bool pair_less(uint64_t t1, int32_t i1, uint64_t t2, int32_t i2) {
  return t1 < t2 || (t1 == t2 && i1 < i2);
}

__device__ __forceinline__ uint64_t kmax(uint64_t a, uint64_t b) { return a > b ? a : b; }

// disk i's next event slot (the crossing wins an exact tie) and its key
__device__ __forceinline__ int next_slot(const SysDev& S, int i, uint64_t* key) {
  const int N = S.B.N;
  const Ev c = S.ev[i], k = S.ev[N + i];
  uint64_t kc = (c.st & 3u) ? time_key(c.t) : KINF;
  uint64_t kk = (k.st & 3u) ? time_key(k.t) : KINF;
  if (kk < kc) { *key = kk; return N + i; }
  *key = kc;
  return kc == KINF ? -1 : i;
}

__device__ __forceinline__ int cell_of(const Box& B, int cx, int cy) { return cy * B.Nxc + cx; }

// target cell of a crossing in direction dir (1..4) from (cx, cy)
__device__ __forceinline__ int target_cell(const Box& B, int cx, int cy, int dir) {
  switch (dir) {
    case 1: cx = cx - 1 < 0 ? B.Nxc - 1 : cx - 1; break;
    case 2: cx = cx + 1 >= B.Nxc ? 0 : cx + 1; break;
    case 3: cy = cy - 1 < 0 ? B.Nyc - 1 : cy - 1; break;
    default: cy = cy + 1 >= B.Nyc ? 0 : cy + 1; break;
  }
  return cell_of(B, cx, cy);
}

// cells a and b are equal or neighbours (periodic)
__device__ __forceinline__ bool adjacent(const Box& B, int a, int b) {
  int dx = a % B.Nxc - b % B.Nxc, dy = a / B.Nxc - b / B.Nxc;
  if (dx > 1) dx -= B.Nxc;
  if (dx < -1) dx += B.Nxc;
  if (dy > 1) dy -= B.Nyc;
  if (dy < -1) dy += B.Nyc;
  return dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1;
}

// next event key and footprint of disk i; the collision slot's `b` field holds
// the partner's cell at prediction time
__device__ __forceinline__ int attribution(const SysDev& S, int i, uint64_t* key, int* c1, int* c2) {
  const int slot = next_slot(S, i, key);
  const Box& B = S.B;
  const int cx = S.cx[i], cy = S.cy[i];
  *c1 = cell_of(B, cx, cy);
  if (slot < 0) *c2 = *c1;
  else if (slot >= B.N) *c2 = (int)S.ev[slot].b;
  else *c2 = target_cell(B, cx, cy, S.ev[slot].j);
  return slot;
}

// FP32 shadow of a disk record for the candidate screen: position relative to
// its cell's corner, velocity, time relative to the epoch.  Values outside the
// range the screen's error bound covers are stored as NaN, which no screen test
// passes, so those pairs always take the FP64 path.
// coordinate relative to the corner of cell c; a disk on the box edge of its
// cell can sit at the other side of the periodic box by rounding
__device__ __forceinline__ float cell_rel(double x, int c, double cs, double L) {
  double r = x - c * cs;
  if (r > cs + 1.0) r -= L;
  else if (r < -1.0) r += L;
  return (float)r;
}

__device__ __forceinline__ void shadow_write(const RoundArgs& A, int64_t g, const Box& B, const Disk& D, int cx,
                                             int cy, double epoch) {
  const float nan = __int_as_float(0x7fffffff);
  float xr = cell_rel(D.x, cx, B.cxs, B.Lx), yr = cell_rel(D.y, cy, B.cys, B.Ly);
  float vx = (float)D.vx, vy = (float)D.vy, tl = (float)(D.tl - epoch);
  const bool ok = xr > -1.0f && xr < (float)B.cxs + 1.0f && yr > -1.0f && yr < (float)B.cys + 1.0f &&
                  fabsf(vx) < 8.0f && fabsf(vy) < 8.0f && fabsf(tl) < 16.0f;
  A.shp[g] = ok ? make_float4(xr, yr, vx, vy) : make_float4(nan, nan, nan, nan);
  A.sht[g] = ok ? tl : nan;
}

// id of disk g's next event: a collision carries its serial tie rank
__device__ __forceinline__ int32_t event_id(const RoundArgs& A, int64_t g, int slot, int N) {
  return (slot >= N ? ((int32_t)A.drank[g] << 24) : 0) | (int32_t)g;
}

// ---------------------------------------------------------------- per call

// Exactly equal times of conflicting events are ordered like the serial queue
// orders them.  The only such ties the serial state carries in quantity are
// mutual predictions a->b, b->a made by one handler from the same positions
// (the initial predictions, and stopGrow, src/EDMD.c:4740-4800, whose coll++
// inside the loop leaves one of the two stale); their serial order is the
// order of their queue keys (b, tie).  Rank 1 or 2 orders such a pair, and
// the serial keys are kept for new_rank: a stale inherited event can tie with
// the valid new prediction its partner makes later for the same pair.
__global__ void k_rank(const SysDev* __restrict__ sys, RoundArgs A) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.TN) return;
  const int s = A.dsys[g];
  const SysDev& S = sys[s];
  const int N = S.B.N;
  const int i = (int)(g - A.doff[s]);
  const Ev e = S.ev[N + i];
  uint8_t rank = 1;
  if (e.st & 3u) {
    const Ev f = S.ev[N + e.j];
    if ((f.st & 3u) && f.j == i && __double_as_longlong(f.t) == __double_as_longlong(e.t))
      rank = (f.b < e.b || (f.b == e.b && f.tie < e.tie)) ? 2 : 1;
  }
  A.drank[g] = rank;
  A.ikb[g] = e.b;                      // k_prep overwrites b and tie next
  A.iktie[g] = e.tie;
}

// Serial order of a new collision event (time tn, inserted at the pop clock
// clk of the event that made it) against an inherited one of equal time with
// serial key (bx, tiex): true when the serial queue pops the new one first.
// The new event's key is what addEventToQueue (src/EDMD.c:2144) would give it:
// the calendar at the creator's pop is the bucket holding its clock, reached
// from the inherited calendar state (k, paulTime) by repeated addition of
// the bucket width as the serial loop does.  Same bucket: class 0 (re-added
// by a wrap) < 1 (bucket list, last pushed first) < 2 (direct insert, first
// inserted first); an event in the overflow list is re-added at the wrap, the
// last pushed first.
__device__ bool new_before_inherited(const SysDev& S, double tn, uint64_t clk, uint32_t bx, uint64_t tiex) {
  const Box& B = S.B;
  const SysState& R = *S.st;
  const double tc = key_time(clk);
  uint64_t k = R.k;
  double P = R.P;
  for (int guard = 0; guard < (1 << 24) && P + B.dtP <= tc; guard++) { P += B.dtP; k++; }
  const double dt = tn - P;
  const bool ovf_new = dt >= B.dtPN;
  if (bx == BINF) return ovf_new;
  if (ovf_new) return false;
  uint64_t by, cy;
  if (!(dt >= B.dtP)) { by = k; cy = 2; }
  else { by = k + (uint64_t)bucket_offset(dt, B.dtP, S.rdtP); cy = 1; }
  const uint64_t cx = tiex >> 62;
  if (by != (uint64_t)bx) return by < (uint64_t)bx;
  if (cy != cx) return cy < cx;
  return cy == 1;
}

// tie rank of the new collision event of disk d (time tn, partner p) made by
// an event of pop clock clk whose other disk is `other`: R_FIRST when it ties
// exactly with p's still inherited event for the mutual pair and the serial
// queue pops it first (a tie of a stale inherited event, such as stopGrow
// leaves, with a valid new one decides the trajectory), else R_NEW
__device__ __forceinline__ uint8_t new_rank(const SysDev& S, const RoundArgs& A, int64_t dbase, int d, int other,
                                            double tn, int p, uint64_t clk) {
  if (p == d || p == other) return R_NEW;
  const int64_t gp = dbase + p;
  const uint8_t rp = A.drank[gp];
  if (rp == R_NEW || rp == R_FIRST) return R_NEW;
  const Ev X = S.ev[S.B.N + p];
  if (!(X.st & 3u) || X.j != d || __double_as_longlong(X.t) != __double_as_longlong(tn)) return R_NEW;
  return new_before_inherited(S, tn, clk, A.ikb[gp], A.iktie[gp]) ? R_FIRST : R_NEW;
}

// serial pop clock and stored partner cell of every pending event, then the
// attribution of every disk
__global__ void k_prep(const SysDev* __restrict__ sys, RoundArgs A) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.TN) return;
  const int s = A.dsys[g];
  const SysDev& S = sys[s];
  const Box& B = S.B;
  const int N = B.N;
  const int i = (int)(g - A.doff[s]);
  const uint64_t clock = time_key(S.st->t);
  for (int k = 0; k < 2; k++) {
    Ev& e = S.ev[k * N + i];
    if (!(e.st & 3u)) continue;
    e.tie = kmax(time_key(e.t), clock);
    if (k == 1) {
      const int own = cell_of(B, S.cx[i], S.cy[i]);
      const int p = e.j;
      const int pc = cell_of(B, S.cx[p], S.cy[p]);
      e.b = (uint32_t)(adjacent(B, own, pc) ? pc : own);
    }
  }
  const double ep = S.st->t;
  if (i == 0) A.epoch[s] = ep;
  shadow_write(A, g, B, S.d[i], S.cx[i], S.cy[i], ep);
  uint64_t key;
  int c1, c2;
  const int slot = attribution(S, i, &key, &c1, &c2);
  A.dkey[g] = key;
  A.dpk[g] = event_id(A, g, slot, N);
  A.fc[2 * g] = c1;
  A.fc[2 * g + 1] = c2;
  if (key != KINF) {
    atomicMin((unsigned long long*)&A.cmt[A.coff[s] + c1], (unsigned long long)key);
    if (c2 != c1) atomicMin((unsigned long long*)&A.cmt[A.coff[s] + c2], (unsigned long long)key);
  }
}

__global__ void k_prep_owner(RoundArgs A) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.TN) return;
  const uint64_t key = A.dkey[g];
  if (key == KINF) return;
  const int64_t base = A.coff[A.dsys[g]];
  const int64_t a = base + A.fc[2 * g], b = base + A.fc[2 * g + 1];
  const int32_t id = A.dpk[g];
  if (A.cmt[a] == key) atomicMin(&A.cmi[a], id);
  if (b != a && A.cmt[b] == key) atomicMin(&A.cmi[b], id);
}

// eligibility bound of every system for the next round
__device__ __forceinline__ uint64_t system_limit(const SysDev& S, const RoundArgs& A, int s) {
  if (S.st->status != EDMD_OK) return 0;
  uint64_t lim = time_key(S.ev[2 * S.B.N + SP_SCREEN].t);
  if (A.tstop_key < lim) lim = A.tstop_key;
  if (A.freeze[s] < lim) lim = A.freeze[s];
  return lim;
}

__global__ void k_limits(const SysDev* __restrict__ sys, RoundArgs A) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < A.nsys) A.lim[s] = system_limit(sys[s], A, s);
}

// ---------------------------------------------------------------- per round


__device__ __forceinline__ int wrapi(int v, int n) {
  if (v >= 0 && v < n) return v;          // inside: the common case, no division
  if (v < 0 && v + n >= 0) return v + n;  // one period off (tiles of systems wider than a tile)
  if (v >= n && v - n < n) return v - n;
  v %= n;
  return v < 0 ? v + n : v;
}

// (time key, event id) as one 96-bit value in a 128-bit word: the unsigned
// order of the word is the lexicographic order pair_less uses (ids are
// non-negative), so a window minimum is one compare-and-select per element
typedef unsigned __int128 kid_t;
__device__ __forceinline__ kid_t kid(uint64_t k, int32_t id) { return ((kid_t)k << 32) | (uint32_t)id; }
__device__ __forceinline__ kid_t kid_min(kid_t a, kid_t b) { return b < a ? b : a; }

// Window minima of S consecutive positions: out[k] = min(a[k .. k+W-1]).
// The W-S+1 middle elements are common to all S windows; each window adds a
// suffix of the left part and a prefix of the right part (a van Herk /
// Gil-Werman block): W + 2S - 4 compares instead of S (W - 1).
template <int S, int W>
__device__ __forceinline__ void block_window_min(const kid_t (&a)[S + W - 1], kid_t (&out)[S]) {
  static_assert(W >= S, "window narrower than the block");
  kid_t c = a[S - 1];
#pragma unroll
  for (int j = S; j < W; j++) c = kid_min(c, a[j]);
  if constexpr (S == 1) {
    out[0] = c;
    return;
  }
  kid_t rp[S];
  rp[0] = c;
#pragma unroll
  for (int k = 1; k < S; k++) rp[k] = kid_min(rp[k - 1], a[W + k - 1]);
  out[S - 1] = rp[S - 1];
  if constexpr (S > 1) {
    kid_t ls = a[S - 2];
#pragma unroll
    for (int k = S - 2; k >= 0; k--) {
      if (k < S - 2) ls = kid_min(ls, a[k]);
      out[k] = kid_min(ls, rp[k]);
    }
  }
}

// tile geometry of the selection for window radius R: cell minima with a
// halo, horizontal minima of rows, window minima (padded so that every block
// of SB outputs reads in range; the padding's outputs are never used)
template <int R>
struct SelGeom {
  // two outputs per thread: measured best of 1, 2 and 4 (fewer compares per
  // output against idle threads at the tile's barriers)
  static constexpr int H = R + 1, W = 2 * R + 1, SB = 2;
  static constexpr int HW = TX + 2;                    // outputs per row: columns -1..TX
  static constexpr int NHB = (HW + SB - 1) / SB;
  static constexpr int CW = NHB * SB + W - 1;          // input columns
  static constexpr int VR = TY + 2;                    // outputs per column: rows -1..TY
  static constexpr int NVB = (VR + SB - 1) / SB;
  static constexpr int CH = NVB * SB + W - 1;          // rows of cell and horizontal minima
  static constexpr size_t bytes = (size_t)(CH * CW + CH * HW + NVB * SB * HW) * sizeof(kid_t);
};

// Window minima of one tile in shared memory and selection of its events;
// the window radius R is a compile-time constant (3..12).
template <int R>
__global__ void __launch_bounds__(TX * TY, 4) k_select(const SysDev* __restrict__ sys, RoundArgs A) {
  using G = SelGeom<R>;
  constexpr int H = G::H, W = G::W, SB = G::SB, HW = G::HW, CW = G::CW, CH = G::CH;
  extern __shared__ kid_t sel_smem[];
  // the round's count of running systems is rebuilt by k_barrier
  if (blockIdx.x == 0 && threadIdx.x == 0) *A.active = 0;
  kid_t* ck = sel_smem;                // CH x CW
  kid_t* hk = ck + CH * CW;            // CH x HW
  kid_t* wk = hk + CH * HW;            // NVB*SB x HW
  for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
  const int s = A.tsys[t];
  const uint64_t lim = A.lim[s];
  if (lim == 0) continue;             // the system has stopped: nothing to select
  const Box& B = sys[s].B;
  const int Nxc = B.Nxc, Nyc = B.Nyc;
  const int x0 = A.tx0[t], y0 = A.ty0[t];
  const int64_t base = A.coff[s];
  if (x0 >= H && x0 - H + CW <= Nxc && y0 >= H && y0 - H + CH <= Nyc) {
    // a tile away from the periodic edges: no wrap
    const int64_t c0 = base + (int64_t)(y0 - H) * Nxc + (x0 - H);
    for (int q = threadIdx.x; q < CW * CH; q += blockDim.x) {
      const int lx = q % CW, ly = q / CW;
      const int64_t c = c0 + (int64_t)ly * Nxc + lx;
      ck[q] = kid(A.cmt[c], A.cmi[c]);
    }
  } else {
    for (int q = threadIdx.x; q < CW * CH; q += blockDim.x) {
      const int lx = q % CW, ly = q / CW;
      const int gx = wrapi(x0 + lx - H, Nxc), gy = wrapi(y0 + ly - H, Nyc);
      const int64_t c = base + (int64_t)gy * Nxc + gx;
      ck[q] = kid(A.cmt[c], A.cmi[c]);
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < CH * G::NHB; q += blockDim.x) {
    const int ly = q / G::NHB, hx0 = (q % G::NHB) * SB;
    kid_t a[SB + W - 1], o[SB];
#pragma unroll
    for (int j = 0; j < SB + W - 1; j++) a[j] = ck[ly * CW + hx0 + j];
    block_window_min<SB, W>(a, o);
#pragma unroll
    for (int k = 0; k < SB; k++)
      if (hx0 + k < HW) hk[ly * HW + hx0 + k] = o[k];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < HW * G::NVB; q += blockDim.x) {
    const int wx = q % HW, wy0 = (q / HW) * SB;
    kid_t a[SB + W - 1], o[SB];
#pragma unroll
    for (int j = 0; j < SB + W - 1; j++) a[j] = hk[(wy0 + j) * HW + wx];
    block_window_min<SB, W>(a, o);
#pragma unroll
    for (int k = 0; k < SB; k++) wk[(wy0 + k) * HW + wx] = o[k];
  }
  __syncthreads();
  const int ix = threadIdx.x % TX, iy = threadIdx.x / TX;
  const int cx = x0 + ix, cy = y0 + iy;
  bool sel = false;
  int32_t g = 0;
  if (cx < Nxc && cy < Nyc) {
    const kid_t v = ck[(iy + H) * CW + ix + H];
    const uint64_t k = (uint64_t)(v >> 32);
    const int32_t id = (int32_t)(uint32_t)v;
    g = id & GMASK;
    const int w = (iy + 1) * HW + ix + 1;
    if (k < lim && wk[w] == v) {
      const int c = cy * Nxc + cx;
      if (A.fc[2 * (int64_t)g] == c) {
        const int c2 = A.fc[2 * (int64_t)g + 1];
        if (c2 == c) {
          sel = true;
        } else {
          int dx = c2 % Nxc - cx, dy = c2 / Nxc - cy;
          if (dx > 1) dx -= Nxc;
          if (dx < -1) dx += Nxc;
          if (dy > 1) dy -= Nyc;
          if (dy < -1) dy += Nyc;
          if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1) sel = wk[(iy + 1 + dy) * HW + ix + 1 + dx] == v;
        }
      }
    }
  }
  const unsigned m = __ballot_sync(FULLM, sel);
  if (m) {
    const int lane = threadIdx.x & 31;
    const int lead = __ffs(m) - 1;
    int pos = 0;
    if (lane == lead) pos = atomicAdd(A.nsafe, __popc(m));
    pos = __shfl_sync(FULLM, pos, lead);
    if (sel) A.safe[pos + __popc(m & ((1u << lane) - 1))] = g;
    if (lane == lead) A.selflag[s] = 1;
  }
  __syncthreads();
  }
}

// causality stamp of a write of local cell c
__device__ bool stamp_write(const RoundArgs& A, int64_t base, int c, uint64_t clk) {
  const int64_t gc = base + c;
  const bool bad = A.lw[gc] > clk || A.lr[gc] > clk;
  atomicMax((unsigned long long*)&A.lw[gc], (unsigned long long)clk);
  return bad;
}

// collisionEventNormal (src/EDMD.c:2829-2905) for disks a0 and a1 (a1 may be
// -1), each current at time t, by one warp: lanes 0..8 walk a0's 3x3 cells and
// lanes 16..24 a1's (dy outer, dx inner), the candidates are packed over the
// warp and each lane solves a share of the pairs; the result is the first
// strict minimum below NEVER in the reference's scan order (lexicographic
// (time, scan position)); with none the partner stays 0 and collActual is
// disk 0's counter.
struct Pred {
  double dt;
  int partner;
  uint32_t ca;
  int pcell;     // partner's cell, or the owner's when there is none
};
struct WarpScratch {
  int32_t reg[32 * MAXC];
  int32_t comp[2 * 9 * MAXC];
  int16_t ord[2 * 9 * MAXC];
};

__device__ __forceinline__ void merge(double& bd, uint64_t& bk, int& bo, int& bp, uint32_t& bc,
                                      double d, uint64_t kd, int o, int p, uint32_t c) {
  if (kd < bk || (kd == bk && o < bo)) { bd = d; bk = kd; bo = o; bp = p; bc = c; }
}

__device__ void predict_warp(const SysDev& S, int a0, const Disk& A0, int X0, int Y0, int a1,
                             const Disk& A1, int X1, int Y1, double t, Pred& r0, Pred& r1,
                             WarpScratch* W, int lane, unsigned long long* npair, bool* ovl, int* oa,
                             int* ob) {
  const Box& B = S.B;
  const int grp = lane >> 4, q = lane & 15;
  const int a = grp ? a1 : a0;
  const int X = grp ? X1 : X0, Y = grp ? Y1 : Y0;
  int cnt = 0;
  bool lcorrupt = false;
  int32_t* reg = W->reg + lane * MAXC;
  if (a >= 0 && q < 9) {
    int p = S.head[pbc_cy(B, Y + q / 3 - 1) * B.Nxc + pbc_cx(B, X + q % 3 - 1)];
    int guard = 0;                   // a list is never longer than N
    while (p != NIL && guard++ < B.N) {
      if (p != a) {
        if (cnt < MAXC) reg[cnt] = p;
        cnt++;
      }
      p = S.d[p].nxt;
    }
    if (p != NIL) { lcorrupt = true; }   // a list longer than N is corrupt
  }
  const bool spill = __any_sync(FULLM, cnt > MAXC);
  const uint64_t knever = time_key(NEVER);
  double bd0 = NEVER, bd1 = NEVER;
  uint64_t bk0 = knever, bk1 = knever;
  int bo0 = -1, bo1 = -1, bp0 = 0, bp1 = 0;
  uint32_t bc0 = 0, bc1 = 0;
  bool lovl = false;
  int la = -1, lb = -1;               // the predicting disk and the partner that overlaps it
  unsigned long long tot;
  if (!spill) {
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
      const int v = __shfl_up_sync(FULLM, incl, o, 16);
      if (q >= o) incl += v;
    }
    const int excl = incl - cnt;
    const int tot0 = __shfl_sync(FULLM, incl, 15), tot1 = __shfl_sync(FULLM, incl, 31);
    const int bse = grp ? tot0 : 0;
    for (int k = 0; k < cnt; k++) {
      W->comp[bse + excl + k] = reg[k];
      W->ord[bse + excl + k] = (int16_t)(q * MAXC + k);
    }
    __syncwarp();
    tot = (unsigned long long)(tot0 + tot1);
    for (int f = lane; f < tot0 + tot1; f += 32) {
      const int p = W->comp[f];
      const int o = W->ord[f];
      const Disk P = S.d[p];
      const bool g1 = f >= tot0;
      bool ov = false;
      const double d = coll_time_normal_i(B, g1 ? A1 : A0, P, t, &ov);
      if (ov) { lovl = true; la = g1 ? a1 : a0; lb = p; }
      const uint64_t kd = time_key(d);
      if (g1) merge(bd1, bk1, bo1, bp1, bc1, d, kd, o, p, P.coll);
      else merge(bd0, bk0, bo0, bp0, bc0, d, kd, o, p, P.coll);
    }
    __syncwarp();
  } else {
    // a list longer than MAXC: every lane walks and solves its own list
    unsigned long long mine = 0;
    if (a >= 0 && q < 9) {
      const Disk& AA = grp ? A1 : A0;
      int p = S.head[pbc_cy(B, Y + q / 3 - 1) * B.Nxc + pbc_cx(B, X + q % 3 - 1)];
      int k = 0, guard = 0;
      while (p != NIL && guard++ < B.N) {
        const Disk P = S.d[p];
        if (p != a) {
          bool ov = false;
          const double d = coll_time_normal_i(B, AA, P, t, &ov);
          if (ov) { lovl = true; la = a; lb = p; }
          const uint64_t kd = time_key(d);
          if (grp) merge(bd1, bk1, bo1, bp1, bc1, d, kd, q * (1 << 20) + k, p, P.coll);
          else merge(bd0, bk0, bo0, bp0, bc0, d, kd, q * (1 << 20) + k, p, P.coll);
          k++;
          mine++;
        }
        p = P.nxt;
      }
      if (p != NIL) lcorrupt = true;
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(FULLM, mine, o);
    tot = mine;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double d = __shfl_xor_sync(FULLM, bd0, o);
    uint64_t kd = __shfl_xor_sync(FULLM, bk0, o);
    int oo = __shfl_xor_sync(FULLM, bo0, o), pp = __shfl_xor_sync(FULLM, bp0, o);
    uint32_t cc = __shfl_xor_sync(FULLM, bc0, o);
    merge(bd0, bk0, bo0, bp0, bc0, d, kd, oo, pp, cc);
    d = __shfl_xor_sync(FULLM, bd1, o);
    kd = __shfl_xor_sync(FULLM, bk1, o);
    oo = __shfl_xor_sync(FULLM, bo1, o);
    pp = __shfl_xor_sync(FULLM, bp1, o);
    cc = __shfl_xor_sync(FULLM, bc1, o);
    merge(bd1, bk1, bo1, bp1, bc1, d, kd, oo, pp, cc);
  }
  const int div = spill ? (1 << 20) : MAXC;
  r0.dt = bd0; r0.partner = bp0; r0.ca = bo0 < 0 ? S.d[0].coll : bc0;
  {
    const int qq = bo0 < 0 ? 4 : bo0 / div;
    r0.pcell = pbc_cy(B, Y0 + qq / 3 - 1) * B.Nxc + pbc_cx(B, X0 + qq % 3 - 1);
  }
  if (a1 >= 0) {
    r1.dt = bd1; r1.partner = bp1; r1.ca = bo1 < 0 ? S.d[0].coll : bc1;
    const int qq = bo1 < 0 ? 4 : bo1 / div;
    r1.pcell = pbc_cy(B, Y1 + qq / 3 - 1) * B.Nxc + pbc_cx(B, X1 + qq % 3 - 1);
  }
  *npair += tot;
  const unsigned m = __ballot_sync(FULLM, lovl);
  if (m) {
    *ovl = true;
    *oa = __shfl_sync(FULLM, la, __ffs(m) - 1);
    *ob = __shfl_sync(FULLM, lb, __ffs(m) - 1);
  }
  if (__any_sync(FULLM, lcorrupt)) { *ovl = true; *oa = a0; *ob = OB_CORRUPT; }
}

__device__ __forceinline__ void set_event(const SysDev& S, int slot, double t, int j, uint32_t ca,
                                          uint32_t pcell, uint64_t clock) {
  Ev e;
  e.t = t; e.tie = kmax(time_key(t), clock); e.b = pcell; e.j = j; e.ca = ca; e.st = ST_QUEUED;
  S.ev[slot] = e;
}

// new attribution of disk i (global index g); its cells join the dirty list
__device__ __forceinline__ void reattribute(const SysDev& S, const RoundArgs& A, int i, int64_t g,
                                            int64_t base, int32_t* dc, int* nd) {
  uint64_t key;
  int c1, c2;
  const int slot = attribution(S, i, &key, &c1, &c2);
  A.dkey[g] = key;
  A.dpk[g] = event_id(A, g, slot, S.B.N);
  A.fc[2 * g] = c1;
  A.fc[2 * g + 1] = c2;
  dc[(*nd)++] = (int32_t)(base + c1);
  if (c2 != c1) dc[(*nd)++] = (int32_t)(base + c2);
}

// read stamps of the 3x3 cells around c by lanes l0..l0+8 (warp-wide result)
__device__ __forceinline__ bool stamp_read_warp(const Box& B, const RoundArgs& A, int64_t base, int c,
                                                uint64_t clk, int lane, int l0) {
  bool bad = false;
  const int q = lane - l0;
  if (q >= 0 && q < 9) {
    const int x = c % B.Nxc, y = c / B.Nxc;
    const int64_t gc = base + pbc_cy(B, y + q / 3 - 1) * B.Nxc + pbc_cx(B, x + q % 3 - 1);
    if (A.lw[gc] > clk) bad = true;
    if (A.lr[gc] < clk) atomicMax((unsigned long long*)&A.lr[gc], (unsigned long long)clk);
  }
  return __any_sync(FULLM, bad);
}

__device__ __forceinline__ void cnt_add(const RoundArgs& A, int s, int stripe, int k, unsigned long long v) {
  if (v) atomicAdd((unsigned long long*)&A.cnt[((int64_t)s * NSTRIPE + stripe) * NCNT + k], v);
}
__device__ __forceinline__ void cnt_addf(const RoundArgs& A, int s, int stripe, int k, double v) {
  atomicAdd((double*)&A.cnt[((int64_t)s * NSTRIPE + stripe) * NCNT + k], v);
}

__device__ __forceinline__ Disk shfl_disk(const Disk& v, int src) {
  Disk r;
  r.x = __shfl_sync(FULLM, v.x, src);
  r.y = __shfl_sync(FULLM, v.y, src);
  r.vx = __shfl_sync(FULLM, v.vx, src);
  r.vy = __shfl_sync(FULLM, v.vy, src);
  r.tl = __shfl_sync(FULLM, v.tl, src);
  r.rad = __shfl_sync(FULLM, v.rad, src);
  r.m = __shfl_sync(FULLM, v.m, src);
  r.nxt = __shfl_sync(FULLM, v.nxt, src);
  r.coll = __shfl_sync(FULLM, v.coll, src);
  return r;
}

// outcome of one processed event (lane 0 holds everything but `ct`, which
// lane q < 4 holds for virial term q)
struct EvResult {
  int32_t dc[MAXDIRTY];              // cells whose minimum can have changed
  int nd;
  unsigned long long npair, npred, ncol, ncross, nstale, nscreen;
  double ct;
  uint64_t key;
  bool bad, ovl;
  int a, ob;
};

// one selected event g of system s processed by one warp: doTheCollisionNormal
// (src/EDMD.c:3542, elastic rule 3802-3827), its stale branch (3553-3556) or
// doTheCrossing (2501).  The scalar work is repeated by every lane (same
// values), stores are made by lane 0, predictions are shared by the warp.
__device__ void process_event_warp(const SysDev& S, const RoundArgs& A, int s, int64_t g, WarpScratch* W,
                                   int lane, EvResult& res) {
    const Box& B = S.B;
    const int N = B.N;
    const int64_t base = A.coff[s], dbase = A.doff[s];
    const int a = (int)(g - dbase);
    uint64_t key;
    const int slot = next_slot(S, a, &key);
    const Ev E = S.ev[slot];
    const double t = E.t;
    const uint64_t clk = E.tie;        // serial pop clock of this event
    int32_t dc[MAXDIRTY];
    int nd = 0;
    dc[nd++] = (int32_t)(base + A.fc[2 * g]);
    if (A.fc[2 * g + 1] != A.fc[2 * g]) dc[nd++] = (int32_t)(base + A.fc[2 * g + 1]);
    Disk Da = S.d[a];
    const int ax = S.cx[a], ay = S.cy[a];
    const int ca = cell_of(B, ax, ay);
    unsigned long long npair = 0, npred = 0, ncol = 0, ncross = 0, nstale = 0;
    double ct[1] = {0};
    bool ovl = false, bad = false;
    int ob = -1;
    // what the shared tail does, set by the handler: the second disk of a
    // collision, the cells of the disks, the cells stamped as written and
    // the centres of the 3x3 blocks stamped as read, new crossing events
    int b = -1;
    int64_t gb = -1;
    int pax = ax, pay = ay, pbx = ax, pby = ay;
    int wc1 = -1, rc0 = ca, rc1 = -1;
    bool cross = false;
    Disk Db = Da;
    if (slot >= N) {
      Db = S.d[E.j];
      if (E.ca != Db.coll) {
        free_fly_i(B, Da, t);
        __syncwarp();
        if (lane == 0) {
          S.d[a] = Da;
          shadow_write(A, g, B, Da, ax, ay, A.epoch[s]);
        }
        nstale = 1;
      } else {
        b = E.j;
        gb = dbase + b;
        dc[nd++] = (int32_t)(base + A.fc[2 * gb]);
        if (A.fc[2 * gb + 1] != A.fc[2 * gb]) dc[nd++] = (int32_t)(base + A.fc[2 * gb + 1]);
        const int bx = S.cx[b], by = S.cy[b];
        const int cb = cell_of(B, bx, by);
        // even lanes advance a, odd lanes b: the per-disk FP64 work of the
        // two disks shares its instructions
        const bool odd = lane & 1;
        Disk M = odd ? Db : Da;
        free_fly_i(B, M, t);
        M.coll++;
        Da = shfl_disk(M, 0);
        Db = shfl_disk(M, 1);
        double dx = Db.x - Da.x, dy = Db.y - Da.y;
        const double dvx = Db.vx - Da.vx, dvy = Db.vy - Da.vy;
        const double msum = Da.m + Db.m;
        const double invMass = __double_as_longlong(msum) == 0x4000000000000000ll ? 0.5 : 1 / msum;
        pbc_i(B, dx, dy);
        const double collKernel = invMass * (1 + S.res) * (dx * dvx + dy * dvy);
        const double distSquared = contact2(B, Da.rad, Db.rad);
        const double f = __double_as_longlong(distSquared) == 0x4010000000000000ll
            ? collKernel * 0.25 : collKernel / distSquared;
        const double cf = Da.m * Db.m * f;
        // virial term q on lane q: collTermX, Y, XY, YX
        {
          const double u = (lane == 1 || lane == 3) ? dy : dx;
          const double w = (lane == 0 || lane == 3) ? dx : dy;
          ct[0] = cf * u * w;
        }
        // v - x as v + (-x) (the same rounding): no divergent branch
        {
          const double fm = f * (odd ? Da.m : Db.m);
          M.vx = M.vx + flip(fm * dx, odd);
          M.vy = M.vy + flip(fm * dy, odd);
        }
        Da.vx = __shfl_sync(FULLM, M.vx, 0);
        Da.vy = __shfl_sync(FULLM, M.vy, 0);
        Db.vx = __shfl_sync(FULLM, M.vx, 1);
        Db.vy = __shfl_sync(FULLM, M.vy, 1);
        __syncwarp();
        if (lane == 0) {
          S.d[a] = Da;
          S.d[b] = Db;
          shadow_write(A, g, B, Da, ax, ay, A.epoch[s]);
          shadow_write(A, gb, B, Db, bx, by, A.epoch[s]);
          if ((A.flags & EDMD_F_TRACE) && S.trace) {
            const unsigned long long k = atomicAdd((unsigned long long*)&S.st->ntrace, 1ull);
            if ((int64_t)k < S.trace_cap) {
              edmd_collision* tr = (edmd_collision*)S.trace + k;
              tr->i = a; tr->j = b; tr->cell_i = ca; tr->cell_j = cb; tr->t = t;
            }
          }
        }
        pbx = bx; pby = by;
        wc1 = cb; rc1 = cb;
        cross = true;
        ncol = 1;
      }
    } else {
      free_fly_i(B, Da, t);
      int cx = ax, cy = ay;
      int wrapx = 0, wrapy = 0;
      switch (E.j) {
        case 1: if (cx - 1 == -1) { cx = B.Nxc - 1; wrapx = -1; } else cx -= 1; break;
        case 2: if (cx + 1 == B.Nxc) { cx = 0; wrapx = 1; } else cx += 1; break;
        case 3: if (cy - 1 == -1) { cy = B.Nyc - 1; wrapy = -1; } else cy -= 1; break;
        default: if (cy + 1 == B.Nyc) { cy = 0; wrapy = 1; } else cy += 1; break;
      }
      const int c = cell_of(B, cx, cy);
      __syncwarp();
      if (lane == 0) {
        // unlink from the old cell, relink at the head of the new one
        const int pv = S.prv[a], nx = Da.nxt;
        if (pv == NIL) S.head[ca] = nx;
        else S.d[pv].nxt = nx;
        if (nx != NIL) S.prv[nx] = pv;
        if (wrapx) S.crossX[a] += wrapx;
        if (wrapy) S.crossY[a] += wrapy;
        const int h = S.head[c];
        S.cx[a] = cx;
        S.cy[a] = cy;
        S.prv[a] = NIL;
        Da.nxt = h;
        S.d[a] = Da;
        shadow_write(A, g, B, Da, cx, cy, A.epoch[s]);
        S.head[c] = a;
        if (h != NIL) S.prv[h] = a;
      }
      pax = cx; pay = cy;
      wc1 = c; rc0 = c;
      cross = true;
      ncross = 1;
    }
    // ---- the tail shared by the three handlers: causality stamps, new
    // crossing events (a on even lanes, b on odd ones), new collision events
    // (collisionEvent for a, then b), the event records and attribution
    bad |= lane == 0 && (stamp_write(A, base, ca, clk) | (wc1 >= 0 && stamp_write(A, base, wc1, clk)));
    bad |= stamp_read_warp(B, A, base, rc0, clk, lane, 0);
    if (rc1 >= 0) bad |= stamp_read_warp(B, A, base, rc1, clk, lane, 16);
    __syncwarp();
    double ctc = 0;
    int cdir = 0;
    if (cross) {
      const bool od = (lane & 1) && b >= 0;
      ctc = crossing_time_lanes(B, od ? Db : Da, od ? pbx : pax, od ? pby : pay, t, lane, 2, &cdir);
    }
    Pred p0, p1;
    int oa = a;
    predict_warp(S, a, Da, pax, pay, b, Db, pbx, pby, t, p0, p1, W, lane, &npair, &ovl, &oa, &ob);
    npred = b >= 0 ? 2 : 1;
    const double tca = __shfl_sync(FULLM, ctc, 0), tcb = __shfl_sync(FULLM, ctc, 1);
    const int dira = __shfl_sync(FULLM, cdir, 0), dirb = __shfl_sync(FULLM, cdir, 1);
    if (lane == 0) {
      if (cross) set_event(S, a, tca, dira, 0, 0, clk);
      if (b >= 0) set_event(S, b, tcb, dirb, 0, 0, clk);
      const uint8_t rka = new_rank(S, A, dbase, a, b, t + p0.dt, p0.partner, clk);
      const uint8_t rkb = b >= 0 ? new_rank(S, A, dbase, b, a, t + p1.dt, p1.partner, clk) : R_NEW;
      set_event(S, N + a, t + p0.dt, p0.partner, p0.ca, p0.pcell, clk);
      if (b >= 0) set_event(S, N + b, t + p1.dt, p1.partner, p1.ca, p1.pcell, clk);
      A.drank[g] = rka;
      if (b >= 0) A.drank[gb] = rkb;
      reattribute(S, A, a, g, base, dc, &nd);
      if (b >= 0) reattribute(S, A, b, gb, base, dc, &nd);
    }
    for (int k = 0; k < MAXDIRTY; k++) res.dc[k] = dc[k];
    res.nd = nd;
    res.npair = npair; res.npred = npred; res.ncol = ncol; res.ncross = ncross; res.nstale = nstale;
    res.nscreen = 0;
    res.ct = ct[0];
    res.key = key;
    res.bad = bad; res.ovl = ovl;
    res.a = oa; res.ob = ob;
}

// ---- one thread per event (rounds with many selected events): the lanes of
// a warp run 32 different events, so their scalar FP64 work shares issue slots

// collisionEventNormal (src/EDMD.c:2829-2905) by one thread: the 3x3 cells dy
// outer, dx inner, each list in order, first strict minimum below NEVER
__device__ Pred predict_thread(const SysDev& S, const RoundArgs& A, int s, int a, const Disk& Da, int X, int Y,
                               double t, unsigned long long* npair, unsigned long long* nscreen, bool* ovl,
                               int* ob) {
  const Box& B = S.B;
  Pred r;
  r.dt = NEVER;
  r.partner = 0;
  r.ca = 0;
  r.pcell = cell_of(B, X, Y);
  uint64_t kb = time_key(NEVER);
  bool found = false;
  // FP32 screen: the owner in its cell's frame at time t.  The bound on the
  // FP32 error of b = dr.dv (|positions| < cell + 1, |v| < 8, |times - epoch|
  // < 16: at most ~7e-4) is below SCREEN_B, so b32 > SCREEN_B proves the FP64
  // b > 0: collisionTimeNormal returns "never" there before any other test.
  constexpr float SCREEN_B = 2e-3f;
  const double dt0 = t - A.epoch[s];
  // with at least 5 cells a side the neighbour cell offset gives the minimum image
  const bool screen = (A.flags & EDMD_F_SCREEN) && dt0 > -16.0 && dt0 < 16.0 && B.Nxc >= 5 && B.Nyc >= 5;
  const float t32 = (float)dt0;
  const float axr = cell_rel(Da.x, X, B.cxs, B.Lx), ayr = cell_rel(Da.y, Y, B.cys, B.Ly);
  const bool own_ok = axr > -1.0f && axr < (float)B.cxs + 1.0f && ayr > -1.0f && ayr < (float)B.cys + 1.0f &&
                      fabs(Da.vx) < 8.0 && fabs(Da.vy) < 8.0;
  const float avx = (float)Da.vx, avy = (float)Da.vy;
  const float cxs = (float)B.cxs, cys = (float)B.cys;
  const int64_t dbase = A.doff[s];
  int guard = 0;                     // a list is never longer than N
  for (int q = 0; q < 9; q++) {
    const int ox = q % 3 - 1, oy = q / 3 - 1;
    const int cell = pbc_cy(B, Y + oy) * B.Nxc + pbc_cx(B, X + ox);
    int p = S.head[cell];
    while (p != NIL && guard++ < 9 * B.N) {
      if (p == a) {
        p = S.d[p].nxt;
        continue;
      }
      (*npair)++;
      if (screen && own_ok) {
        const float4 P = A.shp[dbase + p];
        const float lat = t32 - A.sht[dbase + p];
        const float dx = (P.x + lat * P.z) + ox * cxs - axr;
        const float dy = (P.y + lat * P.w) + oy * cys - ayr;
        const float b = dx * (P.z - avx) + dy * (P.w - avy);
        if (b > SCREEN_B) {          // separating: FP64 would return NEVER
          (*nscreen)++;
          p = S.d[p].nxt;
          continue;
        }
      }
      const Disk P = S.d[p];
      bool ov = false;
      const double d = coll_time_normal_i(B, Da, P, t, &ov);
      if (ov) { *ovl = true; *ob = p; }
      const uint64_t kd = time_key(d);
      if (kd < kb) { r.dt = d; kb = kd; r.partner = p; r.ca = P.coll; r.pcell = cell; found = true; }
      p = P.nxt;
    }
    if (p != NIL) { *ovl = true; *ob = OB_CORRUPT; }   // the lists hold more than N entries: corrupt
  }
  if (!found) r.ca = S.d[0].coll;
  return r;
}

// read stamps of the 3x3 cells around local cell c by one thread
__device__ bool stamp_read_thread(const Box& B, const RoundArgs& A, int64_t base, int c, uint64_t clk) {
  const int x = c % B.Nxc, y = c / B.Nxc;
  bool bad = false;
  for (int q = 0; q < 9; q++) {
    const int64_t gc = base + pbc_cy(B, y + q / 3 - 1) * B.Nxc + pbc_cx(B, x + q % 3 - 1);
    if (A.lw[gc] > clk) bad = true;
    if (A.lr[gc] < clk) atomicMax((unsigned long long*)&A.lr[gc], (unsigned long long)clk);
  }
  return bad;
}

// one selected event by one thread: the handlers of process_event_warp with
// the same arithmetic; all four virial terms end in r.ct4
__device__ void process_event_thread(const SysDev& S, const RoundArgs& A, int s, int64_t g, EvResult& res,
                                     double* ct4) {
  const Box& B = S.B;
  const int N = B.N;
  const int64_t base = A.coff[s], dbase = A.doff[s];
  const int a = (int)(g - dbase);
  uint64_t key;
  const int slot = next_slot(S, a, &key);
  const Ev E = S.ev[slot];
  const double t = E.t;
  const uint64_t clk = E.tie;
  int nd = 0;
  res.dc[nd++] = (int32_t)(base + A.fc[2 * g]);
  if (A.fc[2 * g + 1] != A.fc[2 * g]) res.dc[nd++] = (int32_t)(base + A.fc[2 * g + 1]);
  Disk Da = S.d[a];
  const int ax = S.cx[a], ay = S.cy[a];
  const int ca = cell_of(B, ax, ay);
  res.npair = res.npred = res.ncol = res.ncross = res.nstale = res.nscreen = 0;
  ct4[0] = ct4[1] = ct4[2] = ct4[3] = 0;
  res.ovl = res.bad = false;
  res.ob = -1;
  // what the shared tail does, set by the handler (see process_event_warp)
  int b = -1;
  int64_t gb = -1;
  int pax = ax, pay = ay, pbx = ax, pby = ay;
  int wc1 = -1, rc0 = ca, rc1 = -1;
  bool cross = false;
  Disk Db = Da;
  if (slot >= N) {
    Db = S.d[E.j];
    free_fly_i(B, Da, t);
    if (E.ca != Db.coll) {
      S.d[a] = Da;
      shadow_write(A, g, B, Da, ax, ay, A.epoch[s]);
      res.nstale = 1;
    } else {
      b = E.j;
      gb = dbase + b;
      res.dc[nd++] = (int32_t)(base + A.fc[2 * gb]);
      if (A.fc[2 * gb + 1] != A.fc[2 * gb]) res.dc[nd++] = (int32_t)(base + A.fc[2 * gb + 1]);
      const int bx = S.cx[b], by = S.cy[b];
      const int cb = cell_of(B, bx, by);
      free_fly_i(B, Db, t);
      Da.coll++;
      Db.coll++;
      double dx = Db.x - Da.x, dy = Db.y - Da.y;
      const double dvx = Db.vx - Da.vx, dvy = Db.vy - Da.vy;
      const double msum = Da.m + Db.m;
      const double invMass = __double_as_longlong(msum) == 0x4000000000000000ll ? 0.5 : 1 / msum;
      pbc_i(B, dx, dy);
      const double collKernel = invMass * (1 + S.res) * (dx * dvx + dy * dvy);
      const double distSquared = contact2(B, Da.rad, Db.rad);
      const double f = __double_as_longlong(distSquared) == 0x4010000000000000ll
          ? collKernel * 0.25 : collKernel / distSquared;
      const double cf = Da.m * Db.m * f;
      ct4[0] = cf * dx * dx;
      ct4[1] = cf * dy * dy;
      ct4[2] = cf * dx * dy;
      ct4[3] = cf * dy * dx;
      Da.vx += f * Db.m * dx;
      Da.vy += f * Db.m * dy;
      Db.vx -= f * Da.m * dx;
      Db.vy -= f * Da.m * dy;
      S.d[a] = Da;
      S.d[b] = Db;
      shadow_write(A, g, B, Da, ax, ay, A.epoch[s]);
      shadow_write(A, gb, B, Db, bx, by, A.epoch[s]);
      if ((A.flags & EDMD_F_TRACE) && S.trace) {
        const unsigned long long k = atomicAdd((unsigned long long*)&S.st->ntrace, 1ull);
        if ((int64_t)k < S.trace_cap) {
          edmd_collision* tr = (edmd_collision*)S.trace + k;
          tr->i = a; tr->j = b; tr->cell_i = ca; tr->cell_j = cb; tr->t = t;
        }
      }
      pbx = bx; pby = by;
      wc1 = cb; rc1 = cb;
      cross = true;
      res.ncol = 1;
    }
  } else {
    free_fly_i(B, Da, t);
    int cx = ax, cy = ay;
    const int pv = S.prv[a], nx = Da.nxt;
    if (pv == NIL) S.head[ca] = nx;
    else S.d[pv].nxt = nx;
    if (nx != NIL) S.prv[nx] = pv;
    switch (E.j) {
      case 1: if (cx - 1 == -1) { cx = B.Nxc - 1; S.crossX[a] -= 1; } else cx -= 1; break;
      case 2: if (cx + 1 == B.Nxc) { cx = 0; S.crossX[a] += 1; } else cx += 1; break;
      case 3: if (cy - 1 == -1) { cy = B.Nyc - 1; S.crossY[a] -= 1; } else cy -= 1; break;
      default: if (cy + 1 == B.Nyc) { cy = 0; S.crossY[a] += 1; } else cy += 1; break;
    }
    const int c = cell_of(B, cx, cy);
    const int h = S.head[c];
    S.cx[a] = cx;
    S.cy[a] = cy;
    S.prv[a] = NIL;
    Da.nxt = h;
    S.d[a] = Da;
    shadow_write(A, g, B, Da, cx, cy, A.epoch[s]);
    S.head[c] = a;
    if (h != NIL) S.prv[h] = a;
    pax = cx; pay = cy;
    wc1 = c; rc0 = c;
    cross = true;
    res.ncross = 1;
  }
  // ---- the tail shared by the three handlers, so that lanes running
  // different event kinds share its instructions: causality stamps, then per
  // changed disk (a, then b) its crossing event, its collision event
  // (collisionEvent), the event records and its attribution
  res.bad |= stamp_write(A, base, ca, clk) | (wc1 >= 0 && stamp_write(A, base, wc1, clk));
  res.bad |= stamp_read_thread(B, A, base, rc0, clk);
  if (rc1 >= 0) res.bad |= stamp_read_thread(B, A, base, rc1, clk);
  res.npred = b >= 0 ? 2 : 1;
  for (int q = 0; q < 2; q++) {
    const int d = q ? b : a;
    if (d < 0) break;
    const int64_t gd = q ? gb : g;
    const Disk Dd = q ? Db : Da;
    const int X = q ? pbx : pax, Y = q ? pby : pay;
    if (cross) {
      int dir;
      const double tc = crossing_time_i(B, Dd, X, Y, t, &dir);
      set_event(S, d, tc, dir, 0, 0, clk);
    }
    const bool had = res.ovl;
    const Pred pr = predict_thread(S, A, s, d, Dd, X, Y, t, &res.npair, &res.nscreen, &res.ovl, &res.ob);
    if (res.ovl && !had) res.a = d;        // the disk whose prediction met the overlap
    const uint8_t rk = new_rank(S, A, dbase, d, q ? a : b, t + pr.dt, pr.partner, clk);
    set_event(S, N + d, t + pr.dt, pr.partner, pr.ca, pr.pcell, clk);
    A.drank[gd] = rk;
    uint64_t k2; int c1, c2;
    const int sl = attribution(S, d, &k2, &c1, &c2);
    A.dkey[gd] = k2; A.dpk[gd] = event_id(A, gd, sl, N); A.fc[2 * gd] = c1; A.fc[2 * gd + 1] = c2;
    res.dc[nd++] = (int32_t)(base + c1);
    if (c2 != c1) res.dc[nd++] = (int32_t)(base + c2);
  }
  res.nd = nd;
  res.key = key;
  res.a = a;
}

// sums and maximum over the lanes of mask m (all 32 lanes call these)
__device__ __forceinline__ double group_sum(unsigned m, double v) {
  double acc = 0;
  for (int l = 0; l < 32; l++) {
    const double x = __shfl_sync(FULLM, v, l);
    if ((m >> l) & 1u) acc += x;
  }
  return acc;
}
__device__ __forceinline__ unsigned long long group_sum_u(unsigned m, unsigned long long v) {
  unsigned long long acc = 0;
  for (int l = 0; l < 32; l++) {
    const unsigned long long x = __shfl_sync(FULLM, v, l);
    if ((m >> l) & 1u) acc += x;
  }
  return acc;
}
__device__ __forceinline__ uint64_t group_max(unsigned m, uint64_t v) {
  uint64_t acc = 0;
  for (int l = 0; l < 32; l++) {
    const uint64_t x = __shfl_sync(FULLM, v, l);
    if (((m >> l) & 1u) && x > acc) acc = x;
  }
  return acc;
}

// the next chunk of a round's selected events for a warp of an event kernel:
// past the first wave (each warp's own index), chunks in the order the
// warps ask for them; none when the first wave holds the whole selection
__device__ __forceinline__ int next_chunk(const RoundArgs& A, int lane, int wave, int chunk, int nsafe) {
  if (nsafe <= wave) return nsafe;
  int q = 0;
  if (lane == 0) q = atomicAdd(A.pnext, 1);
  return wave + chunk * __shfl_sync(FULLM, q, 0);
}

// the selected events of a round, one thread each (rounds of at least
// A.thr_min events; k_process takes the others); per-system counters are
// summed over the lanes of a warp that share the system before one atomic
__global__ void __launch_bounds__(32, 16) k_process_thread(const SysDev* __restrict__ sys, RoundArgs A) {
  const int nsafe = *A.nsafe;
  if (nsafe < A.thr_min) return;
  const int lane = threadIdx.x & 31;
  const int wstart = (blockIdx.x * blockDim.x + threadIdx.x) - lane;
  const int wstride = gridDim.x * blockDim.x;
  const int stripe = (wstart >> 5) & (NSTRIPE - 1);
  // one resident wave: each warp takes the 32 events at its own index, then
  // the warps that finish first take the rest, 32 at a time, from a counter
  for (int w = wstart; w < nsafe; w = next_chunk(A, lane, wstride, 32, nsafe)) {
    const int n = w + lane;
    const bool valid = n < nsafe;
    int s = -1;
    EvResult r;
    double ct4[4] = {0, 0, 0, 0};
    r.nd = 0; r.npair = r.npred = r.ncol = r.ncross = r.nstale = r.nscreen = 0; r.key = 0;
    r.bad = r.ovl = false; r.a = r.ob = -1;
    if (valid) {
      const int64_t g = A.safe[n];
      s = A.dsys[g];
      process_event_thread(sys[s], A, s, g, r, ct4);
      for (int k = 0; k < MAXDIRTY; k++) A.dcell[(int64_t)n * MAXDIRTY + k] = k < r.nd ? r.dc[k] : -1;
      if (r.bad) atomicAdd(A.violations, 1ull);
      if (r.ovl) {
        SysState* R = sys[s].st;
        R->err_a = r.a;
        R->err_b = r.ob;
        R->status = r.ob == OB_CORRUPT ? EDMD_ERR_BUDGET : EDMD_ERR_OVERLAP;
      }
    }
    const unsigned m = __match_any_sync(FULLM, s);
    const bool leader = lane == __ffs(m) - 1;
    const double c0 = group_sum(m, ct4[0]), c1 = group_sum(m, ct4[1]);
    const double c2 = group_sum(m, ct4[2]), c3 = group_sum(m, ct4[3]);
    const unsigned long long ncol = group_sum_u(m, r.ncol), ncross = group_sum_u(m, r.ncross);
    const unsigned long long nstale = group_sum_u(m, r.nstale), npair = group_sum_u(m, r.npair);
    const unsigned long long npred = group_sum_u(m, r.npred), nscr = group_sum_u(m, r.nscreen);
    const uint64_t kmx = group_max(m, r.key);
    if (leader && s >= 0) {
      if (ncol) {
        cnt_addf(A, s, stripe, C_CT0, c0);
        cnt_addf(A, s, stripe, C_CT1, c1);
        cnt_addf(A, s, stripe, C_CT2, c2);
        cnt_addf(A, s, stripe, C_CT3, c3);
      }
      cnt_add(A, s, stripe, C_NCOL, ncol);
      cnt_add(A, s, stripe, C_NCROSS, ncross);
      cnt_add(A, s, stripe, C_NSTALE, nstale);
      cnt_add(A, s, stripe, C_NPAIR, npair);
      cnt_add(A, s, stripe, C_NPRED, npred);
      cnt_add(A, s, stripe, C_NEV, (unsigned long long)__popc(m));
      cnt_add(A, s, stripe, C_NSCREEN, nscr);
      atomicMax((unsigned long long*)&A.cnt[((int64_t)s * NSTRIPE + stripe) * NCNT + C_TLAST],
                (unsigned long long)kmx);
    }
  }
}

// the selected events of a round, one warp each; per-system counters go to
// one of NSTRIPE stripes to spread the atomics
__global__ void __launch_bounds__(32 * WPB, 20) k_process(const SysDev* __restrict__ sys, RoundArgs A) {
  __shared__ WarpScratch scr[WPB];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  WarpScratch* W = &scr[wid];
  const int nsafe = *A.nsafe;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicMax(A.maxsafe, nsafe);
  if (A.thread_kernel && nsafe >= A.thr_min) return;   // k_process_thread takes the round
  const int gw = blockIdx.x * WPB + wid, nw = gridDim.x * WPB;
  const int stripe = gw & (NSTRIPE - 1);
  // one resident wave: each warp takes the event at its own index, then the
  // warps that finish first take the rest from a counter (a grid of one
  // block per event would mostly launch blocks that find nothing to do)
  for (int n = gw; n < nsafe; n = next_chunk(A, lane, nw, 1, nsafe)) {
    const int64_t g = A.safe[n];
    const int s = A.dsys[g];
    EvResult r;
    process_event_warp(sys[s], A, s, g, W, lane, r);
    if (r.ncol && lane < 4) cnt_addf(A, s, stripe, C_CT0 + lane, r.ct);
    if (lane == 0) {
      for (int k = 0; k < MAXDIRTY; k++) A.dcell[(int64_t)n * MAXDIRTY + k] = k < r.nd ? r.dc[k] : -1;
      cnt_add(A, s, stripe, C_NCOL, r.ncol);
      cnt_add(A, s, stripe, C_NCROSS, r.ncross);
      cnt_add(A, s, stripe, C_NSTALE, r.nstale);
      cnt_add(A, s, stripe, C_NPAIR, r.npair);
      cnt_add(A, s, stripe, C_NPRED, r.npred);
      cnt_add(A, s, stripe, C_NEV, 1ull);
      atomicMax((unsigned long long*)&A.cnt[((int64_t)s * NSTRIPE + stripe) * NCNT + C_TLAST],
                (unsigned long long)r.key);
      if (r.bad) atomicAdd(A.violations, 1ull);
      if (r.ovl) {
        SysState* R = sys[s].st;
        R->err_a = r.a;
        R->err_b = r.ob;
        R->status = r.ob == OB_CORRUPT ? EDMD_ERR_BUDGET : EDMD_ERR_OVERLAP;
      }
    }
    __syncwarp();
  }
}

// minimum (key, id) of the events attributed to cell gc (global index) of
// system S: one warp, lanes 0..8 walk the lists of the 3x3 block around it
__device__ void recompute_cell(const SysDev& S, const RoundArgs& A, int64_t base, int64_t dbase, int32_t gc,
                               int lane) {
  const Box& B = S.B;
  const int c = (int)(gc - base);
  uint64_t bk = KINF;
  int32_t bi = IINF;
  if (lane < 9) {
    const int x = c % B.Nxc, y = c / B.Nxc;
    int p = S.head[pbc_cy(B, y + lane / 3 - 1) * B.Nxc + pbc_cx(B, x + lane % 3 - 1)];
    int guard = 0;
    while (p != NIL && guard++ < B.N) {
      const int64_t g = dbase + p;
      const uint64_t k = A.dkey[g];
      if (k != KINF && (A.fc[2 * g] == c || A.fc[2 * g + 1] == c) && pair_less(k, A.dpk[g], bk, bi)) {
        bk = k;
        bi = A.dpk[g];
      }
      p = S.d[p].nxt;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t k2 = __shfl_xor_sync(FULLM, bk, o);
    const int32_t i2 = __shfl_xor_sync(FULLM, bi, o);
    if (pair_less(k2, i2, bk, bi)) { bk = k2; bi = i2; }
  }
  if (lane == 0) {
    A.cmt[gc] = bk;
    A.cmi[gc] = bi;
  }
}

// minimum (key, id) of the events on list q of the 3x3 block around local
// cell c that are attributed to c (the walk of recompute_cell for one list)
__device__ __forceinline__ void list_min(const SysDev& S, const RoundArgs& A, int64_t dbase, int c, int q,
                                         uint64_t& bk, int32_t& bi) {
  const Box& B = S.B;
  const int x = c % B.Nxc, y = c / B.Nxc;
  int p = S.head[pbc_cy(B, y + q / 3 - 1) * B.Nxc + pbc_cx(B, x + q % 3 - 1)];
  int guard = 0;
  while (p != NIL && guard++ < B.N) {
    const int64_t g = dbase + p;
    const uint64_t k = A.dkey[g];
    if (k != KINF && (A.fc[2 * g] == c || A.fc[2 * g + 1] == c) && pair_less(k, A.dpk[g], bk, bi)) {
      bk = k;
      bi = A.dpk[g];
    }
    p = S.d[p].nxt;
  }
}

// the cells whose minimum the selected events can have changed: four cells
// per warp, one 8-lane group each (lane q walks list q of the 3x3 block,
// lane 0 also list 8), the same minima as recompute_cell
__device__ void recompute_cells(const SysDev* __restrict__ sys, const RoundArgs& A) {
  const int lane = threadIdx.x & 31, grp = lane >> 3, q = lane & 7;
  const int64_t total = (int64_t)(*A.nsafe) * MAXDIRTY;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 4 < total; w += nwarps) {
    const int64_t item = w * 4 + grp;
    const int32_t gc = item < total ? A.dcell[item] : -1;
    uint64_t bk = KINF;
    int32_t bi = IINF;
    if (gc >= 0) {
      const int s = A.dsys[A.safe[item / MAXDIRTY]];
      const SysDev& S = sys[s];
      const int c = (int)(gc - A.coff[s]);
      const int64_t dbase = A.doff[s];
      list_min(S, A, dbase, c, q, bk, bi);
      if (q == 0) list_min(S, A, dbase, c, 8, bk, bi);
    }
    for (int o = 4; o > 0; o >>= 1) {
      const uint64_t k2 = __shfl_xor_sync(FULLM, bk, o);
      const int32_t i2 = __shfl_xor_sync(FULLM, bi, o);
      if (pair_less(k2, i2, bk, bi)) { bk = k2; bi = i2; }
    }
    if (gc >= 0 && q == 0) {
      A.cmt[gc] = bk;
      A.cmi[gc] = bi;
    }
  }
}

// is (k, id) the minimum of the (2r+1)^2 window around local cell c?
__device__ bool window_min(const RoundArgs& A, int64_t base, int Nxc, int Nyc, int c, uint64_t k, int32_t id,
                           int r) {
  const int x = c % Nxc, y = c / Nxc;
  for (int dy = -r; dy <= r; dy++) {
    const int yy = wrapi(y + dy, Nyc);
    for (int dx = -r; dx <= r; dx++) {
      const int64_t cc = base + (int64_t)yy * Nxc + wrapi(x + dx, Nxc);
      if (pair_less(A.cmt[cc], A.cmi[cc], k, id)) return false;
    }
  }
  return true;
}

// Block mode (EDMD_F_ROUND_BLOCK): one block per system at a time (persistent
// grid pulling systems from a counter).  The block runs the same rounds as the
// grid-wide kernels -- selection over its cells, one warp per selected event,
// minima of the dirty cells, screenshot barriers and the collision budget --
// separated by block barriers instead of kernel boundaries, and keeps the
// system's counters in shared memory.
constexpr int BMAXEV = 128;          // events processed per round and system
constexpr int BWPB = 4;              // warps per system block

__global__ void __launch_bounds__(32 * BWPB, 4) k_block_rounds(const SysDev* __restrict__ sys, RoundArgs A,
                                                            int32_t* __restrict__ work, int64_t max_rounds) {
  __shared__ WarpScratch scr[BWPB];
  __shared__ int32_t evl[BMAXEV];
  __shared__ int32_t dl[BMAXEV * MAXDIRTY];
  __shared__ int nev, ndl, s_sh, go, stop;
  __shared__ uint64_t tlast, freeze;
  __shared__ unsigned long long c_ncol, c_ncross, c_nstale, c_npair, c_npred, c_nev;
  __shared__ double c_ct[4];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (;;) {
    if (tid == 0) s_sh = atomicAdd(work, 1);
    __syncthreads();
    const int s = s_sh;
    if (s >= A.nsys) break;
    const SysDev& S = sys[s];
    const Box& B = S.B;
    const int N = B.N, C = B.Nxc * B.Nyc;
    const int64_t base = A.coff[s], dbase = A.doff[s];
    if (tid == 0) {
      c_ncol = c_ncross = c_nstale = c_npair = c_npred = c_nev = 0;
      c_ct[0] = c_ct[1] = c_ct[2] = c_ct[3] = 0;
      tlast = 0;
      freeze = KINF;
      stop = S.st->status != EDMD_OK;
    }
    __syncthreads();
    int64_t rounds = 0;
    while (!stop) {
      if (++rounds > max_rounds) {
        if (tid == 0) atomicAdd(A.active, 1);          // budget exhausted
        break;
      }
      if (tid == 0) { nev = 0; ndl = 0; }
      __syncthreads();
      uint64_t lim = time_key(S.ev[2 * N + SP_SCREEN].t);
      if (A.tstop_key < lim) lim = A.tstop_key;
      if (freeze < lim) lim = freeze;
      for (int c = tid; c < C; c += blockDim.x) {
        const uint64_t k = A.cmt[base + c];
        if (k >= lim) continue;
        const int32_t id = A.cmi[base + c];
        const int64_t g = id & GMASK;
        if (A.fc[2 * g] != c) continue;                 // decided at the owner's cell
        if (!window_min(A, base, B.Nxc, B.Nyc, c, k, id, A.radius)) continue;
        const int c2 = A.fc[2 * g + 1];
        if (c2 != c && !window_min(A, base, B.Nxc, B.Nyc, c2, k, id, A.radius)) continue;
        const int q = atomicAdd(&nev, 1);
        if (q < BMAXEV) evl[q] = (int32_t)g;          // the rest waits for the next round
      }
      __syncthreads();
      const int n = nev < BMAXEV ? nev : BMAXEV;
      if (n == 0) {
        // nothing eligible before the screenshot: pass it (takeAScreenshot,
        // src/EDMD.c:4657-4661) or stop
        const double tbar = S.ev[2 * N + SP_SCREEN].t;
        const uint64_t fl = A.tstop_key < freeze ? A.tstop_key : freeze;
        if (tid == 0) {
          go = time_key(tbar) < fl ? 1 : 0;
          if (!go) stop = 1;
        }
        __syncthreads();
        if (go) {
          for (int i = tid; i < N; i += blockDim.x) {
            Disk p = S.d[i];
            free_fly_i(B, p, tbar);
            S.d[i] = p;
            shadow_write(A, dbase + i, B, p, S.cx[i], S.cy[i], A.epoch[s]);
          }
          __syncthreads();
          if (tid == 0) {
            S.ev[2 * N + SP_SCREEN].t = tbar + S.dtime;
            tlast = kmax(tlast, time_key(tbar));
          }
        }
        __syncthreads();
        continue;
      }
      for (int e = wid; e < n; e += BWPB) {
        EvResult r;
        process_event_warp(S, A, s, evl[e], &scr[wid], lane, r);
        if (r.ncol && lane < 4) atomicAdd(&c_ct[lane], r.ct);
        if (lane == 0) {
          const int q = atomicAdd(&ndl, r.nd);
          for (int k = 0; k < r.nd; k++) dl[q + k] = r.dc[k];
          atomicAdd(&c_ncol, r.ncol);
          atomicAdd(&c_ncross, r.ncross);
          atomicAdd(&c_nstale, r.nstale);
          atomicAdd(&c_npair, r.npair);
          atomicAdd(&c_npred, r.npred);
          atomicAdd(&c_nev, 1ull);
          atomicMax((unsigned long long*)&tlast, (unsigned long long)r.key);
          if (r.bad) atomicAdd(A.violations, 1ull);
          if (r.ovl) {
            S.st->err_a = r.a;
            S.st->err_b = r.ob;
            S.st->status = r.ob == OB_CORRUPT ? EDMD_ERR_BUDGET : EDMD_ERR_OVERLAP;
          }
        }
        __syncwarp();
      }
      __syncthreads();
      for (int w = wid; w < ndl; w += BWPB) recompute_cell(S, A, base, dbase, dl[w], lane);
      __syncthreads();
      if (tid == 0) {
        if (S.st->status != EDMD_OK) stop = 1;
        if (freeze == KINF && S.st->ncol + c_ncol >= A.target[s]) freeze = tlast + 1;
      }
      __syncthreads();
    }
    if (tid == 0) {
      SysState* R = S.st;
      for (int k = 0; k < 4; k++) R->collT[k] += c_ct[k];
      R->ncol += c_ncol;
      R->ncol_total += c_ncol;
      R->ncross += c_ncross;
      R->nstale += c_nstale;
      R->npair += c_npair;
      R->npred += c_npred;
      R->nevents += c_nev;
      if (tlast != 0) {
        const double t = key_time(tlast);
        if (t > R->t) R->t = t;
      }
      R->stop_reason = freeze != KINF ? EDMD_STOP_COLL : EDMD_STOP_TIME;
      A.tlast[s] = rounds;                            // rounds this system took
    }
    __syncthreads();
  }
}

// per system, after the round: a system that has met its collision budget
// stops taking events later than the latest one it processed (the earlier
// ones still pending are drained, so the call ends on a state of the serial
// run); a system with nothing eligible left before its screenshot time
// free-flies every disk to it (takeAScreenshot, src/EDMD.c:4657-4661) and
// reschedules it; then the eligibility bound of the next round
__device__ void barrier_systems(const SysDev* __restrict__ sys, const RoundArgs& A, int first, int stride) {
  __shared__ int go;
  for (int s = first; s < A.nsys; s += stride) {
    if (A.lim[s] == 0) continue;      // stopped for the rest of the call
    const SysDev& S = sys[s];
    const int N = S.B.N;
    bool run = false;
    if (threadIdx.x < 32) {
      const int l = threadIdx.x;
      const uint64_t* c = A.cnt + ((int64_t)s * NSTRIPE + l) * NCNT;
      unsigned long long nc = c[C_NCOL];
      uint64_t tl = c[C_TLAST];
      for (int o = 16; o > 0; o >>= 1) {
        nc += __shfl_xor_sync(FULLM, nc, o);
        const uint64_t t2 = __shfl_xor_sync(FULLM, tl, o);
        tl = t2 > tl ? t2 : tl;
      }
      if (l == 0) {
        const SysState* R = S.st;
        const bool ok = R->status == EDMD_OK;
        uint64_t fz = A.freeze[s];
        if (ok && fz == KINF && R->ncol + nc >= A.target[s]) {
          fz = kmax(tl, A.tlast[s]) + 1;
          A.freeze[s] = fz;
        }
        const uint64_t lim = A.tstop_key < fz ? A.tstop_key : fz;
        const int selected = A.selflag[s];
        go = (ok && !selected && time_key(S.ev[2 * N + SP_SCREEN].t) < lim) ? 1 : 0;
        run = ok && (selected || go);
        if (run) atomicAdd(A.active, 1);
        A.selflag[s] = 0;
        // a system with nothing selected and no screenshot to pass has stopped
        if (!run) A.lim[s] = 0;
      }
    }
    __syncthreads();
    if (go) {
      const double tbar = S.ev[2 * N + SP_SCREEN].t;
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        Disk p = S.d[i];
        free_fly_i(S.B, p, tbar);
        // position and time only: the list links are read concurrently by
        // the minima recompute of the same kernel
        S.d[i].x = p.x;
        S.d[i].y = p.y;
        S.d[i].tl = p.tl;
        shadow_write(A, A.doff[s] + i, S.B, p, S.cx[i], S.cy[i], A.epoch[s]);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        S.ev[2 * N + SP_SCREEN].t = tbar + S.dtime;
        A.tlast[s] = kmax(A.tlast[s], time_key(tbar));
      }
    }
    if (threadIdx.x == 0 && A.lim[s] != 0) A.lim[s] = system_limit(S, A, s);
    __syncthreads();
  }
}

// After the round: the per-system barrier (blocks 0 .. nbar-1, one system at
// a time) and the minima of the dirty cells (all blocks) in one launch.  The
// two are independent: the barrier reads the round's counters and writes
// each system's limits and, when it passes a screenshot, the disks'
// positions; the recompute reads event keys, footprints and list links.
__global__ void __launch_bounds__(256) k_recompute_barrier(const SysDev* __restrict__ sys, RoundArgs A,
                                                          int nbar) {
  // the next round's selection count starts empty (this round's is still read)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *A.nsafe_next = 0;
    *A.pnext = 0;                    // the event kernels of this round are done with it
  }
  if ((int)blockIdx.x < nbar) barrier_systems(sys, A, blockIdx.x, nbar);
  recompute_cells(sys, A);
}

// fold the call's counters into each system's state; its time is the last
// processed event or screenshot
__global__ void k_round_finish(const SysDev* __restrict__ sys, RoundArgs A) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= A.nsys) return;
  SysState* R = sys[s].st;
  unsigned long long v[NCNT];
  double ct[4] = {0, 0, 0, 0};
  for (int k = 0; k < NCNT; k++) v[k] = 0;
  uint64_t tl = A.tlast[s];
  for (int l = 0; l < NSTRIPE; l++) {
    const uint64_t* c = A.cnt + ((int64_t)s * NSTRIPE + l) * NCNT;
    for (int k = 0; k < 4; k++) ct[k] += __longlong_as_double((long long)c[k]);
    for (int k = C_NCOL; k <= C_NSCREEN; k++) v[k] += c[k];
    tl = kmax(tl, c[C_TLAST]);
  }
  for (int k = 0; k < 4; k++) R->collT[k] += ct[k];
  R->ncol += v[C_NCOL];
  R->ncol_total += v[C_NCOL];
  R->ncross += v[C_NCROSS];
  R->nstale += v[C_NSTALE];
  R->npair += v[C_NPAIR];
  R->npred += v[C_NPRED];
  R->nevents += v[C_NEV];
  R->nscreen += v[C_NSCREEN];
  if (tl != 0) {
    const double t = key_time(tl);
    if (t > R->t) R->t = t;
  }
  R->stop_reason = A.freeze[s] != KINF ? EDMD_STOP_COLL : EDMD_STOP_TIME;
}

__global__ void k_round_setup(const int64_t* __restrict__ doff, const SysDev* __restrict__ sys,
                              int32_t* dsys) {
  const int s = blockIdx.y;
  const int N = sys[s].B.N;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    dsys[doff[s] + i] = s;
}

struct RoundBufs {
  int32_t *dsys = nullptr, *fc = nullptr, *cmi = nullptr, *safe = nullptr, *nsafe = nullptr;
  int32_t *dcell = nullptr, *selflag = nullptr, *active = nullptr, *dpk = nullptr, *work = nullptr;
  uint8_t *drank = nullptr, *drank_bak = nullptr;
  uint32_t* ikb = nullptr;
  uint64_t* iktie = nullptr;
  int32_t *tsys = nullptr, *tx0 = nullptr, *ty0 = nullptr;
  int64_t *doff = nullptr, *coff = nullptr;
  uint64_t *dkey = nullptr, *cmt = nullptr, *lw = nullptr, *lr = nullptr;
  uint64_t *lim = nullptr, *target = nullptr, *freeze = nullptr, *tlast = nullptr, *cnt = nullptr;
  float4* shp = nullptr;
  float* sht = nullptr;
  double* epoch = nullptr;
  unsigned long long* viol = nullptr;
  int64_t ntiles = 0;
};

int round_init(edmd_ctx* ctx) {
  if (ctx->round) return EDMD_OK;
  for (const SysDev& S : ctx->hs)
    if (S.B.Nxc < 3 || S.B.Nyc < 3) return set_err(ctx, EDMD_ERR_ARG, "the round engine needs at least 3x3 cells");
  RoundBufs* R = new RoundBufs();
  ctx->round = R;
  const int64_t TN = ctx->total_N, TC = ctx->total_C;
  std::vector<int32_t> tsys, tx0, ty0;
  for (int s = 0; s < ctx->nsys; s++) {
    const Box& B = ctx->hs[s].B;
    for (int y = 0; y < B.Nyc; y += TY)
      for (int x = 0; x < B.Nxc; x += TX) {
        tsys.push_back(s);
        tx0.push_back(x);
        ty0.push_back(y);
      }
  }
  R->ntiles = (int64_t)tsys.size();
  if (TN > GMASK) return set_err(ctx, EDMD_ERR_CAPACITY, "the round engine supports up to 2^24 disks per context");
  CK(dalloc(&R->dsys, TN)); CK(dalloc(&R->fc, 2 * TN)); CK(dalloc(&R->dkey, TN)); CK(dalloc(&R->dpk, TN));
  CK(dalloc(&R->drank, TN)); CK(dalloc(&R->drank_bak, TN));
  CK(dalloc(&R->ikb, TN)); CK(dalloc(&R->iktie, TN));
  CK(dalloc(&R->cmi, TC)); CK(dalloc(&R->cmt, TC)); CK(dalloc(&R->lw, TC)); CK(dalloc(&R->lr, TC));
  CK(dalloc(&R->safe, TN)); CK(dalloc(&R->nsafe, 3)); CK(dalloc(&R->dcell, TN * MAXDIRTY));
  CK(dalloc(&R->selflag, ctx->nsys)); CK(dalloc(&R->active, 2)); CK(dalloc(&R->work, 1));
  CK(dalloc(&R->doff, ctx->nsys)); CK(dalloc(&R->coff, ctx->nsys));
  CK(dalloc(&R->lim, ctx->nsys)); CK(dalloc(&R->target, ctx->nsys)); CK(dalloc(&R->freeze, ctx->nsys));
  CK(dalloc(&R->tlast, ctx->nsys)); CK(dalloc(&R->viol, 1));
  CK(dalloc(&R->cnt, (int64_t)ctx->nsys * NSTRIPE * NCNT));
  CK(dalloc(&R->shp, TN)); CK(dalloc(&R->sht, TN)); CK(dalloc(&R->epoch, ctx->nsys));
  CK(dalloc(&R->tsys, R->ntiles)); CK(dalloc(&R->tx0, R->ntiles)); CK(dalloc(&R->ty0, R->ntiles));
  CK(sync_copy(ctx, R->doff, ctx->disk_off.data(), ctx->nsys * 8, cudaMemcpyHostToDevice));
  CK(sync_copy(ctx, R->coff, ctx->cell_off.data(), ctx->nsys * 8, cudaMemcpyHostToDevice));
  CK(sync_copy(ctx, R->tsys, tsys.data(), R->ntiles * 4, cudaMemcpyHostToDevice));
  CK(sync_copy(ctx, R->tx0, tx0.data(), R->ntiles * 4, cudaMemcpyHostToDevice));
  CK(sync_copy(ctx, R->ty0, ty0.data(), R->ntiles * 4, cudaMemcpyHostToDevice));
  CK(sync_set(ctx, R->selflag, 0, ctx->nsys * 4));
  // selection tiles of wide windows need more than the default 48 KB of
  // dynamic shared memory
  CK(cudaFuncSetAttribute(k_select<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<3>::bytes));
  CK(cudaFuncSetAttribute(k_select<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<4>::bytes));
  CK(cudaFuncSetAttribute(k_select<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<5>::bytes));
  CK(cudaFuncSetAttribute(k_select<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<6>::bytes));
  CK(cudaFuncSetAttribute(k_select<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<7>::bytes));
  CK(cudaFuncSetAttribute(k_select<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<8>::bytes));
  CK(cudaFuncSetAttribute(k_select<9>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<9>::bytes));
  CK(cudaFuncSetAttribute(k_select<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<10>::bytes));
  CK(cudaFuncSetAttribute(k_select<11>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<11>::bytes));
  CK(cudaFuncSetAttribute(k_select<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SelGeom<12>::bytes));
  k_round_setup<<<dim3(64, ctx->nsys), 256, 0, ctx->stream>>>(R->doff, ctx->ds, R->dsys);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return EDMD_OK;
}


// one round: selection, processing, minima, barriers
cudaError_t enqueue_round(edmd_ctx* ctx, const RoundBufs* R, const RoundArgs& A0, int nsm, int k,
                          bool with_thread) {
  cudaStream_t st = ctx->stream;
  RoundArgs A = A0;                  // round k selects into count k % 2 and empties the other
  A.nsafe = R->nsafe + (k & 1);
  A.nsafe_next = R->nsafe + ((k + 1) & 1);
  A.thread_kernel = with_thread ? 1 : 0;
  const unsigned tgrid = (unsigned)(R->ntiles < nsm * 8 ? R->ntiles : nsm * 8);
  switch (A.radius) {
#define SEL_CASE(R) \
    case R: k_select<R><<<tgrid, TX * TY, SelGeom<R>::bytes, st>>>(ctx->ds, A); break;
    SEL_CASE(3) SEL_CASE(4) SEL_CASE(5) SEL_CASE(6) SEL_CASE(7)
    SEL_CASE(8) SEL_CASE(9) SEL_CASE(10) SEL_CASE(11) SEL_CASE(12)
#undef SEL_CASE
    default: break;   // radius is checked to be 3..RTILE before any round
  }
  // one resident wave of each event kernel: one-warp blocks, 20 per SM (k_process)
  // and 16 per SM (k_process_thread), measured best
  k_process<<<nsm * 20 / WPB, 32 * WPB, 0, st>>>(ctx->ds, A);
  if (with_thread) k_process_thread<<<nsm * 16, 32, 0, st>>>(ctx->ds, A);
  k_recompute_barrier<<<nsm * 8, 256, 0, st>>>(ctx->ds, A, ctx->nsys < nsm * 8 ? ctx->nsys : nsm * 8);
  return cudaGetLastError();
}

}  // namespace

void round_free(edmd_ctx* ctx) {
  RoundBufs* R = (RoundBufs*)ctx->round;
  if (!R) return;
  void* p[] = {R->dsys, R->fc, R->cmi, R->safe, R->nsafe, R->dcell, R->selflag, R->active,
               R->tsys, R->tx0, R->ty0, R->doff, R->coff, R->dkey, R->cmt, R->lw, R->lr,
               R->lim, R->target, R->freeze, R->tlast, R->cnt, R->viol, R->dpk, R->drank,
               R->drank_bak, R->ikb, R->iktie, R->work, R->shp, R->sht, R->epoch};
  for (void* q : p)
    if (q) cudaFree(q);
  delete R;
  ctx->round = nullptr;
}

// rounds until every system has stopped
static int run_rounds(edmd_ctx* ctx, const std::vector<uint64_t>& tgt, double t_stop, uint32_t flags,
                      int32_t radius, bool fresh, int64_t max_rounds, int64_t* rounds_out,
                      int32_t* active_out, unsigned long long* viol_out) {
  const RoundBufs* R = (const RoundBufs*)ctx->round;
  cudaStream_t st = ctx->stream;
  const int64_t TN = ctx->total_N, TC = ctx->total_C;
  CK(cudaMemcpyAsync(R->target, tgt.data(), ctx->nsys * 8, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(R->freeze, 0xff, ctx->nsys * 8, st));
  CK(cudaMemsetAsync(R->tlast, 0, ctx->nsys * 8, st));
  CK(cudaMemsetAsync(R->cnt, 0, (size_t)ctx->nsys * NSTRIPE * NCNT * 8, st));
  CK(cudaMemsetAsync(R->viol, 0, 8, st));
  CK(cudaMemsetAsync(R->lw, 0, TC * 8, st));
  CK(cudaMemsetAsync(R->lr, 0, TC * 8, st));
  CK(cudaMemsetAsync(R->cmt, 0xff, TC * 8, st));
  CK(cudaMemsetAsync(R->cmi, 0x7f, TC * 4, st));
  RoundArgs A;
  A.nsys = ctx->nsys; A.radius = radius; A.TN = TN; A.flags = flags; A.ntiles = (int32_t)R->ntiles;
  {
    // the order-preserving integer image of t_stop (time_key on the host)
    uint64_t u;
    memcpy(&u, &t_stop, 8);
    if (u == 0x8000000000000000ull) u = 0;
    A.tstop_key = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
  }
  A.dsys = R->dsys; A.doff = R->doff; A.coff = R->coff;
  A.dkey = R->dkey; A.dpk = R->dpk; A.drank = R->drank; A.ikb = R->ikb; A.iktie = R->iktie; A.fc = R->fc; A.cmt = R->cmt; A.cmi = R->cmi; A.lw = R->lw; A.lr = R->lr;
  A.safe = R->safe; A.nsafe = R->nsafe; A.dcell = R->dcell; A.selflag = R->selflag;
  A.pnext = R->nsafe + 2;
  A.active = R->active; A.lim = R->lim; A.target = R->target; A.freeze = R->freeze;
  A.maxsafe = R->active + 1; A.thread_kernel = 1;
  // one thread per event needs enough events to keep every SM busy with one
  // lane each: the cells of small systems stay in L2, so 4096 events do; the
  // events of a large system are far apart, each cell list walk misses L2,
  // and below ~16k events a warp's 32 lanes per event hide that latency
  // better (4096-system batch: mixed 2.6e7 coll/s, warp-only 2.4e7,
  // thread-only 2.0e7; 10^6 disks, 8k events a round: warp 3.0e7, thread
  // 2.1e7; 4*10^6 disks, 22k events a round: thread 3.2e7, warp 2.9e7)
  A.thr_min = (flags & EDMD_F_ROUND_THREAD) ? 0
            : (flags & EDMD_F_ROUND_WARP) ? INT32_MAX
            : (TN / ctx->nsys <= 65536 ? 4096 : 16384);
  A.tlast = R->tlast; A.cnt = R->cnt; A.shp = R->shp; A.sht = R->sht; A.epoch = R->epoch; A.tsys = R->tsys; A.tx0 = R->tx0; A.ty0 = R->ty0; A.violations = R->viol;
  const unsigned gd = (unsigned)((TN + 255) / 256);
  // the serial queue keys are still in the event records only when the
  // state comes from a serial engine
  if (fresh) k_rank<<<gd, 256, 0, st>>>(ctx->ds, A);
  k_prep<<<gd, 256, 0, st>>>(ctx->ds, A);
  k_prep_owner<<<gd, 256, 0, st>>>(A);
  k_limits<<<(ctx->nsys + 127) / 128, 128, 0, st>>>(ctx->ds, A);
  ctx->last_launches += fresh ? 4 : 3;
  CK(cudaGetLastError());
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  // grid-wide rounds unless asked otherwise: on the 4096-system batch they
  // run 2.6e7 coll/s against 1.8e7 for one block per system, whose four
  // warps leave the SMs' FP64 pipes idle at the block barriers
  const bool block_mode = (flags & EDMD_F_ROUND_BLOCK) != 0;
  if (block_mode) {
    // enough systems to fill the GPU: one block per system, no grid-wide rounds
    CK(cudaMemsetAsync(R->work, 0, 4, st));
    CK(cudaMemsetAsync(R->active, 0, 4, st));
    k_block_rounds<<<nsm * 4, 32 * BWPB, 0, st>>>(ctx->ds, A, R->work, max_rounds);
    CK(cudaGetLastError());
    ctx->last_launches += 1;
    std::vector<uint64_t> rs(ctx->nsys);
    int32_t capped = 0;
    CK(cudaMemcpyAsync(rs.data(), R->tlast, ctx->nsys * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&capped, R->active, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(viol_out, R->viol, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    uint64_t mx = 0;
    for (uint64_t v : rs) mx = v > mx ? v : mx;
    *rounds_out += (int64_t)mx;
    *active_out = capped;
    return EDMD_OK;
  }
  // A block of rounds is captured into a graph and replayed until every
  // system has stopped; the host polls the active count between blocks.
  // Two graphs: with the thread-per-event kernel, and without it (k_process
  // then takes every round).  Both give the same results; the host runs the
  // second while the rounds stay well below the thread kernel's threshold,
  // which saves a kernel per round that would return at once.
  const int per_graph = 32;         // measured: 32 rounds 0.2-1.6% faster than 16, 64 about the same as 32
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  auto capture = [&](bool with_thread, cudaGraphExec_t* out) -> cudaError_t {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t ce = cudaSuccess;
    for (int k = 0; k < per_graph && ce == cudaSuccess; k++) ce = enqueue_round(ctx, R, A, nsm, k, with_thread);
    cudaError_t ee = cudaStreamEndCapture(st, &graph);
    if (ce == cudaSuccess) ce = ee;
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(out, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    return ce;
  };
  const bool may_thread = A.thr_min != INT32_MAX;
  const bool only_thread = A.thr_min == 0;
  cudaError_t ce = capture(may_thread, &exec[may_thread ? 1 : 0]);
  if (ce != cudaSuccess) return set_err(ctx, EDMD_ERR_CUDA, std::string("round graph: ") + cudaGetErrorString(ce));
  int32_t* active_h = nullptr;
  ce = cudaMallocHost((void**)&active_h, 2 * sizeof(int32_t));
  if (ce != cudaSuccess) {
    for (auto& x : exec) if (x) cudaGraphExecDestroy(x);
    CK(ce);
  }
  int64_t rounds = 0;
  int32_t active = 1;
  bool with_thread = may_thread;
  ce = cudaMemsetAsync(R->nsafe, 0, 12, st);
  while (ce == cudaSuccess && active && rounds < max_rounds) {
    if (!exec[with_thread ? 1 : 0]) {
      ce = capture(with_thread, &exec[with_thread ? 1 : 0]);
      if (ce != cudaSuccess) break;
    }
    ce = cudaMemsetAsync(A.maxsafe, 0, 4, st);
    if (ce == cudaSuccess) ce = cudaGraphLaunch(exec[with_thread ? 1 : 0], st);
    if (ce == cudaSuccess) ctx->last_launches += (int64_t)per_graph * (with_thread ? 4 : 3);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(active_h, R->active, 8, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) break;
    rounds += per_graph;
    active = active_h[0];
    // the thread kernel's graph while rounds come within 3/4 of its threshold
    with_thread = may_thread && (only_thread || (int64_t)active_h[1] * 4 >= (int64_t)A.thr_min * 3);
  }
  for (auto& x : exec) if (x) cudaGraphExecDestroy(x);
  cudaFreeHost(active_h);
  if (ce != cudaSuccess) return set_err(ctx, EDMD_ERR_CUDA, std::string("round graph: ") + cudaGetErrorString(ce));
  k_round_finish<<<(ctx->nsys + 127) / 128, 128, 0, st>>>(ctx->ds, A);
  CK(cudaGetLastError());
  ctx->last_launches += 1;
  CK(cudaMemcpyAsync(viol_out, R->viol, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *rounds_out += rounds;
  *active_out = active;
  return EDMD_OK;
}

extern "C" int edmd_advance_rounds(edmd_ctx* ctx, int64_t max_coll, double t_stop, uint32_t flags,
                                   int32_t radius, int64_t max_rounds, float* elapsed_ms,
                                   int64_t* rounds_out, int64_t* violations_out) {
  if (!ctx) return EDMD_ERR_ARG;
  if (max_coll < 0 || radius < 3 || radius > RTILE || max_rounds < 1)
    return set_err(ctx, EDMD_ERR_ARG, "bad round-engine limits (radius 3..12)");
  int rc = round_init(ctx);
  if (rc) return rc;
  std::vector<SysState> st(ctx->nsys);
  CK(sync_copy(ctx, st.data(), ctx->st, ctx->nsys * sizeof(SysState), cudaMemcpyDeviceToHost));
  std::vector<uint64_t> tgt(ctx->nsys);
  for (int s = 0; s < ctx->nsys; s++) {
    if (st[s].grow) return set_err(ctx, EDMD_ERR_ARG, "the round engine runs the constant-radius phase only");
    if (st[s].status != EDMD_OK) return set_err(ctx, st[s].status, "system is in an error state");
    tgt[s] = st[s].ncol + (uint64_t)max_coll;
  }
  const bool exact = (flags & EDMD_F_EXACT) != 0;
  const bool fresh = !ctx->round_dirty;
  const RoundBufs* R = (const RoundBufs*)ctx->round;
  if (exact) {
    rc = ckpt_save(ctx, CKPT_ROUND);
    if (rc) return rc;
    if (!fresh) CK(cudaMemcpyAsync(R->drank_bak, R->drank, ctx->total_N, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  ctx->round_dirty = true;
  ctx->last_launches = 0;
  CK(cudaEventRecord(ctx->e0, ctx->stream));
  int64_t rounds = 0, viol_total = 0;
  int32_t active = 0;
  int32_t r = radius;
  for (;;) {
    unsigned long long v = 0;
    rc = run_rounds(ctx, tgt, t_stop, flags, r, fresh, max_rounds, &rounds, &active, &v);
    if (rc) return rc;
    viol_total += (int64_t)v;
    if (!exact || v == 0 || active) break;
    // a violation: replay the whole call from its start with a wider window
    if (r >= RTILE) return set_err(ctx, EDMD_ERR_BUDGET, "round engine: violation at the widest window");
    rc = ckpt_restore(ctx, CKPT_ROUND);
    if (rc) return rc;
    if (!fresh) CK(cudaMemcpyAsync(R->drank, R->drank_bak, ctx->total_N, cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->round_dirty = true;
    r = r < 4 ? 4 : (r * 2 < RTILE ? r * 2 : RTILE);
  }
  CK(cudaEventRecord(ctx->e1, ctx->stream));
  CK(cudaEventSynchronize(ctx->e1));
  CK(cudaEventElapsedTime(&ctx->last_ms, ctx->e0, ctx->e1));
  if (elapsed_ms) *elapsed_ms = ctx->last_ms;
  if (rounds_out) *rounds_out = rounds;
  if (violations_out) *violations_out = viol_total;
  const int rs = report_status(ctx, "advance_rounds");
  if (rs != EDMD_OK) return rs;
  if (active) return set_err(ctx, EDMD_ERR_BUDGET, "round budget exhausted");
  return EDMD_OK;
}
