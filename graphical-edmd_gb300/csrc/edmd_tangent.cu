// edmd_tangent.cu -- tangent-linear and adjoint dynamics of the hard-disk system,
// engine checkpoints, and the collision-geometry log that feeds them.
//
// The reference has no derivatives; this is the differentiation pattern built on
// top of its dynamics.  Between collisions a disk flies freely,
//     dr(t) = dr(t0) + dv (t - t0),   dv constant,
// and at an elastic collision of i and j (src/EDMD.c:3587-3827: r = r_j - r_i at
// contact, v = v_j - v_i before it, f = (1+res)/(m_i+m_j) (r.v)/sigma^2,
// v_i += f m_j r, v_j -= f m_i r) the tangent map is that of Dellago, Posch and
// Hoover (Phys. Rev. E 53, 1485 (1996)), re-derived here:
//     dt_c = -(r . dr_ij) / (r . v)                  shift of the collision time
//     drc  = dr_ij + v dt_c                          relative position at contact
//     df   = (f / (r . v)) (v . drc + r . dv_ij)
//     w    = df r + f drc
//     dr_i' = dr_i - Dv_i dt_c,  dr_j' = dr_j - Dv_j dt_c     (Dv = velocity jumps)
//     dv_i' = dv_i + m_j w,      dv_j' = dv_j - m_i w
// The adjoint applies the transpose of the same map backwards over the log.
#include "edmd_ctx.h"

#include <cmath>
#include <cstring>
#include <random>

namespace {

// ---------------------------------------------------------------- tangent kernels

// T is row-major [4N][K]: row 4i+c holds component c (dx, dy, dvx, dvy) of disk
// i for the K tangent vectors, so lane k of a warp reads one coalesced row.
__device__ __forceinline__ void tangent_apply_warp(const edmd_log_entry* __restrict__ log, int64_t M,
                                                   const Disk* __restrict__ d, double* __restrict__ T,
                                                   double* __restrict__ tl, int K, int k) {
  for (int64_t n = 0; n < M; n++) {
    const edmd_log_entry L = log[n];
    const int i = L.i, j = L.j;
    const double mi = d[i].m, mj = d[j].m;
    const double ti = tl[i], tj = tl[j];
    double* Ri = T + (size_t)4 * i * K;
    double* Rj = T + (size_t)4 * j * K;
    if (k < K) {
      double xi = Ri[k], yi = Ri[K + k], vxi = Ri[2 * K + k], vyi = Ri[3 * K + k];
      double xj = Rj[k], yj = Rj[K + k], vxj = Rj[2 * K + k], vyj = Rj[3 * K + k];
      // free flight to the collision
      xi += vxi * (L.t - ti); yi += vyi * (L.t - ti);
      xj += vxj * (L.t - tj); yj += vyj * (L.t - tj);
      const double rv = L.dx * L.dvx + L.dy * L.dvy;
      const double drx = xj - xi, dry = yj - yi, dvx = vxj - vxi, dvy = vyj - vyi;
      const double dtc = -(L.dx * drx + L.dy * dry) / rv;
      const double rcx = drx + L.dvx * dtc, rcy = dry + L.dvy * dtc;
      const double df = (L.f / rv) * (L.dvx * rcx + L.dvy * rcy + L.dx * dvx + L.dy * dvy);
      const double wx = df * L.dx + L.f * rcx, wy = df * L.dy + L.f * rcy;
      const double Dvix = L.f * mj * L.dx, Dviy = L.f * mj * L.dy;
      const double Dvjx = -L.f * mi * L.dx, Dvjy = -L.f * mi * L.dy;
      Ri[k] = xi - Dvix * dtc;       Ri[K + k] = yi - Dviy * dtc;
      Rj[k] = xj - Dvjx * dtc;       Rj[K + k] = yj - Dvjy * dtc;
      Ri[2 * K + k] = vxi + mj * wx; Ri[3 * K + k] = vyi + mj * wy;
      Rj[2 * K + k] = vxj - mi * wx; Rj[3 * K + k] = vyj - mi * wy;
    }
    __syncwarp();
    if (k == 0) { tl[i] = L.t; tl[j] = L.t; }
    __syncwarp();
  }
}

__global__ void k_tangent_apply(const edmd_log_entry* __restrict__ log, int64_t M,
                                const Disk* __restrict__ d, double* __restrict__ T,
                                double* __restrict__ tl, int K) {
  tangent_apply_warp(log, M, d, T, tl, K, threadIdx.x);
}

// value of row e at the common time tq (virtual free flight, T itself unchanged)
__device__ __forceinline__ double row_at(const double* T, const double* tl, int e, int k, int K,
                                         double tq) {
  int c = e & 3;
  double v = T[(size_t)e * K + k];
  if (c < 2) v += T[(size_t)(e + 2) * K + k] * (tq - tl[e >> 2]);
  return v;
}

// per-block partial Gram matrices of the tangent vectors flown to tq; summed
// over the blocks in a fixed order by k_gram_sum, so the result is
// reproducible run to run
__global__ void k_gram(const double* __restrict__ T, const double* __restrict__ tl, int N, int K,
                       const double* __restrict__ tqp, double* __restrict__ Gp) {
  const double tq = *tqp;
  __shared__ double rows[32][33];
  const int k = threadIdx.x & 31, l = threadIdx.x >> 5;   // 32 x 32 threads
  double acc = 0;
  for (int e0 = blockIdx.x * 32; e0 < 4 * N; e0 += gridDim.x * 32) {
    int e = e0 + l;
    rows[l][k] = (e < 4 * N && k < K) ? row_at(T, tl, e, k, K, tq) : 0.0;
    __syncthreads();
    if (k < K && l < K)
      for (int r = 0; r < 32; r++) acc += rows[r][k] * rows[r][l];
    __syncthreads();
  }
  if (k < K && l < K) Gp[(size_t)blockIdx.x * K * K + k * K + l] = acc;
}

__global__ void k_gram_sum(const double* __restrict__ Gp, int nblocks, int K, double* __restrict__ G) {
  const int e = threadIdx.x;
  if (e >= K * K) return;
  double s = 0;
  for (int b = 0; b < nblocks; b++) s += Gp[(size_t)b * K * K + e];
  G[e] = s;
}

// Cholesky G = R^T R (R upper) of one K x K Gram matrix by one warp, logs of
// diag(R) accumulated, Rinv = R^-1.  Right-looking on the warp's shared copy
// M: step j takes the square root of the pivot, scales row j, and lane c
// updates column c of the trailing upper triangle; then lane c solves
// R x = e_c by back substitution into column c of Q.
__device__ void chol_warp(const double* __restrict__ G, int K, double* __restrict__ Rinv,
                          double* __restrict__ logdiag, int accumulate, int* __restrict__ fail,
                          double (*M)[33], double (*Q)[33], int lane) {
  for (int a = 0; a < K; a++)
    if (lane < K) M[a][lane] = G[a * K + lane];
  __syncwarp();
  for (int j = 0; j < K; j++) {
    const double s = M[j][j];
    if (!(s > 0)) {                                 // the same value in every lane
      if (lane == 0) *fail = 1;
      return;
    }
    const double d = sqrt(s);
    __syncwarp();
    if (lane > j && lane < K) M[j][lane] /= d;
    if (lane == j) M[j][j] = d;
    __syncwarp();
    if (lane > j && lane < K) {
      const double rjc = M[j][lane];
      for (int a2 = j + 1; a2 <= lane; a2++) M[a2][lane] -= M[j][a2] * rjc;
    }
    __syncwarp();
  }
  if (accumulate && lane < K) logdiag[lane] += log(M[lane][lane]);
  if (lane < K) {
    for (int a2 = K - 1; a2 >= 0; a2--) {
      double v = (a2 == lane) ? 1.0 : 0.0;
      for (int p = a2 + 1; p < K; p++) v -= M[a2][p] * Q[p][lane];
      Q[a2][lane] = v / M[a2][a2];
    }
    for (int a2 = 0; a2 < K; a2++) Rinv[a2 * K + lane] = Q[a2][lane];
  }
  __syncwarp();
}

__global__ void __launch_bounds__(32) k_chol(const double* __restrict__ G, int K, double* __restrict__ Rinv,
                                             double* __restrict__ logdiag, int accumulate, int* __restrict__ fail) {
  __shared__ double M[32][33], Q[32][33];
  chol_warp(G, K, Rinv, logdiag, accumulate, fail, M, Q, threadIdx.x);
}

// T <- T' Rinv at the common time tq (every disk's tangent clock set to tq)
__device__ __forceinline__ void apply_rinv_disk(double* __restrict__ T, double* __restrict__ tl, int i, int K,
                                                double tq, const double* __restrict__ Rinv) {
  double row[4][32];
  for (int c = 0; c < 4; c++)
    for (int k = 0; k < K; k++) row[c][k] = row_at(T, tl, 4 * i + c, k, K, tq);
  for (int c = 0; c < 4; c++)
    for (int k = 0; k < K; k++) {
      double s = 0;
      for (int l = 0; l <= k; l++) s += row[c][l] * Rinv[l * K + k];
      T[(size_t)(4 * i + c) * K + k] = s;
    }
  tl[i] = tq;
}

__global__ void k_apply_rinv(double* __restrict__ T, double* __restrict__ tl, int N, int K,
                             const double* __restrict__ tqp, const double* __restrict__ Rinv) {
  const double tq = *tqp;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  apply_rinv_disk(T, tl, i, K, tq, Rinv);
}

// ---------------------------------------------------------------- adjoint kernels

// one thread: sweep a segment of the log backwards, applying the transpose of
// the collision map and of the free flights between collisions.
// A is [N][4]: (g_x, g_y, g_vx, g_vy) of each disk at its time ta[i].
__device__ void adjoint_segment(const edmd_log_entry* __restrict__ log, int64_t M,
                                const Disk* __restrict__ d, double* __restrict__ A,
                                double* __restrict__ ta) {
  for (int64_t n = M - 1; n >= 0; n--) {
    const edmd_log_entry L = log[n];
    const int i = L.i, j = L.j;
    const double mi = d[i].m, mj = d[j].m;
    double* ai = A + 4 * (size_t)i;
    double* aj = A + 4 * (size_t)j;
    // transpose of the free flights from the collision to each disk's adjoint time
    double gxi = ai[0], gyi = ai[1], gvxi = ai[2] + ai[0] * (ta[i] - L.t), gvyi = ai[3] + ai[1] * (ta[i] - L.t);
    double gxj = aj[0], gyj = aj[1], gvxj = aj[2] + aj[0] * (ta[j] - L.t), gvyj = aj[3] + aj[1] * (ta[j] - L.t);
    const double rv = L.dx * L.dvx + L.dy * L.dvy;
    const double Dvix = L.f * mj * L.dx, Dviy = L.f * mj * L.dy;
    const double Dvjx = -L.f * mi * L.dx, Dvjy = -L.f * mi * L.dy;
    // w enters dv_i' with +m_j and dv_j' with -m_i
    const double gwx = mj * gvxi - mi * gvxj, gwy = mj * gvyi - mi * gvyj;
    // dt_c enters the positions through -Dv dt_c
    double gdt = -(Dvix * gxi + Dviy * gyi) - (Dvjx * gxj + Dvjy * gyj);
    // w = df r + f drc
    const double gdf = L.dx * gwx + L.dy * gwy;
    double grcx = L.f * gwx, grcy = L.f * gwy;
    // df = (f/rv) (v . drc + r . dv_ij)
    const double s = (L.f / rv) * gdf;
    grcx += s * L.dvx; grcy += s * L.dvy;
    const double gdvx = s * L.dx, gdvy = s * L.dy;
    // drc = dr_ij + v dt_c
    gdt += L.dvx * grcx + L.dvy * grcy;
    // dt_c = -(r . dr_ij)/rv
    const double grx = grcx - (gdt / rv) * L.dx, gry = grcy - (gdt / rv) * L.dy;
    // dr_ij = dr_j - dr_i, dv_ij = dv_j - dv_i
    ai[0] = gxi - grx; ai[1] = gyi - gry; ai[2] = gvxi - gdvx; ai[3] = gvyi - gdvy;
    aj[0] = gxj + grx; aj[1] = gyj + gry; aj[2] = gvxj + gdvx; aj[3] = gvyj + gdvy;
    ta[i] = L.t; ta[j] = L.t;
  }
}

__global__ void k_adjoint_segment(const edmd_log_entry* __restrict__ log, int64_t M,
                                  const Disk* __restrict__ d, double* __restrict__ A,
                                  double* __restrict__ ta) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  adjoint_segment(log, M, d, A, ta);
}

// every disk's adjoint brought back to t0 (transpose of the first free flight)
__global__ void k_adjoint_finish(int N, double* __restrict__ A, const double* __restrict__ ta, double t0) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  A[4 * i + 2] += A[4 * i + 0] * (ta[i] - t0);
  A[4 * i + 3] += A[4 * i + 1] * (ta[i] - t0);
}

__global__ void k_fill(double* p, int64_t n, double v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// ---------------------------------------------------------------- batched kernels
// Every system of a context at once: system s owns the disks doff[s] ..
// doff[s] + N_s - 1 of the concatenated arrays and rows 4 doff[s] .. of T.

// system index of each disk
__global__ void k_disk_sys(const SysDev* __restrict__ sys, const int64_t* __restrict__ doff, int nsys,
                           int32_t* __restrict__ dsys) {
  for (int s = blockIdx.y; s < nsys; s += gridDim.y)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < sys[s].B.N; i += gridDim.x * blockDim.x)
      dsys[doff[s] + i] = s;
}

// every disk's clock set to its system's current time
__global__ void k_fill_sys_time(const SysDev* __restrict__ sys, const int32_t* __restrict__ dsys, int64_t TN,
                                double* __restrict__ tl) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < TN) tl[g] = sys[dsys[g]].st->t;
}

// one warp per system: the tangent map over the system's collision log
__global__ void k_tangent_apply_b(const SysDev* __restrict__ sys, const int64_t* __restrict__ doff,
                                  double* __restrict__ T, double* __restrict__ tl, int K) {
  const SysDev& S = sys[blockIdx.x];
  int64_t M = (int64_t)S.st->nlog;
  if (M > S.log_cap) M = S.log_cap;
  const int64_t o = doff[blockIdx.x];
  tangent_apply_warp((const edmd_log_entry*)S.log, M, S.d, T + (size_t)4 * o * K, tl + o, K, threadIdx.x);
}

// one block of 32 x 32 threads per system: its Gram matrix at its current
// time, rows taken 32 at a time in index order (deterministic)
__global__ void k_gram_b(const SysDev* __restrict__ sys, const int64_t* __restrict__ doff,
                         const double* __restrict__ T, const double* __restrict__ tl, int K,
                         const double* __restrict__ tqs, double* __restrict__ G) {
  __shared__ double rows[32][33];
  const SysDev& S = sys[blockIdx.x];
  const int N = S.B.N;
  const double tq = tqs[blockIdx.x];            // the system's time at the end of the chunk
  const int64_t o = doff[blockIdx.x];
  const double* Ts = T + (size_t)4 * o * K;
  const double* tls = tl + o;
  const int k = threadIdx.x & 31, l = threadIdx.x >> 5;
  double acc = 0;
  for (int e0 = 0; e0 < 4 * N; e0 += 32) {
    const int e = e0 + l;
    rows[l][k] = (e < 4 * N && k < K) ? row_at(Ts, tls, e, k, K, tq) : 0.0;
    __syncthreads();
    if (k <= l && l < K)                            // the upper triangle; G is symmetric
      for (int r = 0; r < 32; r++) acc += rows[r][k] * rows[r][l];
    __syncthreads();
  }
  if (k <= l && l < K) {
    G[(size_t)blockIdx.x * K * K + k * K + l] = acc;
    G[(size_t)blockIdx.x * K * K + l * K + k] = acc;
  }
}

// one warp per system
__global__ void __launch_bounds__(32) k_chol_b(const double* __restrict__ G, int nsys, int K,
                                               double* __restrict__ Rinv, double* __restrict__ logdiag,
                                               int accumulate, int* __restrict__ fail) {
  __shared__ double M[32][33], Q[32][33];
  const int s = blockIdx.x;
  if (s >= nsys) return;
  chol_warp(G + (size_t)s * K * K, K, Rinv + (size_t)s * K * K, logdiag + (size_t)s * K, accumulate, fail + s,
            M, Q, threadIdx.x);
}

__global__ void k_apply_rinv_b(const int64_t* __restrict__ doff, const int32_t* __restrict__ dsys, int64_t TN,
                               double* __restrict__ T, double* __restrict__ tl, int K,
                               const double* __restrict__ tqs, const double* __restrict__ Rinv) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= TN) return;
  const int s = dsys[g];
  const int64_t o = doff[s];
  apply_rinv_disk(T + (size_t)4 * o * K, tl + o, (int)(g - o), K, tqs[s], Rinv + (size_t)s * K * K);
}

// one thread per system: the transposed map backwards over its segment log
__global__ void k_adjoint_segment_b(const SysDev* __restrict__ sys, const int64_t* __restrict__ doff, int nsys,
                                    double* __restrict__ A, double* __restrict__ ta) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const SysDev& S = sys[s];
  int64_t M = (int64_t)S.st->nlog;
  if (M > S.log_cap) M = S.log_cap;
  adjoint_segment((const edmd_log_entry*)S.log, M, S.d, A + 4 * (size_t)doff[s], ta + doff[s]);
}

// every disk's position flown (virtually) to its system's current time
__global__ void k_positions_now_b(const SysDev* __restrict__ sys, const int64_t* __restrict__ doff,
                                  const int32_t* __restrict__ dsys, int64_t TN, double* __restrict__ x,
                                  double* __restrict__ y) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= TN) return;
  const int s = dsys[g];
  const Disk p = sys[s].d[g - doff[s]];
  const double t = sys[s].st->t;
  x[g] = p.x + p.vx * (t - p.tl);
  y[g] = p.y + p.vy * (t - p.tl);
}

// one block per system: MSD = (1/N) sum |u_i - <u>|^2 of the minimum-image
// displacements u from (x0, y0) to (x1, y1), its gradient with respect to
// the final positions in A (velocity parts zero) and the direct term
// 2 (u_i - <u>) / N in (dux, duy); sums over disks by a fixed tree
__global__ void k_msd_b(const SysDev* __restrict__ sys, const int64_t* __restrict__ doff,
                        const double* __restrict__ x0, const double* __restrict__ y0,
                        const double* __restrict__ x1, const double* __restrict__ y1, double* __restrict__ A,
                        double* __restrict__ ta, double* __restrict__ dux, double* __restrict__ duy,
                        double* __restrict__ msd) {
  __shared__ double sx[256], sy[256];
  const SysDev& S = sys[blockIdx.x];
  const int N = S.B.N;
  const double Lx = S.B.Lx, Ly = S.B.Ly, T = S.st->t;
  const int64_t o = doff[blockIdx.x];
  auto disp = [&](int i, double* ux, double* uy) {
    double dx = x1[o + i] - x0[o + i], dy = y1[o + i] - y0[o + i];
    dx -= Lx * nearbyint(dx / Lx);
    dy -= Ly * nearbyint(dy / Ly);
    *ux = dx; *uy = dy;
  };
  double ax = 0, ay = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double ux, uy;
    disp(i, &ux, &uy);
    ax += ux; ay += uy;
  }
  sx[threadIdx.x] = ax; sy[threadIdx.x] = ay;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) { sx[threadIdx.x] += sx[threadIdx.x + w]; sy[threadIdx.x] += sy[threadIdx.x + w]; }
    __syncthreads();
  }
  const double mx = sx[0] / N, my = sy[0] / N;
  __syncthreads();
  double acc = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double ux, uy;
    disp(i, &ux, &uy);
    const double a = ux - mx, b = uy - my;
    acc += a * a + b * b;
    double* Ai = A + 4 * (o + i);
    Ai[0] = 2.0 * a / N; Ai[1] = 2.0 * b / N; Ai[2] = 0; Ai[3] = 0;
    dux[o + i] = 2.0 * a / N; duy[o + i] = 2.0 * b / N;
    ta[o + i] = T;
  }
  sx[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sx[threadIdx.x] += sx[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) msd[blockIdx.x] = sx[0] / N;
}

// every disk's adjoint brought back to its system's initial time t0[s]
__global__ void k_adjoint_finish_b(const int32_t* __restrict__ dsys, int64_t TN, double* __restrict__ A,
                                   const double* __restrict__ ta, const double* __restrict__ t0) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= TN) return;
  const double t = t0[dsys[g]];
  A[4 * g + 2] += A[4 * g + 0] * (ta[g] - t);
  A[4 * g + 3] += A[4 * g + 1] * (ta[g] - t);
}

__global__ void k_sys_times(const SysDev* __restrict__ sys, int nsys, double* __restrict__ t) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) t[s] = sys[s].st->t;
}

// positions of one system flown (virtually) to time t, without touching the state
__global__ void k_positions_at(const Disk* __restrict__ d, int N, double t, double* __restrict__ x,
                               double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  Disk p = d[i];
  x[i] = p.x + p.vx * (t - p.tl);
  y[i] = p.y + p.vy * (t - p.tl);
}

}  // namespace

// ==================================================================== log + checkpoints

static int upload_sysdev(edmd_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->ds, ctx->hs.data(), ctx->nsys * sizeof(SysDev), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return EDMD_OK;
}

extern "C" int edmd_set_log_capacity(edmd_ctx* ctx, int64_t cap) {
  if (!ctx || cap < 0) return EDMD_ERR_ARG;
  if (cap > ctx->log_cap) {
    if (ctx->logbuf) cudaFree(ctx->logbuf);
    ctx->logbuf = nullptr;
    CK(dalloc(&ctx->logbuf, (size_t)ctx->nsys * cap));
    ctx->log_cap = cap;
  }
  for (int s = 0; s < ctx->nsys; s++) {
    ctx->hs[s].log = ctx->logbuf + (size_t)s * ctx->log_cap;
    ctx->hs[s].log_cap = ctx->log_cap;
  }
  return upload_sysdev(ctx);
}

extern "C" int edmd_clear_log(edmd_ctx* ctx) {
  if (!ctx) return EDMD_ERR_ARG;
  for (int s = 0; s < ctx->nsys; s++) CK(cudaMemsetAsync(&ctx->st[s].nlog, 0, 8, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return EDMD_OK;
}

extern "C" int edmd_get_log(edmd_ctx* ctx, int32_t s, edmd_log_entry* out, int64_t cap, int64_t* n) {
  if (!ctx || s < 0 || s >= ctx->nsys || !n) return EDMD_ERR_ARG;
  uint64_t nl = 0;
  CK(sync_copy(ctx, &nl, &ctx->st[s].nlog, 8, cudaMemcpyDeviceToHost));
  *n = (int64_t)nl;
  int64_t k = (int64_t)nl < cap ? (int64_t)nl : cap;
  if (k > ctx->log_cap) k = ctx->log_cap;
  if (out && k > 0)
    CK(sync_copy(ctx, out, ctx->hs[s].log, k * sizeof(edmd_log_entry), cudaMemcpyDeviceToHost));
  return (int64_t)nl > ctx->log_cap ? EDMD_ERR_CAPACITY : EDMD_OK;
}

// the arrays that make up the engine state of every system in the context
static void state_parts(edmd_ctx* ctx, std::vector<std::pair<void*, size_t>>& parts) {
  const size_t TN = ctx->total_N;
  size_t TE = 0, TT = 0;
  for (const SysDev& S : ctx->hs) {
    TE += 2 * (size_t)S.B.N + NSPECIAL;
    for (int h = 0; h < S.nlev; h++) TT += S.lev_cnt[h];
  }
  parts = {{ctx->d, TN * sizeof(Disk)}, {ctx->vr, TN * 8}, {ctx->cx, TN * 4}, {ctx->cy, TN * 4},
           {ctx->prv, TN * 4}, {ctx->crossX, TN * 4}, {ctx->crossY, TN * 4},
           {ctx->head, (size_t)ctx->total_C * 4}, {ctx->ev, TE * sizeof(Ev)}, {ctx->on, TE * 4},
           {ctx->op, TE * 4}, {ctx->tree, TT * sizeof(Node)}, {ctx->st, ctx->nsys * sizeof(SysState)}};
  if (ctx->cal) parts.push_back({ctx->cal, TN * CAL_SUB * CAL_LINE * 2});
  if (ctx->mask) parts.push_back({ctx->mask, TN * 2});
}

int ckpt_save(edmd_ctx* ctx, int32_t slot) {
  std::vector<std::pair<void*, size_t>> parts;
  state_parts(ctx, parts);
  size_t total = 0;
  for (auto& p : parts) total += align_up(p.second, 256);
  if ((int)ctx->ckpt.size() <= slot) ctx->ckpt.resize(slot + 1, nullptr);
  if ((int)ctx->ckpt_dirty.size() <= slot) ctx->ckpt_dirty.resize(slot + 1, 0);
  ctx->ckpt_dirty[slot] = ctx->round_dirty ? 1 : 0;
  if (!ctx->ckpt[slot]) CK(cudaMalloc(&ctx->ckpt[slot], total));
  char* dst = (char*)ctx->ckpt[slot];
  for (auto& p : parts) {
    CK(cudaMemcpyAsync(dst, p.first, p.second, cudaMemcpyDeviceToDevice, ctx->stream));
    dst += align_up(p.second, 256);
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return EDMD_OK;
}

int ckpt_restore(edmd_ctx* ctx, int32_t slot) {
  if (slot >= (int)ctx->ckpt.size() || !ctx->ckpt[slot]) return EDMD_ERR_ARG;
  std::vector<std::pair<void*, size_t>> parts;
  state_parts(ctx, parts);
  const char* src = (const char*)ctx->ckpt[slot];
  for (auto& p : parts) {
    CK(cudaMemcpyAsync(p.first, src, p.second, cudaMemcpyDeviceToDevice, ctx->stream));
    src += align_up(p.second, 256);
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->round_dirty = ctx->ckpt_dirty[slot] != 0;
  return EDMD_OK;
}

extern "C" int edmd_checkpoint_save(edmd_ctx* ctx, int32_t slot) {
  if (!ctx || slot < 0 || slot > CKPT_PUBLIC_MAX) return EDMD_ERR_ARG;
  return ckpt_save(ctx, slot);
}

extern "C" int edmd_checkpoint_restore(edmd_ctx* ctx, int32_t slot) {
  if (!ctx || slot < 0 || slot > CKPT_PUBLIC_MAX) return EDMD_ERR_ARG;
  return ckpt_restore(ctx, slot);
}

// ==================================================================== tangent driver

static int current_time(edmd_ctx* ctx, int s, double* t) {
  CK(sync_copy(ctx, t, &ctx->st[s].t, 8, cudaMemcpyDeviceToHost));
  return EDMD_OK;
}

// one advance of every system, logging collision geometry; returns the log length of `s`
static int advance_logged(edmd_ctx* ctx, int s, int64_t ncoll, int64_t* nlog) {
  int rc = edmd_clear_log(ctx);
  if (rc) return rc;
  rc = edmd_advance(ctx, ncoll, INFINITY, EDMD_F_LOG | EDMD_F_COUNT_NORMAL, (int64_t)1 << 60, nullptr);
  if (rc) return rc;
  uint64_t nl = 0;
  CK(sync_copy(ctx, &nl, &ctx->st[s].nlog, 8, cudaMemcpyDeviceToHost));
  if ((int64_t)nl > ctx->log_cap) return set_err(ctx, EDMD_ERR_CAPACITY, "collision log overflow");
  *nlog = (int64_t)nl;
  return EDMD_OK;
}

constexpr int GRAM_BLOCKS = 1024;

// CholQR2 of one system's tangent block at the time *tqp, on stream st
static int cholqr(edmd_ctx* ctx, double* T, double* tl, int N, int K, const double* tqp, double* G, double* Gp,
                  double* Rinv, double* logdiag, int* fail, bool accumulate, cudaStream_t st) {
  for (int pass = 0; pass < 2; pass++) {    // CholQR2: the second pass restores orthogonality
    int blocks = (4 * N + 31) / 32;
    if (blocks > GRAM_BLOCKS) blocks = GRAM_BLOCKS;
    k_gram<<<blocks, 1024, 0, st>>>(T, tl, N, K, tqp, Gp);
    k_gram_sum<<<1, 1024, 0, st>>>(Gp, blocks, K, G);
    k_chol<<<1, 32, 0, st>>>(G, K, Rinv, logdiag, accumulate ? 1 : 0, fail);
    k_apply_rinv<<<(N + 127) / 128, 128, 0, st>>>(T, tl, N, K, tqp, Rinv);
    CK(cudaGetLastError());
  }
  return EDMD_OK;
}

extern "C" int edmd_tangent_run(edmd_ctx* ctx, int32_t s, int32_t K, int64_t n_coll, int64_t qr_every,
                                uint64_t seed, double* tangent_io, double* lyap_out) {
  if (!ctx || s < 0 || s >= ctx->nsys || K < 1 || K > 32 || n_coll < 0 || qr_every < 0)
    return EDMD_ERR_ARG;
  if (ctx->engine != EDMD_ENGINE_WARP) return set_err(ctx, EDMD_ERR_ARG, "tangents need the warp engine");
  const int N = ctx->hs[s].B.N;
  int64_t chunk = qr_every > 0 ? qr_every : (n_coll > 0 ? n_coll : 1);
  int rc = edmd_set_log_capacity(ctx, chunk + 16);
  if (rc) return rc;
  double *T = nullptr, *tl = nullptr, *G = nullptr, *Gp = nullptr, *Rinv = nullptr, *logdiag = nullptr;
  double* tqd = nullptr;
  int* fail = nullptr;
  CK(dalloc(&T, (size_t)4 * N * K));
  CK(dalloc(&tl, N));
  CK(dalloc(&G, K * K));
  CK(dalloc(&Gp, (size_t)GRAM_BLOCKS * K * K));
  CK(dalloc(&Rinv, K * K));
  CK(dalloc(&logdiag, K));
  CK(dalloc(&fail, 1));
  CK(dalloc(&tqd, 1));
  struct Free { void* p[8]; ~Free() { for (void* q : p) if (q) cudaFree(q); } } guard{{T, tl, G, Gp, Rinv, logdiag, fail, tqd}};
  // as in the batched form: each chunk's QR on a second stream beside the
  // next chunk's forward run, at the chunk's end time copied on the device
  if (!ctx->stream2) CK(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
  struct Ev {
    cudaEvent_t e = nullptr;
    ~Ev() { if (e) cudaEventDestroy(e); }
  } ea, eq;
  CK(cudaEventCreateWithFlags(&ea.e, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&eq.e, cudaEventDisableTiming));
  CK(call_begin(ctx));
  double t0;
  if ((rc = current_time(ctx, s, &t0))) return rc;
  // initial vectors: the caller's ([K][N][4]) or seeded random orthonormal ones
  std::vector<double> h((size_t)4 * N * K);
  if (tangent_io) {
    for (int k = 0; k < K; k++)
      for (int e = 0; e < 4 * N; e++) h[(size_t)e * K + k] = tangent_io[(size_t)k * 4 * N + e];
  } else {
    std::mt19937_64 g(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (auto& v : h) v = nd(g);
  }
  CK(cudaMemcpyAsync(T, h.data(), h.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  k_fill<<<(N + 255) / 256, 256, 0, ctx->stream>>>(tl, N, t0);
  CK(cudaMemsetAsync(logdiag, 0, K * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(fail, 0, 4, ctx->stream));
  k_sys_times<<<1, 32, 0, ctx->stream>>>(ctx->ds + s, 1, tqd);
  if (!tangent_io && (rc = cholqr(ctx, T, tl, N, K, tqd, G, Gp, Rinv, logdiag, fail, false, ctx->stream)))
    return rc;
  CK(cudaEventRecord(eq.e, ctx->stream));
  int64_t done = 0;
  while (done < n_coll) {
    int64_t want = n_coll - done < chunk ? n_coll - done : chunk;
    int64_t nl = 0;
    if ((rc = advance_logged(ctx, s, want, &nl))) return rc;
    CK(cudaStreamWaitEvent(ctx->stream, eq.e, 0));             // the previous QR is done
    k_tangent_apply<<<1, 32, 0, ctx->stream>>>((const edmd_log_entry*)ctx->hs[s].log, nl, ctx->hs[s].d, T, tl, K);
    CK(cudaGetLastError());
    if (qr_every > 0) {
      k_sys_times<<<1, 32, 0, ctx->stream>>>(ctx->ds + s, 1, tqd);
      CK(cudaEventRecord(ea.e, ctx->stream));
      CK(cudaStreamWaitEvent(ctx->stream2, ea.e, 0));
      if ((rc = cholqr(ctx, T, tl, N, K, tqd, G, Gp, Rinv, logdiag, fail, true, ctx->stream2))) return rc;
      CK(cudaEventRecord(eq.e, ctx->stream2));
    }
    done += want;
    if (nl < want) break;     // the run ended early (tmax or t_stop)
  }
  CK(cudaStreamWaitEvent(ctx->stream, eq.e, 0));
  {
    int hf = 0;
    CK(sync_copy(ctx, &hf, fail, 4, cudaMemcpyDeviceToHost));
    if (hf) return set_err(ctx, EDMD_ERR_ARG, "tangent vectors became linearly dependent");
  }
  double t = t0;
  if ((rc = current_time(ctx, s, &t))) return rc;
  if (lyap_out) {
    std::vector<double> ld(K);
    CK(sync_copy(ctx, ld.data(), logdiag, K * 8, cudaMemcpyDeviceToHost));
    for (int k = 0; k < K; k++) lyap_out[k] = (t > t0) ? ld[k] / (t - t0) : 0.0;
  }
  if (tangent_io) {
    // tangents at the final time (virtual flight of every row)
    CK(sync_copy(ctx, h.data(), T, h.size() * 8, cudaMemcpyDeviceToHost));
    std::vector<double> htl(N);
    CK(sync_copy(ctx, htl.data(), tl, N * 8, cudaMemcpyDeviceToHost));
    for (int k = 0; k < K; k++)
      for (int i = 0; i < N; i++)
        for (int c = 0; c < 4; c++) {
          double v = h[(size_t)(4 * i + c) * K + k];
          if (c < 2) v += h[(size_t)(4 * i + c + 2) * K + k] * (t - htl[i]);
          tangent_io[(size_t)k * 4 * N + 4 * i + c] = v;
        }
  }
  CK(call_end(ctx));
  return EDMD_OK;
}

// ==================================================================== adjoint driver

extern "C" int edmd_msd_gradient(edmd_ctx* ctx, int32_t s, int64_t n_coll, int64_t ckpt_every,
                                 double t_obs, double* msd_out, double* g_vx, double* g_vy,
                                 double* g_x, double* g_y) {
  if (!ctx || s < 0 || s >= ctx->nsys || n_coll < 1 || ckpt_every < 1) return EDMD_ERR_ARG;
  if (ctx->engine != EDMD_ENGINE_WARP) return set_err(ctx, EDMD_ERR_ARG, "adjoints need the warp engine");
  const int N = ctx->hs[s].B.N;
  const double Lx = ctx->hs[s].B.Lx, Ly = ctx->hs[s].B.Ly;
  int rc = edmd_set_log_capacity(ctx, ckpt_every + 16);
  if (rc) return rc;
  double *A = nullptr, *ta = nullptr, *px = nullptr, *py = nullptr;
  CK(dalloc(&A, 4 * (size_t)N));
  CK(dalloc(&ta, N));
  CK(dalloc(&px, N));
  CK(dalloc(&py, N));
  struct Free { void* p[4]; ~Free() { for (void* q : p) if (q) cudaFree(q); } } guard{{A, ta, px, py}};
  CK(call_begin(ctx));
  double t0, T;
  if ((rc = current_time(ctx, s, &t0))) return rc;
  std::vector<double> x0(N), y0(N), x1(N), y1(N);
  k_positions_at<<<(N + 127) / 128, 128, 0, ctx->stream>>>(ctx->hs[s].d, N, t0, px, py);
  CK(cudaMemcpyAsync(x0.data(), px, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(y0.data(), py, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // forward sweep: exact engine checkpoints at every segment boundary
  const int64_t nseg = (n_coll + ckpt_every - 1) / ckpt_every;
  std::vector<int64_t> seglen(nseg);
  for (int64_t g = 0; g < nseg; g++) {
    if ((rc = edmd_checkpoint_save(ctx, (int32_t)g))) return rc;
    seglen[g] = (g == nseg - 1) ? n_coll - g * ckpt_every : ckpt_every;
    rc = edmd_advance(ctx, seglen[g], INFINITY, EDMD_F_COUNT_NORMAL, (int64_t)1 << 60, nullptr);
    if (rc) return rc;
  }
  if ((rc = edmd_checkpoint_save(ctx, (int32_t)nseg))) return rc;
  if ((rc = current_time(ctx, s, &T))) return rc;
  if (t_obs >= 0) {
    if (t_obs < T) return set_err(ctx, EDMD_ERR_ARG, "t_obs precedes the last processed event");
    T = t_obs;
  }
  k_positions_at<<<(N + 127) / 128, 128, 0, ctx->stream>>>(ctx->hs[s].d, N, T, px, py);
  CK(cudaMemcpyAsync(x1.data(), px, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(y1.data(), py, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // MSD = (1/N) sum |u_i - mean(u)|^2, u = minimum-image displacement
  std::vector<double> ux(N), uy(N);
  double mx = 0, my = 0;
  for (int i = 0; i < N; i++) {
    double dx = x1[i] - x0[i], dy = y1[i] - y0[i];
    dx -= Lx * std::nearbyint(dx / Lx);
    dy -= Ly * std::nearbyint(dy / Ly);
    ux[i] = dx; uy[i] = dy; mx += dx; my += dy;
  }
  mx /= N; my /= N;
  double msd = 0;
  std::vector<double> hA(4 * (size_t)N, 0.0);
  for (int i = 0; i < N; i++) {
    double a = ux[i] - mx, b = uy[i] - my;
    msd += a * a + b * b;
    hA[4 * i + 0] = 2.0 * a / N;
    hA[4 * i + 1] = 2.0 * b / N;
  }
  msd /= N;
  CK(cudaMemcpyAsync(A, hA.data(), hA.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  k_fill<<<(N + 255) / 256, 256, 0, ctx->stream>>>(ta, N, T);
  // reverse sweep: recompute each segment from its checkpoint, then its adjoint
  for (int64_t g = nseg - 1; g >= 0; g--) {
    if ((rc = edmd_checkpoint_restore(ctx, (int32_t)g))) return rc;
    int64_t nl = 0;
    if ((rc = advance_logged(ctx, s, seglen[g], &nl))) return rc;
    k_adjoint_segment<<<1, 1, 0, ctx->stream>>>((const edmd_log_entry*)ctx->hs[s].log, nl, ctx->hs[s].d, A, ta);
    CK(cudaGetLastError());
  }
  k_adjoint_finish<<<(N + 127) / 128, 128, 0, ctx->stream>>>(N, A, ta, t0);
  CK(cudaMemcpyAsync(hA.data(), A, hA.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // leave the engine at the end of the run
  if ((rc = edmd_checkpoint_restore(ctx, (int32_t)nseg))) return rc;
  // u = r(t) - r(0) also depends on the initial positions directly
  for (int i = 0; i < N; i++) {
    if (g_x) g_x[i] = hA[4 * i + 0] - 2.0 * (ux[i] - mx) / N;
    if (g_y) g_y[i] = hA[4 * i + 1] - 2.0 * (uy[i] - my) / N;
    if (g_vx) g_vx[i] = hA[4 * i + 2];
    if (g_vy) g_vy[i] = hA[4 * i + 3];
  }
  if (msd_out) *msd_out = msd;
  CK(call_end(ctx));
  return EDMD_OK;
}

// ==================================================================== batched drivers

namespace {

// device arrays every batched driver needs: each system's first disk and each
// disk's system; freed with the scope
struct BatchIndex {
  int64_t* doff = nullptr;
  int32_t* dsys = nullptr;
  ~BatchIndex() {
    if (doff) cudaFree(doff);
    if (dsys) cudaFree(dsys);
  }
};

int batch_index(edmd_ctx* ctx, BatchIndex& bi) {
  CK(dalloc(&bi.doff, ctx->nsys));
  CK(dalloc(&bi.dsys, ctx->total_N));
  CK(cudaMemcpyAsync(bi.doff, ctx->disk_off.data(), ctx->nsys * sizeof(int64_t), cudaMemcpyHostToDevice,
                     ctx->stream));
  dim3 g((unsigned)((ctx->maxN + 255) / 256), (unsigned)(ctx->nsys < 65535 ? ctx->nsys : 65535));
  k_disk_sys<<<g, 256, 0, ctx->stream>>>(ctx->ds, bi.doff, ctx->nsys, bi.dsys);
  CK(cudaGetLastError());
  return EDMD_OK;
}

// one advance of every system with the collision log; EDMD_ERR_CAPACITY when
// a system logged more than the log holds
int advance_logged_all(edmd_ctx* ctx, int64_t ncoll) {
  int rc = edmd_clear_log(ctx);
  if (rc) return rc;
  rc = edmd_advance(ctx, ncoll, INFINITY, EDMD_F_LOG | EDMD_F_COUNT_NORMAL, (int64_t)1 << 60, nullptr);
  if (rc) return rc;
  std::vector<uint64_t> nl(ctx->nsys);
  CK(sync_copy2d(ctx, nl.data(), 8, &ctx->st[0].nlog, sizeof(SysState), 8, ctx->nsys, cudaMemcpyDeviceToHost));
  for (uint64_t v : nl)
    if ((int64_t)v > ctx->log_cap) return set_err(ctx, EDMD_ERR_CAPACITY, "collision log overflow");
  return EDMD_OK;
}

// CholQR2 of every system's tangent block at the times tqs, on stream st
int cholqr_b(edmd_ctx* ctx, const BatchIndex& bi, double* T, double* tl, int K, double* G, double* Rinv,
             double* logdiag, int* fail, bool accumulate, const double* tqs, cudaStream_t st) {
  const int64_t TN = ctx->total_N;
  for (int pass = 0; pass < 2; pass++) {    // CholQR2: the second pass restores orthogonality
    k_gram_b<<<ctx->nsys, 1024, 0, st>>>(ctx->ds, bi.doff, T, tl, K, tqs, G);
    k_chol_b<<<ctx->nsys, 32, 0, st>>>(G, ctx->nsys, K, Rinv, logdiag, accumulate ? 1 : 0, fail);
    k_apply_rinv_b<<<(unsigned)((TN + 127) / 128), 128, 0, st>>>(bi.doff, bi.dsys, TN, T, tl, K, tqs, Rinv);
    CK(cudaGetLastError());
  }
  return EDMD_OK;
}

int check_fail(edmd_ctx* ctx, const int* fail) {
  std::vector<int> h(ctx->nsys);
  CK(sync_copy(ctx, h.data(), fail, ctx->nsys * sizeof(int), cudaMemcpyDeviceToHost));
  for (int s = 0; s < ctx->nsys; s++)
    if (h[s]) return set_err(ctx, EDMD_ERR_ARG, "tangent vectors of system " + std::to_string(s) +
                                                    " became linearly dependent");
  return EDMD_OK;
}

int sys_times(edmd_ctx* ctx, double* host) {
  CK(sync_copy2d(ctx, host, 8, &ctx->st[0].t, sizeof(SysState), 8, ctx->nsys, cudaMemcpyDeviceToHost));
  return EDMD_OK;
}

}  // namespace

extern "C" int edmd_tangent_run_batch(edmd_ctx* ctx, int32_t K, int64_t n_coll, int64_t qr_every, uint64_t seed,
                                      double* lyap_out) {
  if (!ctx || K < 1 || K > 32 || n_coll < 0 || qr_every < 0) return EDMD_ERR_ARG;
  if (ctx->engine != EDMD_ENGINE_WARP) return set_err(ctx, EDMD_ERR_ARG, "tangents need the warp engine");
  const int64_t TN = ctx->total_N;
  const int nsys = ctx->nsys;
  const int64_t chunk = qr_every > 0 ? qr_every : (n_coll > 0 ? n_coll : 1);
  int rc = edmd_set_log_capacity(ctx, chunk + 16);
  if (rc) return rc;
  BatchIndex bi;
  if ((rc = batch_index(ctx, bi))) return rc;
  double *T = nullptr, *tl = nullptr, *G = nullptr, *Rinv = nullptr, *logdiag = nullptr, *tqs = nullptr;
  int* fail = nullptr;
  CK(dalloc(&T, (size_t)4 * TN * K));
  CK(dalloc(&tl, TN));
  CK(dalloc(&G, (size_t)nsys * K * K));
  CK(dalloc(&Rinv, (size_t)nsys * K * K));
  CK(dalloc(&logdiag, (size_t)nsys * K));
  CK(dalloc(&fail, nsys));
  CK(dalloc(&tqs, nsys));
  struct Free { void* p[7]; ~Free() { for (void* q : p) if (q) cudaFree(q); } } guard{{T, tl, G, Rinv, logdiag, fail, tqs}};
  // the QR of a chunk runs on a second stream beside the next chunk's forward
  // run (which does not touch the tangent vectors); the next tangent map
  // waits for it
  if (!ctx->stream2) CK(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
  struct Ev {
    cudaEvent_t e = nullptr;
    ~Ev() { if (e) cudaEventDestroy(e); }
  } ea, eq;
  CK(cudaEventCreateWithFlags(&ea.e, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&eq.e, cudaEventDisableTiming));
  const unsigned gs = (unsigned)((nsys + 127) / 128);
  // system s starts from the vectors edmd_tangent_run draws from seed + s
  // (drawn on the host before the timed part of the call)
  std::vector<double> h((size_t)4 * TN * K);
  for (int s = 0; s < nsys; s++) {
    std::mt19937_64 g(seed + (uint64_t)s);
    std::normal_distribution<double> nd(0.0, 1.0);
    double* hs = h.data() + (size_t)4 * ctx->disk_off[s] * K;
    for (size_t e = 0; e < (size_t)4 * ctx->hs[s].B.N * K; e++) hs[e] = nd(g);
  }
  CK(call_begin(ctx));
  std::vector<double> t0(nsys), t1(nsys);
  if ((rc = sys_times(ctx, t0.data()))) return rc;
  CK(cudaMemcpyAsync(T, h.data(), h.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  k_fill_sys_time<<<(unsigned)((TN + 255) / 256), 256, 0, ctx->stream>>>(ctx->ds, bi.dsys, TN, tl);
  CK(cudaMemsetAsync(logdiag, 0, (size_t)nsys * K * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(fail, 0, nsys * sizeof(int), ctx->stream));
  k_sys_times<<<gs, 128, 0, ctx->stream>>>(ctx->ds, nsys, tqs);
  if ((rc = cholqr_b(ctx, bi, T, tl, K, G, Rinv, logdiag, fail, false, tqs, ctx->stream))) return rc;
  CK(cudaEventRecord(eq.e, ctx->stream));
  for (int64_t done = 0; done < n_coll;) {
    const int64_t want = n_coll - done < chunk ? n_coll - done : chunk;
    if ((rc = advance_logged_all(ctx, want))) return rc;
    CK(cudaStreamWaitEvent(ctx->stream, eq.e, 0));             // the previous QR is done
    k_tangent_apply_b<<<nsys, 32, 0, ctx->stream>>>(ctx->ds, bi.doff, T, tl, K);
    CK(cudaGetLastError());
    if (qr_every > 0) {
      k_sys_times<<<gs, 128, 0, ctx->stream>>>(ctx->ds, nsys, tqs);   // the chunk's end times
      CK(cudaEventRecord(ea.e, ctx->stream));
      CK(cudaStreamWaitEvent(ctx->stream2, ea.e, 0));
      if ((rc = cholqr_b(ctx, bi, T, tl, K, G, Rinv, logdiag, fail, true, tqs, ctx->stream2))) return rc;
      CK(cudaEventRecord(eq.e, ctx->stream2));
    }
    done += want;
  }
  CK(cudaStreamWaitEvent(ctx->stream, eq.e, 0));
  if ((rc = check_fail(ctx, fail))) return rc;
  if (lyap_out) {
    std::vector<double> ld((size_t)nsys * K);
    CK(sync_copy(ctx, ld.data(), logdiag, ld.size() * 8, cudaMemcpyDeviceToHost));
    if ((rc = sys_times(ctx, t1.data()))) return rc;
    for (int s = 0; s < nsys; s++)
      for (int k = 0; k < K; k++)
        lyap_out[(size_t)s * K + k] = (t1[s] > t0[s]) ? ld[(size_t)s * K + k] / (t1[s] - t0[s]) : 0.0;
  }
  CK(call_end(ctx));
  return EDMD_OK;
}

extern "C" int edmd_msd_gradient_batch(edmd_ctx* ctx, int64_t n_coll, int64_t ckpt_every, double* msd_out,
                                       double* g_vx, double* g_vy, double* g_x, double* g_y) {
  if (!ctx || n_coll < 1 || ckpt_every < 1) return EDMD_ERR_ARG;
  if (ctx->engine != EDMD_ENGINE_WARP) return set_err(ctx, EDMD_ERR_ARG, "adjoints need the warp engine");
  const int64_t TN = ctx->total_N;
  const int nsys = ctx->nsys;
  int rc = edmd_set_log_capacity(ctx, ckpt_every + 16);
  if (rc) return rc;
  BatchIndex bi;
  if ((rc = batch_index(ctx, bi))) return rc;
  double *A = nullptr, *ta = nullptr, *x0 = nullptr, *y0 = nullptr, *x1 = nullptr, *y1 = nullptr;
  double *dux = nullptr, *duy = nullptr, *t0 = nullptr, *msd = nullptr;
  CK(dalloc(&A, 4 * (size_t)TN));
  CK(dalloc(&ta, TN)); CK(dalloc(&x0, TN)); CK(dalloc(&y0, TN)); CK(dalloc(&x1, TN)); CK(dalloc(&y1, TN));
  CK(dalloc(&dux, TN)); CK(dalloc(&duy, TN)); CK(dalloc(&t0, nsys)); CK(dalloc(&msd, nsys));
  struct Free { void* p[10]; ~Free() { for (void* q : p) if (q) cudaFree(q); } }
      guard{{A, ta, x0, y0, x1, y1, dux, duy, t0, msd}};
  CK(call_begin(ctx));
  const unsigned gT = (unsigned)((TN + 127) / 128);
  k_sys_times<<<(nsys + 127) / 128, 128, 0, ctx->stream>>>(ctx->ds, nsys, t0);
  k_positions_now_b<<<gT, 128, 0, ctx->stream>>>(ctx->ds, bi.doff, bi.dsys, TN, x0, y0);
  CK(cudaGetLastError());
  // forward sweep: exact engine checkpoints at every segment boundary
  const int64_t nseg = (n_coll + ckpt_every - 1) / ckpt_every;
  std::vector<int64_t> seglen(nseg);
  for (int64_t g = 0; g < nseg; g++) {
    if ((rc = edmd_checkpoint_save(ctx, (int32_t)g))) return rc;
    seglen[g] = (g == nseg - 1) ? n_coll - g * ckpt_every : ckpt_every;
    rc = edmd_advance(ctx, seglen[g], INFINITY, EDMD_F_COUNT_NORMAL, (int64_t)1 << 60, nullptr);
    if (rc) return rc;
  }
  if ((rc = edmd_checkpoint_save(ctx, (int32_t)nseg))) return rc;
  k_positions_now_b<<<gT, 128, 0, ctx->stream>>>(ctx->ds, bi.doff, bi.dsys, TN, x1, y1);
  k_msd_b<<<nsys, 256, 0, ctx->stream>>>(ctx->ds, bi.doff, x0, y0, x1, y1, A, ta, dux, duy, msd);
  CK(cudaGetLastError());
  // reverse sweep: recompute each segment from its checkpoint, then its adjoint
  for (int64_t g = nseg - 1; g >= 0; g--) {
    if ((rc = edmd_checkpoint_restore(ctx, (int32_t)g))) return rc;
    if ((rc = advance_logged_all(ctx, seglen[g]))) return rc;
    k_adjoint_segment_b<<<(nsys + 63) / 64, 64, 0, ctx->stream>>>(ctx->ds, bi.doff, nsys, A, ta);
    CK(cudaGetLastError());
  }
  k_adjoint_finish_b<<<gT, 128, 0, ctx->stream>>>(bi.dsys, TN, A, ta, t0);
  CK(cudaGetLastError());
  // leave the engine at the end of the run
  if ((rc = edmd_checkpoint_restore(ctx, (int32_t)nseg))) return rc;
  std::vector<double> hA(4 * (size_t)TN), hx(TN), hy(TN);
  CK(sync_copy(ctx, hA.data(), A, hA.size() * 8, cudaMemcpyDeviceToHost));
  CK(sync_copy(ctx, hx.data(), dux, TN * 8, cudaMemcpyDeviceToHost));
  CK(sync_copy(ctx, hy.data(), duy, TN * 8, cudaMemcpyDeviceToHost));
  if (msd_out) CK(sync_copy(ctx, msd_out, msd, nsys * 8, cudaMemcpyDeviceToHost));
  // u = r(t) - r(0) also depends on the initial positions directly
  for (int64_t g = 0; g < TN; g++) {
    if (g_x) g_x[g] = hA[4 * g + 0] - hx[g];
    if (g_y) g_y[g] = hA[4 * g + 1] - hy[g];
    if (g_vx) g_vx[g] = hA[4 * g + 2];
    if (g_vy) g_vy[g] = hA[4 * g + 3];
  }
  CK(call_end(ctx));
  return EDMD_OK;
}
