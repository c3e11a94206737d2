// edmd_observe.cu -- observables computed on the device from the engine state.
//
// Pair correlation g(r) of calculate_pcf (src/pcf.c:16-75): every unordered
// pair closer than max_r (minimum image, PBC src/EDMD.c:5896) adds 2 to bin
// (int)(r / dr); the histogram is then divided by 2 pi r dr rho N at the bin
// centres r = (i + 0.5) dr.  The device counts pairs exactly (integers) over
// the cell lists, so the result equals the reference's O(N^2) loop bit for
// bit; positions are the stored ones, as the reference reads them.
#include <cmath>
#include "edmd_ctx.h"

namespace {

// one thread per disk i: pairs (i, j > i) in the cells within reach
__global__ void k_pcf(const SysDev* __restrict__ sys, int s, double dr, double max_r, int nb,
                      int kx, int ky, unsigned long long* __restrict__ hist) {
  extern __shared__ unsigned long long sh[];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  const SysDev& S = sys[s];
  const Box& B = S.B;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < B.N) {
    const Disk P = S.d[i];
    const int X = S.cx[i], Y = S.cy[i];
    // offsets covering the whole grid visit every column / row once
    const int x0 = kx * 2 + 1 >= B.Nxc ? 0 : X - kx, nx = kx * 2 + 1 >= B.Nxc ? B.Nxc : 2 * kx + 1;
    const int y0 = ky * 2 + 1 >= B.Nyc ? 0 : Y - ky, ny = ky * 2 + 1 >= B.Nyc ? B.Nyc : 2 * ky + 1;
    for (int oy = 0; oy < ny; oy++) {
      int cy = (y0 + oy) % B.Nyc;
      if (cy < 0) cy += B.Nyc;
      for (int ox = 0; ox < nx; ox++) {
        int cx = (x0 + ox) % B.Nxc;
        if (cx < 0) cx += B.Nxc;
        int j = S.head[cy * B.Nxc + cx];
        int guard = 0;
        while (j != NIL && guard++ < B.N) {
          const Disk Q = S.d[j];
          if (j > i) {
            double dx = Q.x - P.x, dy = Q.y - P.y;
            pbc(B, dx, dy);
            const double r = sqrt(dx * dx + dy * dy);
            if (r < max_r) {
              const int bin = (int)(r / dr);
              if (bin < nb) atomicAdd(&sh[bin], 1ull);
            }
          }
          j = Q.nxt;
        }
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

}  // namespace

extern "C" int edmd_get_pcf(edmd_ctx* ctx, int32_t s, double dr, double max_r, double* g_out,
                            int32_t cap, int32_t* nbins_out) {
  if (!ctx || s < 0 || s >= ctx->nsys || !(dr > 0) || !(max_r > 0) || !g_out || cap < 1)
    return EDMD_ERR_ARG;
  const SysDev& S = ctx->hs[s];
  const Box& B = S.B;
  if (max_r > (B.Lx < B.Ly ? B.Lx : B.Ly) / 2)
    return set_err(ctx, EDMD_ERR_ARG, "max_r above half the box: the minimum image is ambiguous");
  const int nb = (int)(max_r / dr);        // num_bins of calculate_pcf
  if (nb < 1 || nb > 65536) return set_err(ctx, EDMD_ERR_ARG, "bad number of bins");
  if (nb > cap) return set_err(ctx, EDMD_ERR_CAPACITY, "g(r) output too small");
  // a disk's stored position lies in its cell, so partners within max_r are
  // at most ceil(max_r / cell) + 1 cells away
  const int kx = (int)ceil(max_r / B.cxs) + 1, ky = (int)ceil(max_r / B.cys) + 1;
  unsigned long long* hist = nullptr;
  CK(cudaMalloc(&hist, nb * sizeof(unsigned long long)));
  cudaError_t e = cudaMemsetAsync(hist, 0, nb * sizeof(unsigned long long), ctx->stream);
  if (e == cudaSuccess) {
    k_pcf<<<(B.N + 127) / 128, 128, nb * sizeof(unsigned long long), ctx->stream>>>(ctx->ds, s, dr, max_r, nb,
                                                                                     kx, ky, hist);
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> h(nb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), hist, nb * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(hist);
  CK(e);
  // normalisation of calculate_pcf, same operations in the same order
  const double volume = B.Lx * B.Ly;
  const double density = B.N / volume;
  for (int i = 0; i < nb; i++) {
    const double r = (i + 0.5) * dr;
    const double shell_volume = 2 * M_PI * r * dr;
    const double norm = shell_volume * density * B.N;
    const double g = 2.0 * (double)h[i];
    g_out[i] = norm > 0 ? g / norm : 0.0;
  }
  if (nbins_out) *nbins_out = nb;
  return EDMD_OK;
}
