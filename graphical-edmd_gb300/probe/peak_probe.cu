// peak_probe.cu -- measures the ceilings that bound the event engine on this GPU:
// FP64 warp-instruction issue rate (with 32 and with 1 active lane), FP64
// divide+sqrt rate, FP32 FMA rate, and the latency of dependent global loads
// over an HBM-sized and an L2-sized random permutation.  Prints one JSON line.
// Built by build.py as graphical-edmd_gb300/peak_probe.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cuda_runtime.h>

__global__ void k_dfma(double* out, int iters, int active) {
  int lane = threadIdx.x & 31;
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
         a6 = a0 + 6, a7 = a0 + 7;
  const double b = 1.0000001, c = 1e-9;
  if (lane < active)
    for (int i = 0; i < iters; i++) {
      a0 = a0 * b + c; a1 = a1 * b + c; a2 = a2 * b + c; a3 = a3 * b + c;
      a4 = a4 * b + c; a5 = a5 * b + c; a6 = a6 * b + c; a7 = a7 * b + c;
    }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void k_ffma(float* out, int iters) {
  float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5,
        a6 = a0 + 6, a7 = a0 + 7;
  const float b = 1.0000001f, c = 1e-9f;
  for (int i = 0; i < iters; i++) {
    a0 = a0 * b + c; a1 = a1 * b + c; a2 = a2 * b + c; a3 = a3 * b + c;
    a4 = a4 * b + c; a5 = a5 * b + c; a6 = a6 * b + c; a7 = a7 * b + c;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void k_ddiv(double* out, int iters) {
  double a0 = threadIdx.x * 1e-3 + 1, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  for (int i = 0; i < iters; i++) {
    a0 = 3.0 / a0 + 1.0; a1 = 3.0 / a1 + 1.0; a2 = sqrt(a2) + 1.0; a3 = sqrt(a3) + 1.0;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
}
// each thread follows a random cycle; start indices spread over the array
__global__ void k_chase(const int* next, int* out, int steps, int stride) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) * stride;
  int p = next[i];
  for (int s = 0; s < steps; s++) p = next[p];
  out[blockIdx.x * blockDim.x + threadIdx.x] = p;
}

static float timed(cudaEvent_t a, cudaEvent_t b) { float ms; cudaEventSynchronize(b); cudaEventElapsedTime(&ms, a, b); return ms; }

int main() {
  cudaDeviceProp pr;
  if (cudaGetDeviceProperties(&pr, 0) != cudaSuccess) { printf("{\"error\": \"no device\"}\n"); return 1; }
  const int sms = pr.multiProcessorCount, blocks = sms * 8, threads = 256, iters = 4096;
  double* d; float* f; int* o;
  cudaMalloc(&d, (size_t)blocks * threads * 8); cudaMalloc(&f, (size_t)blocks * threads * 4);
  cudaMalloc(&o, (size_t)sms * 32 * 16 * 4);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  const double warps = (double)blocks * threads / 32;
  double dfma[2]; int act[2] = {32, 1};
  for (int k = 0; k < 2; k++) {
    k_dfma<<<blocks, threads>>>(d, 16, act[k]);
    cudaEventRecord(e0); k_dfma<<<blocks, threads>>>(d, iters, act[k]); cudaEventRecord(e1);
    dfma[k] = warps * iters * 8 / (timed(e0, e1) * 1e-3);
  }
  k_ffma<<<blocks, threads>>>(f, 16);
  cudaEventRecord(e0); k_ffma<<<blocks, threads>>>(f, iters); cudaEventRecord(e1);
  double ffma = warps * 32 * iters * 8 / (timed(e0, e1) * 1e-3);
  k_ddiv<<<blocks, threads>>>(d, 16);
  cudaEventRecord(e0); k_ddiv<<<blocks, threads>>>(d, iters / 8); cudaEventRecord(e1);
  double ddiv = warps * 32 * (iters / 8) * 4 / (timed(e0, e1) * 1e-3);
  double lat[2];
  size_t sizes[2] = {(size_t)64 << 20, (size_t)4 << 20};   // 256 MB (HBM), 16 MB (L2)
  for (int k = 0; k < 2; k++) {
    size_t n = sizes[k];
    std::vector<int> h(n);
    for (size_t i = 0; i < n; i++) h[i] = (int)i;
    unsigned long long x = 88172645463325252ull;
    for (size_t i = n - 1; i > 0; i--) {
      x ^= x << 13; x ^= x >> 7; x ^= x << 17;
      size_t j = x % (i + 1); int t = h[i]; h[i] = h[j]; h[j] = t;
    }
    int* nx; cudaMalloc(&nx, n * 4); cudaMemcpy(nx, h.data(), n * 4, cudaMemcpyHostToDevice);
    const int nthreads = 32 * sms, steps = 2000;
    const int stride = (int)(n / nthreads / 2);      // start indices < n/2 < n
    k_chase<<<sms, 32>>>(nx, o, 10, stride);
    cudaEventRecord(e0); k_chase<<<sms, 32>>>(nx, o, steps, stride); cudaEventRecord(e1);
    lat[k] = timed(e0, e1) * 1e6 / steps;
    cudaFree(nx);
  }
  printf("{\"gpu\": \"%s\", \"sms\": %d, \"fp64_warp_inst_per_s_32_lanes\": %.4g, "
         "\"fp64_warp_inst_per_s_1_lane\": %.4g, \"fp64_lane_dfma_per_s\": %.4g, "
         "\"fp32_lane_ffma_per_s\": %.4g, \"fp64_div_sqrt_per_s\": %.4g, "
         "\"dep_load_ns_hbm\": %.1f, \"dep_load_ns_l2\": %.1f, \"error\": \"%s\"}\n",
         pr.name, sms, dfma[0], dfma[1], dfma[0] * 32, ffma, ddiv, lat[0], lat[1],
         cudaGetErrorString(cudaGetLastError()));
  return 0;
}
