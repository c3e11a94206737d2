// edmd_ctx.h -- host-side context shared by the engine translation units
// (internal; the public interface is include/edmd_gpu.h).
#pragma once
#include <cstddef>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "edmd_device.cuh"
#include "../../include/edmd_gpu.h"

using namespace edmd;

struct edmd_ctx {
  int nsys = 0;
  int64_t total_N = 0;
  int maxN = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEvent_t c0 = nullptr, c1 = nullptr;  // whole-call timing of the differentiation drivers
  float last_ms = 0;                       // device time of the last timed call (edmd_get_last_ms)
  int64_t last_launches = 0;               // kernels launched by the last advance or round call
  // shared-memory kernel of the warp engine (EDMD_F_SMEM): its system list,
  // work counter, stream and completion event, made on first use
  int32_t* smem_list = nullptr;
  int32_t* smem_work = nullptr;
  cudaStream_t stream2 = nullptr;
  cudaEvent_t e2 = nullptr;
  std::vector<SysDev> hs;
  std::vector<edmd_system_desc> desc;
  std::vector<int64_t> disk_off, cell_off;
  SysDev* ds = nullptr;
  // device arrays shared by all systems (each system owns a slice)
  Disk* d = nullptr; double* vr = nullptr;
  int32_t *cx = nullptr, *cy = nullptr, *prv = nullptr, *crossX = nullptr, *crossY = nullptr;
  int32_t* head = nullptr;
  Ev* ev = nullptr; int32_t *on = nullptr, *op = nullptr;
  Node* tree = nullptr;
  SysState* st = nullptr;
  edmd_collision* trace = nullptr;
  double* rows = nullptr;
  double* stage = nullptr;          // SoA gather buffer (6 x total_N)
  int32_t* work = nullptr;
  int32_t* order = nullptr;      // warp engine: order the systems are taken in
  uint32_t* cost = nullptr;      // warp engine: each system's run time in the last call
  std::vector<int32_t> order_h;
  edmd_log_entry* logbuf = nullptr; // per-system collision-geometry logs
  int64_t log_cap = 0;
  std::vector<void*> ckpt;          // device snapshots of the whole engine state
  std::vector<size_t> ckpt_parts;   // bytes of each array in a snapshot
  uint16_t* cal = nullptr;          // calendars of the thread-per-system engine
  uint16_t* mask = nullptr;
  int engine = 0;                   // EDMD_ENGINE_WARP or EDMD_ENGINE_LANE
  int64_t total_C = 0;
  void* round = nullptr;            // buffers of the round-parallel engine (edmd_round.cu)
  bool round_dirty = false;         // queue order lost: set by the round engine, cleared by a restage
  bool any_additive = false;        // some system uses additive contact (EDMD_CONTACT_ADDITIVE)
  std::vector<char> ckpt_dirty;     // round_dirty of each checkpoint
  std::string err;
};

void round_free(edmd_ctx* ctx);
// device copies of the whole engine state (edmd_tangent.cu); slots above the
// public range are internal
constexpr int32_t CKPT_PUBLIC_MAX = 4096, CKPT_ROUND = 4097;
int ckpt_save(edmd_ctx* ctx, int32_t slot);
int ckpt_restore(edmd_ctx* ctx, int32_t slot);

static inline int set_err(edmd_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  return code;
}
#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess) return set_err(ctx, EDMD_ERR_CUDA, std::string(#call ": ") +   \
                                                                  cudaGetErrorString(_e)); \
  } while (0)

static inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// status, err_a, err_b of every system (three consecutive int32 of SysState)
// after the context's stream; the first system in an error state sets the
// context's message, naming the disks involved, and its status is returned.
// `what` prefixes the message ("initial configuration", "advance", ...).
static inline int report_status(edmd_ctx* ctx, const char* what) {
  struct Trip { int32_t status, a, b; };
  static_assert(offsetof(SysState, err_b) == offsetof(SysState, status) + 8, "status layout");
  std::vector<Trip> st(ctx->nsys);
  cudaError_t e = cudaMemcpy2DAsync(st.data(), sizeof(Trip), &ctx->st[0].status, sizeof(SysState), sizeof(Trip),
                                    ctx->nsys, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return set_err(ctx, EDMD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  for (int s = 0; s < ctx->nsys; s++) {
    const Trip& t = st[s];
    if (t.status == EDMD_OK) continue;
    std::string m = std::string(what) + ": system " + std::to_string(s);
    if (t.status == EDMD_ERR_OVERLAP)
      m += " has overlapping disks " + std::to_string(t.a) + (t.b >= 0 ? " and " + std::to_string(t.b) : "");
    else if (t.status == EDMD_ERR_BUDGET && (t.a == -2 || t.b == -2))
      m += " has a corrupt cell list (a list walk exceeded N; seen from disk " +
           std::to_string(t.a == -2 ? t.b : t.a) + ")";
    else if (t.status == EDMD_ERR_BUDGET)
      m += " exhausted its event budget";
    else if (t.status == EDMD_ERR_ARG)
      m += " has an invalid disk " + std::to_string(t.a);
    else
      m += " stopped with status " + std::to_string(t.status);
    return set_err(ctx, t.status, m);
  }
  return EDMD_OK;
}

// CUDA events on the context's stream around a whole host-driven call (the
// differentiation drivers launch many kernels with host work in between):
// call_begin records the start, call_end the end and stores the elapsed time,
// idle gaps of the stream included, in last_ms.
static inline cudaError_t call_begin(edmd_ctx* c) {
  cudaError_t e = cudaSuccess;
  if (!c->c0) e = cudaEventCreate(&c->c0);
  if (e == cudaSuccess && !c->c1) e = cudaEventCreate(&c->c1);
  return e == cudaSuccess ? cudaEventRecord(c->c0, c->stream) : e;
}
static inline cudaError_t call_end(edmd_ctx* c) {
  cudaError_t e = cudaEventRecord(c->c1, c->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(c->c1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&c->last_ms, c->c0, c->c1);
  return e;
}

// Copies and sets ordered after everything queued on the context's stream.
// The stream is non-blocking, so a plain cudaMemcpy on the legacy default
// stream would not wait for the context's kernels.
static inline cudaError_t sync_copy(edmd_ctx* c, void* dst, const void* src, size_t n, cudaMemcpyKind k) {
  cudaError_t e = cudaMemcpyAsync(dst, src, n, k, c->stream);
  return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}
static inline cudaError_t sync_copy2d(edmd_ctx* c, void* dst, size_t dp, const void* src, size_t sp, size_t w,
                                      size_t h, cudaMemcpyKind k) {
  cudaError_t e = cudaMemcpy2DAsync(dst, dp, src, sp, w, h, k, c->stream);
  return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}
static inline cudaError_t sync_set(edmd_ctx* c, void* dst, int v, size_t n) {
  cudaError_t e = cudaMemsetAsync(dst, v, n, c->stream);
  return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}

template <class T>
static inline cudaError_t dalloc(T** p, size_t n) { return cudaMalloc((void**)p, (n ? n : 1) * sizeof(T)); }
