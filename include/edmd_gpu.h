/*
 * edmd_gpu.h -- C ABI of the GB300 event-driven hard-disk engine.
 *
 * Drop-in boundary for the no-graphics event loop of Syrocco/Graphical-EDMD.
 * The reference binds its hot path through five function pointers
 * (src/EDMD.c:317-321: collisionEvent, doTheCollision, freeFly, doTheWall,
 * crossingEvent) bound at src/EDMD.c:1974-1990 / 4755-4759 and driven one
 * event at a time by the loop in main (src/EDMD.c:523-618).  A GPU cannot be
 * driven one event per call, so this ABI replaces that whole loop body in
 * chunks: the host creates systems, then advances them by a number of
 * collisions or up to a time, and reads state back at sampling points.
 *
 * Conventions
 *   - Plain C types only.  Host arrays are caller-owned; the context owns all
 *     device memory and one CUDA stream.  A context is not thread-safe.
 *   - Every function returns an int status (EDMD_OK = 0) and records a
 *     message readable with edmd_last_error(ctx).
 *   - Systems are independent; arrays passed for several systems are the
 *     per-system arrays concatenated in system order.
 *   - Device loops are bounded: a call that would exceed its event budget
 *     returns EDMD_ERR_BUDGET instead of spinning.
 */
#ifndef EDMD_GPU_H
#define EDMD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define EDMD_OK             0
#define EDMD_ERR_ARG        1   /* bad argument or configuration              */
#define EDMD_ERR_CUDA       2   /* a CUDA runtime call failed                 */
#define EDMD_ERR_OVERLAP    3   /* overlap found, as src/EDMD.c:2708-2717     */
#define EDMD_ERR_BUDGET     4   /* per-call event budget exhausted            */
#define EDMD_ERR_CAPACITY   5   /* an internal buffer is too small            */
#define EDMD_ERR_NODEV      6   /* no CUDA device                             */

/* per-system stop reasons reported by edmd_advance */
#define EDMD_STOP_COLL      1   /* max_coll accepted collisions reached       */
#define EDMD_STOP_TIME      2   /* next event at or after t_stop              */
#define EDMD_STOP_TMAX      3   /* loop condition t <= tmax failed            */
#define EDMD_STOP_SCREEN    4   /* stopped right after a screenshot           */
#define EDMD_STOP_GROW      5   /* stopped right after the growth stop        */

/* engines (edmd_set_engine) */
#define EDMD_ENGINE_AUTO    0   /* the thread-per-system engine for contexts of at
                                   least 16384 systems of N <= 32766 (faster there),
                                   else the warp engine; the differentiation calls
                                   need EDMD_ENGINE_WARP */
#define EDMD_ENGINE_WARP    1   /* one warp per system: single large systems  */
#define EDMD_ENGINE_LANE    2   /* one thread per system: large batches, N <= 32766 */

/* edmd_advance flags */
#define EDMD_F_STOP_AT_SCREEN  1u  /* return after each screenshot event      */
#define EDMD_F_STOP_AT_GROW    2u  /* return after the growth-stop event      */
#define EDMD_F_TRACE           4u  /* record accepted collisions              */
#define EDMD_F_COUNT_NORMAL    8u  /* max_coll counts normal-phase only       */
#define EDMD_F_LOG            16u  /* record collision geometry (edmd_log_entry) */
#define EDMD_F_EXACT          32u  /* edmd_advance_rounds: replay on a causality violation */
#define EDMD_F_ROUND_GRID     64u  /* edmd_advance_rounds: grid-wide rounds (the default) */
#define EDMD_F_ROUND_BLOCK   128u  /* edmd_advance_rounds: one block per system, rounds between block barriers */
#define EDMD_F_SCREEN        256u  /* edmd_advance_rounds: FP32 screen of separating pairs before FP64 */
#define EDMD_F_ROUND_THREAD  512u  /* edmd_advance_rounds: one thread per selected event in every round */
#define EDMD_F_ROUND_WARP   1024u  /* edmd_advance_rounds: one warp per selected event in every round */
#define EDMD_F_SMEM         2048u  /* edmd_advance, warp engine with 32 lanes: systems whose engine state
                                      fits one block's shared memory run from shared memory, in a kernel
                                      of their own beside the others (same results) */

/*
 * One periodic 2D system.  Replaces the globals that constantInit
 * (src/EDMD.c:745-1219) and eventListInit (src/EDMD.c:1935-2019) set up.
 */
typedef struct edmd_system_desc {
	int32_t N;             /* number of disks                                  */
	double  Lx, Ly;        /* periodic box                                     */
	double  res;           /* restitution coefficient (-r), 1 = elastic        */
	double  Einit;         /* energy per disk after the growth stop (-E)       */
	double  first_screen;  /* first screenshot time (firstScreen, growth-adjusted) */
	double  dtime;         /* screenshot period (-D)                           */
	double  first_thermo;  /* first thermo time (firstThermo, growth-adjusted) */
	double  dtime_thermo;  /* thermo period (-o)                               */
	double  t_growstop;    /* 1/vr for a growth start, < 0 for a direct start  */
	double  tmax;          /* loop bound (-t, +1/vr for a growth start)        */
	int32_t contact;       /* contact rule, EDMD_CONTACT_* (zero-initialise:
	                          0 is the reference's default)                    */
} edmd_system_desc;

/* Contact distance of disks of radii r1, r2 (DIST / DIST2, src/EDMD.c:35-43).
 * The reference selects it at compile time with NONADDITIVE (0 by default);
 * here it is per system, in every engine and phase (pair solves
 * collisionTimeNormal / collisionTimeGrow and the elastic collision rule). */
#define EDMD_CONTACT_NONADDITIVE 0   /* 2 sqrt(r1 r2): NONADDITIVE 0 */
#define EDMD_CONTACT_ADDITIVE    1   /* r1 + r2:       NONADDITIVE 1 */

/* one accepted collision, as logged by the reference harness */
typedef struct edmd_collision {
	int32_t i, j;          /* owner and partner disk                           */
	int32_t cell_i, cell_j;/* linear cells Y*Nxcells+X                         */
	double  t;
} edmd_collision;

/* geometry of one accepted normal-phase collision, enough to differentiate
 * the elastic map of doTheCollisionNormal (src/EDMD.c:3587-3827) */
typedef struct edmd_log_entry {
	int32_t i, j;          /* owner and partner                               */
	double  t;             /* collision time                                  */
	double  dx, dy;        /* r_j - r_i at contact (nearest periodic image)   */
	double  dvx, dvy;      /* v_j - v_i before the collision                  */
	double  f;             /* funkyFactor: v_i += f m_j (dx,dy), v_j -= f m_i (dx,dy) */
} edmd_log_entry;

/* per-system counters, cumulative since creation */
typedef struct edmd_counters {
	uint64_t ncol;         /* accepted collisions (ncol, reset at growth stop) */
	uint64_t ncol_total;   /* accepted collisions including the growth phase   */
	uint64_t ncross;       /* cell crossings                                   */
	uint64_t nstale;       /* stale collision events popped                    */
	uint64_t npair;        /* pair contact-time solves                         */
	uint64_t npred;        /* collision predictions                            */
	uint64_t nevents;      /* popped events                                    */
	double   t;            /* current simulation time                          */
	int32_t  growing;      /* 1 while the growth phase runs                    */
	int32_t  stop_reason;  /* EDMD_STOP_* of the last advance                  */
	uint64_t nscreen;      /* of npair: pairs the FP32 screen proved separating */
} edmd_counters;

typedef struct edmd_ctx edmd_ctx;

/* Create `nsys` systems (replaces particlesInit's hand-off, cellListInit
 * src/EDMD.c:1906 and eventListInit src/EDMD.c:1935).  Arrays hold the sum
 * of desc[k].N entries.  `vr` (growth rate per disk) may be NULL for direct
 * starts.  Positions must lie in [0,L); radii must be zero or normal
 * positive below 2^1020 (EDMD_ERR_ARG otherwise).  trace_cap is the per-system
 * capacity of the collision trace (0 disables tracing).  *out is set even when
 * the call fails, so that edmd_last_error can be read; destroy it either way. */
int edmd_create(int32_t nsys, const edmd_system_desc* desc,
                const double* x, const double* y, const double* vx, const double* vy,
                const double* rad, const double* m, const double* vr,
                int64_t trace_cap, edmd_ctx** out);

/* Restart every system from host state (the -l load path, particlesInit
 * src/EDMD.c:1366-1451 + cellListInit + eventListInit): clocks, counters and
 * queues are rebuilt, the normal phase is used, the first screenshot is at
 * t = 1 and the first thermo at t = 1000 (src/EDMD.c:244-247). */
int edmd_load_state(edmd_ctx* ctx, const double* x, const double* y, const double* vx,
                    const double* vy, const double* rad, const double* m);

/* Advance every system (replaces the loop body src/EDMD.c:523-618).  Each
 * system stops on its own at max_coll accepted collisions of this call, at
 * the first event with t >= t_stop, when t > tmax, or per `flags`.
 * max_events bounds the events one system may pop in this call.
 * elapsed_ms (may be NULL) receives the device time of the call measured with
 * CUDA events on the context's stream. */
int edmd_advance(edmd_ctx* ctx, int64_t max_coll, double t_stop, uint32_t flags,
                 int64_t max_events, float* elapsed_ms);

/* Round-parallel advance of the constant-radius phase (replaces the same loop
 * body as edmd_advance, src/EDMD.c:523-618, for many events at once).  Each
 * round processes, in every system, the pending events that are the earliest
 * within `radius` cells (3..12) of their footprint (owner's cell plus partner's
 * or target cell), one GPU warp or thread per event; screenshot events act as barriers
 * (every disk is free-flown to them, src/EDMD.c:4657-4661).  A system stops at
 * t_stop, or once it has accepted max_coll collisions in this call: it then
 * finishes the pending events earlier than the latest one it processed, so
 * the call always ends on a state of the serial run (ncol may exceed max_coll
 * by the events of that drain).  At most max_rounds rounds are run (rounded up
 * to a multiple of 32).  Thermo rows are not produced.
 * Collisions, crossings and the final state are those of the serial algorithm
 * unless *violations_out > 0: events processed before an earlier event of the
 * same region, detected exactly with per-cell time stamps (a larger radius
 * makes them rarer).  With EDMD_F_EXACT the call keeps a device copy of the
 * engine state and, after a violation, replays from it with a wider window
 * (3 -> 4 -> 8 -> 12; a violation at 12 returns EDMD_ERR_BUDGET), so a successful
 * call is always the serial result and *violations_out counts the discarded
 * ones.
 * Rounds are grid-wide (selection over every tile, one kernel per step);
 * EDMD_F_ROUND_BLOCK runs them inside one block per system instead.  A round
 * of many events runs one thread per event (from 4096 events when the systems
 * average at most 65536 disks, else from 16384), a smaller one one warp per
 * event; EDMD_F_ROUND_THREAD / EDMD_F_ROUND_WARP force either.  EDMD_F_SCREEN
 * lets the thread path reject separating pairs in FP32 first, with a bound on
 * the FP32 error that keeps every FP64 decision.  All choices give the same
 * results.
 * EDMD_F_TRACE records collisions in processing order.  After this call
 * edmd_advance refuses the context until edmd_load_state restages it. */
int edmd_advance_rounds(edmd_ctx* ctx, int64_t max_coll, double t_stop, uint32_t flags,
                        int32_t radius, int64_t max_rounds, float* elapsed_ms,
                        int64_t* rounds_out, int64_t* violations_out);

/* Free-fly every disk of every system to its current time, the first step of
 * takeAScreenshot (src/EDMD.c:4657-4661). */
int edmd_sync(edmd_ctx* ctx);

/* Pair correlation g(r) of one system, calculate_pcf (src/pcf.c:16-75) as
 * save_pcf calls it (src/EDMD.c:5637): bins of width dr up to max_r
 * (<= half the shorter box side), counted exactly on the device over the cell
 * lists and normalised by 2 pi r dr rho N at the bin centres, so the values
 * are the reference's bit for bit.  Uses the stored positions (call edmd_sync
 * first for positions at the current time).  *nbins_out = (int)(max_r/dr). */
int edmd_get_pcf(edmd_ctx* ctx, int32_t sys, double dr, double max_r, double* g_out, int32_t cap,
                 int32_t* nbins_out);

/* Copy the state of one system to host arrays (any pointer may be NULL). */
int edmd_get_state(edmd_ctx* ctx, int32_t sys, double* x, double* y, double* vx,
                   double* vy, double* rad, double* m, int32_t* cell, uint32_t* coll);

/* The state of every system, concatenated in system order (one gather
 * kernel and one copy per array; any pointer may be NULL). */
int edmd_get_states(edmd_ctx* ctx, double* x, double* y, double* vx, double* vy,
                    double* rad, double* m);

int edmd_get_counters(edmd_ctx* ctx, int32_t sys, edmd_counters* out);
int edmd_get_all_counters(edmd_ctx* ctx, edmd_counters* out);   /* nsys entries */

/* Collision-virial accumulators collTermX, collTermY, collTermXY, collTermYX
 * (src/EDMD.c:3809-3817) of one system; reset them if `reset`. */
int edmd_get_virial(edmd_ctx* ctx, int32_t sys, double out[4], int32_t reset);

/* Thermo rows of one system (t Ncol E p px py pxy pyx a2, saveThermo
 * src/EDMD.c:5232-5697 with Nthermo = 1); returns the row count in *n. */
int edmd_get_thermo(edmd_ctx* ctx, int32_t sys, double* rows, int32_t cap, int32_t* n);

/* edmd_get_thermo, then empty the system's row buffer, so that a long run
 * can drain its rows between calls (each system holds 1024 rows; rows made
 * beyond that are counted in *n but lost, and the call returns
 * EDMD_ERR_CAPACITY). */
int edmd_take_thermo(edmd_ctx* ctx, int32_t sys, double* rows, int32_t cap, int32_t* n);

/* Collision trace of one system recorded since creation (EDMD_F_TRACE). */
int edmd_get_trace(edmd_ctx* ctx, int32_t sys, edmd_collision* out, int64_t cap, int64_t* n);

/* Engine used by contexts created afterwards (default EDMD_ENGINE_AUTO) and
 * the block size of the thread-per-system engine.  Both engines pop events in
 * the reference's exact order and give bit-identical results. */
int edmd_set_engine(int32_t kind);
int edmd_set_lane_threads(int32_t threads_per_block);

/* Lanes per system of the warp engine: 32 (one system per warp, the
 * default), 16, 8 or 4 (two, four or eight systems per warp, each group of
 * lanes running its own system).  All give identical results. */
int edmd_set_warp_group(int32_t lanes);
int edmd_get_engine(const edmd_ctx* ctx);
/* Device time, in ms, of the last edmd_advance, edmd_advance_rounds,
 * edmd_tangent_run(_batch) or edmd_msd_gradient(_batch) call on ctx: CUDA events recorded on
 * the context's stream at the call's start and end (for the host-driven
 * differentiation calls this includes the stream's idle gaps between their
 * kernels).  No reference counterpart (the reference reports no timings). */
int edmd_get_last_ms(const edmd_ctx* ctx, float* ms);

/* Number of this library's kernels launched by the last edmd_advance or
 * edmd_advance_rounds call on ctx (graph-launched rounds counted kernel by
 * kernel).  No reference counterpart. */
int edmd_get_last_launches(const edmd_ctx* ctx, int64_t* n);

/* Select the CUDA device used by contexts created afterwards in this thread
 * (one process per GPU). */
int edmd_set_device(int32_t dev);

/* ---- differentiation (no counterpart in the reference, which has no derivatives) */

/* Per-system capacity of the collision-geometry log written under
 * EDMD_F_LOG; edmd_clear_log resets the logs, edmd_get_log reads one. */
int edmd_set_log_capacity(edmd_ctx* ctx, int64_t cap);
int edmd_clear_log(edmd_ctx* ctx);
int edmd_get_log(edmd_ctx* ctx, int32_t sys, edmd_log_entry* out, int64_t cap, int64_t* n);

/* Exact binary checkpoints of the whole engine state of every system (disks,
 * cell lists, queue, counters): restoring and advancing again reproduces the
 * same events bit for bit. */
int edmd_checkpoint_save(edmd_ctx* ctx, int32_t slot);
int edmd_checkpoint_restore(edmd_ctx* ctx, int32_t slot);

/* Tangent-linear run.  Advances the context n_coll accepted collisions while
 * propagating K <= 32 tangent vectors of system `sys` through the free
 * flights and collisions (the Dellago-Posch-Hoover map).  tangent_io, if not
 * NULL, holds K vectors [K][N][4] (dx, dy, dvx, dvy per disk) on entry and
 * the propagated vectors at the final time on return; if NULL, random
 * orthonormal vectors from `seed` are used.  With qr_every > 0 the vectors are
 * re-orthonormalised every qr_every collisions (Cholesky QR, twice) and
 * lyap_out (K entries, may be NULL) receives the Lyapunov exponents
 * sum(log R_kk) / elapsed time.  Single-system contexts; warp engine. */
int edmd_tangent_run(edmd_ctx* ctx, int32_t sys, int32_t K, int64_t n_coll, int64_t qr_every,
                     uint64_t seed, double* tangent_io, double* lyap_out);

/* Adjoint of the final mean-square displacement.  Advances n_coll accepted
 * collisions from the current state, with exact engine checkpoints every
 * ckpt_every collisions; the reverse pass recomputes each segment from its
 * checkpoint and applies the transposed collision and free-flight maps.
 * The observable is taken at t_obs (>= the time of the last processed event;
 * t_obs < 0 means that time): msd_out = (1/N) sum |u_i - <u>|^2 with u the
 * minimum-image displacement; g_vx, g_vy (g_x, g_y) receive d MSD / d v(0)
 * (d r(0)) at fixed t_obs; any may be NULL.  The context is left at the end
 * of the run.  Single-system contexts; warp engine. */
int edmd_msd_gradient(edmd_ctx* ctx, int32_t sys, int64_t n_coll, int64_t ckpt_every, double t_obs,
                      double* msd_out, double* g_vx, double* g_vy, double* g_x, double* g_y);

/* Batched tangent-linear run: every system of the context at once, in one
 * persistent advance per chunk and one tangent launch per chunk for all
 * systems.  System s propagates K <= 32 random vectors drawn from seed + s
 * (the vectors edmd_tangent_run draws for that seed), re-orthonormalised by
 * CholQR2 every qr_every of its collisions; lyap_out (nsys*K, may be NULL)
 * receives each system's exponents.  No reference counterpart (the reference
 * has no derivatives).  Warp engine. */
int edmd_tangent_run_batch(edmd_ctx* ctx, int32_t K, int64_t n_coll, int64_t qr_every, uint64_t seed,
                           double* lyap_out);

/* Batched adjoint of the final mean-square displacement of every system: the
 * forward sweep with whole-context checkpoints every ckpt_every collisions
 * and the reverse sweep one thread per system.  The observable of system s is
 * taken at the time of its last processed event; msd_out (nsys) and the
 * gradients (total N, concatenated in system order like edmd_get_states) may
 * be NULL.  No reference counterpart.  Warp engine. */
int edmd_msd_gradient_batch(edmd_ctx* ctx, int64_t n_coll, int64_t ckpt_every, double* msd_out,
                            double* g_vx, double* g_vy, double* g_x, double* g_y);

/* Page-locked host buffers for fast host<->device staging. */
int edmd_host_alloc(void** p, int64_t bytes);
int edmd_host_free(void* p);

/*
 * Allocation-free run of one system.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc -- code in a loop where
 * device allocation is forbidden, or a host framework that owns every device
 * buffer.  x, y, vx, vy, rad, m are the CALLER's DEVICE arrays of desc->N
 * entries; the call starts the system from them directly, exactly as
 * edmd_create with vr = NULL does: t = 0, normal phase, first screenshot and
 * thermo events at desc->first_screen and desc->first_thermo, positions used
 * as given (no periodic wrap; a position outside [0, Lx) x [0, Ly), or a
 * radius that is not zero or normal positive below 2^1020, returns
 * EDMD_ERR_ARG naming the disk, as edmd_create does).  It runs until max_coll accepted
 * collisions, t_stop or desc->tmax, free-flies every disk to the final time
 * and writes x, y, vx, vy back.  ncol_out / t_out (host, may be NULL) receive
 * the collisions run and the final time.  `stream` is a cudaStream_t (NULL:
 * default stream).  The call is synchronous: it waits for its stream and
 * reads the result back before it returns.
 *
 * Limits: N <= 8192, Nxcells*Nycells <= 65536, direct starts only
 * (desc->t_growstop < 0); larger systems return EDMD_ERR_CAPACITY.  Each
 * call may process at most 256 events per requested collision plus 256 per
 * disk plus 2^20; beyond that it stops with EDMD_ERR_BUDGET and still writes
 * the state at the stop back (a very dilute system, with many cell crossings
 * per collision, can continue with another call).
 * It allocates nothing: all engine state lives in one file-scope 4 MiB
 * __device__ array that each GPU using this library keeps until exit.  The
 * first call on a device looks up that array's address (once per device, with
 * the device current), so make the first call before any stream capture.
 * Every call reuses the same array and re-initialises what it needs, so calls
 * that overlap on the GPU (other streams, other host threads) race and must
 * be serialised by the caller.  Errors are readable with edmd_last_error(NULL).
 */
int edmd_run_noalloc(const edmd_system_desc* desc, double* x, double* y, double* vx, double* vy,
                     const double* rad, const double* m, int64_t max_coll, double t_stop,
                     int64_t* ncol_out, double* t_out, void* stream);

int edmd_destroy(edmd_ctx* ctx);
/* message of the last failed call on `ctx`; NULL gives edmd_run_noalloc's */
const char* edmd_last_error(const edmd_ctx* ctx);
int edmd_device_info(char* name, int32_t cap, int32_t* sm_count);

#ifdef __cplusplus
}
#endif
#endif
