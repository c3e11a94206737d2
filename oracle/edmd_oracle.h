/*
 * edmd_oracle.h -- CPU oracle for the 2D hard-disk event loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the serial
 * event-driven hard-disk algorithm of Syrocco/Graphical-EDMD (no-graphics
 * build, src/EDMD.c).  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it, and only as the
 * checker or as the timed CPU baseline.  The GPU product never calls it.
 *
 * Parity status: pinned.  Its collision traces and final states are checked
 * bit-for-bit against the reference's own C, compiled unmodified from the
 * reference sources by oracle/Makefile (target `ref`), see
 * tests/golden/make_golden.py.
 */
#ifndef EDMD_ORACLE_H
#define EDMD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* start modes (src/EDMD.c particlesInit 1356-1839) */
enum { ORC_START_HEX = 1, ORC_START_GROW = 2, ORC_START_ARRAYS = 3 };

typedef struct orc_params {
	int    N;            /* requested N (-N); Hex rounds it to Nx*Ny        */
	double phi;          /* --phi                                           */
	double xs;           /* -x, fraction of small disks                     */
	double q;            /* -q, size ratio of small disks                   */
	double aspect;       /* -a                                              */
	double Einit;        /* -E, energy per disk after normalisation         */
	double res;          /* -r, restitution (1 = elastic)                   */
	double tmax;         /* -t                                              */
	double dtime;        /* -D, screenshot period                           */
	double dtimeThermo;  /* -o                                              */
	double firstScreen;  /* first screenshot time (EDMD.c:244)              */
	double firstThermo;  /* first thermo time (EDMD.c:247)                  */
	uint32_t seed;       /* -v                                              */
	int    start;        /* ORC_START_*                                     */
} orc_params;

typedef struct orc_sys orc_sys;

/* one accepted collision, in processing order */
typedef struct orc_coll {
	int32_t i, j, ci, cj;   /* owner, partner, linear cells Y*Nx+X        */
	double  t;
} orc_coll;

/* all popped events (debug / fine-grained parity) */
typedef struct orc_event {
	int32_t type;           /* 0 crossing, 1 collision, 2 screenshot, 3 thermo, 9 growstop */
	int32_t i, j;           /* j: crossing direction or partner            */
	int32_t stale;          /* collision popped with an outdated partner count */
	double  t;
} orc_event;

void     orc_default_params(orc_params* p);
orc_sys* orc_create(const orc_params* p);
/* Build a normal-phase system from explicit state (all disks at time 0). */
orc_sys* orc_create_from_arrays(int N, double Lx, double Ly,
                                const double* x, const double* y,
                                const double* vx, const double* vy,
                                const double* rad, const double* m,
                                const int32_t* type, double res,
                                double firstScreen, double dtime,
                                double firstThermo, double dtimeThermo);
void     orc_destroy(orc_sys* s);

/* Run the reference main loop until `max_coll` accepted normal-phase
 * collisions have been logged, the loop condition t <= tmax fails, or the
 * next event would have time >= t_stop (it is then left in the queue).
 * Collisions are appended to coll_out (capacity coll_cap), events to
 * ev_out (capacity ev_cap, may be NULL).  Returns the number of collisions
 * logged by this call. */
int64_t  orc_run(orc_sys* s, int64_t max_coll, double t_stop,
                 orc_coll* coll_out, int64_t coll_cap,
                 orc_event* ev_out, int64_t ev_cap, int64_t* n_ev_out);

/* free-fly every disk to the current time (takeAScreenshot's first step) */
void     orc_sync_all(orc_sys* s);

/* accessors */
int      orc_N(const orc_sys* s);
void     orc_box(const orc_sys* s, double* Lx, double* Ly, int* Nxcells, int* Nycells);
double   orc_time(const orc_sys* s);
int      orc_growing(const orc_sys* s);
void     orc_counters(const orc_sys* s, uint64_t* ncol, uint64_t* ncross,
                      uint64_t* nstale, uint64_t* npair, uint64_t* npred);
void     orc_state(const orc_sys* s, double* x, double* y, double* vx, double* vy,
                   double* tl, double* rad, double* m, int32_t* type, int32_t* cell,
                   uint64_t* coll);
/* physicalQ (EDMD.c:5968-6013): E, px, py */
void     orc_physicalq(const orc_sys* s, double* E, double* px, double* py);
/* collision virial accumulators collTermX,Y,XY,YX since the last reset */
void     orc_virial(orc_sys* s, double out[4], int reset);
/* g(r) histogram (pcf.c:61-120), counts then normalised */
int      orc_pcf(const orc_sys* s, double dr, double max_r, double* g, int nbins);
double   orc_vr(const orc_sys* s);
/* orc_run returns right after processing the growth-stop event (stopGrow,
 * src/EDMD.c:4740) when on != 0: the point where a growth start enters the
 * normal phase, as the engine's EDMD_F_STOP_AT_GROW */
void     orc_set_stop_at_grow(orc_sys* s, int on);
/* contact rule of systems created from now on: 0 = 2 sqrt(r1 r2) (the
 * reference's NONADDITIVE 0, EDMD.c:35-39), 1 = r1 + r2 (NONADDITIVE 1,
 * EDMD.c:40-42).  Returns the previous setting. */
int      orc_set_contact(int additive);
/* thermo rows (t Ncol E p px py pxy pyx a2), 9 doubles each; returns count */
int      orc_thermo_rows(const orc_sys* s, double* out, int cap);

/* MT19937 exposed for tests of the host-side init */
void     orc_mt_seed(uint32_t s);
uint32_t orc_mt_next(void);

#ifdef __cplusplus
}
#endif
#endif
