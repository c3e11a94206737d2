/*
 * edmd_oracle.c -- CPU oracle: serial restatement of the reference's
 * 2D hard-disk event loop (Syrocco/Graphical-EDMD, no-graphics build).
 *
 * TEST INFRASTRUCTURE ONLY (see edmd_oracle.h).  Every function follows a
 * reference routine and cites it as src/<file>:<line>.  The arithmetic is
 * written in the same operation order as the reference so that, compiled
 * with IEEE semantics (-O2 -fno-fast-math -ffp-contract=off), the event
 * sequence and the state are bit-identical to the reference's own C built
 * the same way.  The data structures are the reference's algorithms
 * (array doubly-linked cell list, bucket calendar of width 5/N feeding an
 * unbalanced BST with ties to the right) written over integer indices.
 */
#include "edmd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define NEVER 100000000000000000000000000.0   /* EDMD.h:8 */
#define NIL   (-1)

enum { EV_CROSS = 0, EV_COLL = 1, EV_SCREEN = 2, EV_THERMO = 3, EV_GROWSTOP = 9 };

/* ------------------------------------------------------------------ */
/* MT19937 (src/mersenne.c:68-81 init_genrand, 113-148 genrand_int32,  */
/* 185-189 genrand): the published Matsumoto-Nishimura generator.      */
/* ------------------------------------------------------------------ */
#define MT_N 624
#define MT_M 397
static uint32_t mt_s[MT_N];
static int      mt_i = MT_N + 1;

void orc_mt_seed(uint32_t s)
{
	mt_s[0] = s;
	for (mt_i = 1; mt_i < MT_N; mt_i++)
		mt_s[mt_i] = 1812433253u * (mt_s[mt_i - 1] ^ (mt_s[mt_i - 1] >> 30)) + (uint32_t)mt_i;
}

uint32_t orc_mt_next(void)
{
	uint32_t y;
	if (mt_i >= MT_N) {
		if (mt_i == MT_N + 1) orc_mt_seed(5489u);
		for (int k = 0; k < MT_N; k++) {
			y = (mt_s[k] & 0x80000000u) | (mt_s[(k + 1) % MT_N] & 0x7fffffffu);
			mt_s[k] = mt_s[(k + MT_M) % MT_N] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
		}
		mt_i = 0;
	}
	y = mt_s[mt_i++];
	y ^= (y >> 11);
	y ^= (y << 7) & 0x9d2c5680u;
	y ^= (y << 15) & 0xefc60000u;
	y ^= (y >> 18);
	return y;
}

/* genrand() (mersenne.c:185-189) and drand() (EDMD.c:5699-5701) */
static double genrand01(void) { return orc_mt_next() * (1.0 / 4294967296.0); }
static double drand_(double lo, double hi) { return (genrand01() * (hi - lo)) + lo; }

/* ------------------------------------------------------------------ */
/* system state                                                       */
/* ------------------------------------------------------------------ */
typedef struct ev_t {
	double   t;
	int32_t  i, j, q, type;
	uint64_t collActual;
	int32_t  lft, rgt, top;
} ev_t;

typedef struct thermo_row { double t, ncol, E, p, px, py, pxy, pyx, a2; } thermo_row;

struct orc_sys {
	int N;
	double Lx, Ly, halfLx, halfLy;
	int Nxc, Nyc;
	double cxs, cys, cxf, cyf;
	double dtPaul;
	double res, Einit;
	double tmax, dtime, dtimeThermo, firstScreen, firstThermo;
	double vr;
	int grow;               /* 1 while the Lubachevsky-Stillinger growth runs */
	int stop_at_grow;       /* orc_run returns right after the growth-stop event */
	int additive;           /* contact distance r1 + r2 instead of 2 sqrt(r1 r2) */
	/* disks */
	double *x, *y, *vx, *vy, *tl, *rad, *m, *vrd;
	int32_t *type, *cx, *cy, *prv, *nxt, *crossX, *crossY;
	uint64_t *coll;
	int32_t *head;
	/* events: [0,N) crossing, [N,2N) collision, 2N root, 2N+1 screen, 2N+3 thermo, 2N+5 growstop */
	ev_t *ev;
	int32_t *paul;          /* N+1 bucket heads */
	double paulTime;
	int actual;
	int root, treeMin;
	double t;
	uint64_t ncol, ncross, nstale, npair, npred;
	double collT[4];
	double lastScreen;
	thermo_row* rows; int nrows, caprows;
};

/* ------------------------------------------------------------------ */
/* periodic helpers (EDMD.c:5896-5959)                                 */
/* ------------------------------------------------------------------ */
static inline void pbc(const orc_sys* s, double* dx, double* dy)
{
	if (*dx >= s->halfLx) *dx -= s->Lx;
	else if (*dx < -s->halfLx) *dx += s->Lx;
	if (*dy >= s->halfLy) *dy -= s->Ly;
	else if (*dy < -s->halfLy) *dy += s->Ly;
}
static inline double pbc_in_x(const orc_sys* s, double d)
{
	if (d >= s->halfLx) return d - s->Lx;
	else if (d < -s->halfLx) return d + s->Lx;
	return d;
}
static inline double pbc_in_y(const orc_sys* s, double d)
{
	if (d >= s->halfLy) return d - s->Ly;
	else if (d < -s->halfLy) return d + s->Ly;
	return d;
}
static inline void pbc_post(const orc_sys* s, double* x, double* y)
{
	if (*x < 0) *x += s->Lx;
	else if (*x >= s->Lx) *x -= s->Lx;
	if (*y < 0) *y += s->Ly;
	else if (*y >= s->Ly) *y -= s->Ly;
}
static inline int pbc_cx(const orc_sys* s, int a) { return a < 0 ? a + s->Nxc : (a >= s->Nxc ? a - s->Nxc : a); }
static inline int pbc_cy(const orc_sys* s, int a) { return a < 0 ? a + s->Nyc : (a >= s->Nyc ? a - s->Nyc : a); }

/* ------------------------------------------------------------------ */
/* event queue: calendar + BST (EDMD.c:2144-2327)                     */
/* ------------------------------------------------------------------ */
static void tree_add(orc_sys* s, int e)                     /* addEventToTree 2175 */
{
	ev_t* E = s->ev;
	int w = s->root;
	for (;;) {
		if (E[e].t < E[w].t) {
			if (E[w].lft == NIL) { E[w].lft = e; break; }
			w = E[w].lft;
		} else {
			if (E[w].rgt == NIL) { E[w].rgt = e; break; }
			w = E[w].rgt;
		}
	}
	E[e].lft = NIL; E[e].rgt = NIL; E[e].top = w;
	if (s->treeMin == NIL || E[e].t < E[s->treeMin].t) s->treeMin = e;
}

static void queue_add(orc_sys* s, int e)                    /* addEventToQueue 2144 */
{
	ev_t* E = s->ev;
	double dt = E[e].t - s->paulTime;
	if (dt < s->dtPaul) {
		E[e].q = s->actual;
		tree_add(s, e);
	} else {
		int idx;
		if (dt >= s->dtPaul * s->N) idx = s->N;
		else {
			idx = s->actual + (int)(dt / s->dtPaul);
			if (idx >= s->N) idx -= s->N;
		}
		E[e].q = idx;
		E[e].lft = NIL;
		E[e].rgt = s->paul[idx];
		if (E[e].rgt != NIL) E[E[e].rgt].lft = e;
		s->paul[idx] = e;
	}
}

static void tree_remove(orc_sys* s, int e)                  /* removeEventFromTree 2228 */
{
	ev_t* E = s->ev;
	int top = E[e].top, n;
	if (e == s->treeMin) {
		if (E[e].rgt != NIL) {
			int m = E[e].rgt;
			while (E[m].lft != NIL) m = E[m].lft;
			s->treeMin = m;
		} else s->treeMin = (top == s->root) ? NIL : top;
	}
	if (E[e].lft == NIL && E[e].rgt == NIL) n = NIL;
	else if (E[e].lft == NIL) { n = E[e].rgt; E[n].top = top; }
	else if (E[e].rgt == NIL) { n = E[e].lft; E[n].top = top; }
	else {
		n = E[e].rgt;
		while (E[n].lft != NIL) n = E[n].lft;
		if (E[n].top != e) {
			E[E[n].top].lft = E[n].rgt;
			if (E[n].rgt != NIL) E[E[n].rgt].top = E[n].top;
			E[E[e].rgt].top = n;
			E[n].rgt = E[e].rgt;
		}
		E[E[e].lft].top = n;
		E[n].lft = E[e].lft;
		E[n].top = top;
	}
	if (E[top].lft == e) E[top].lft = n;
	else E[top].rgt = n;
}

static void queue_remove(orc_sys* s, int e)                 /* removeEventFromQueue 2209 */
{
	ev_t* E = s->ev;
	if (E[e].q != s->actual) {
		if (E[e].rgt != NIL) E[E[e].rgt].lft = E[e].lft;
		if (E[e].lft != NIL) E[E[e].lft].rgt = E[e].rgt;
		else s->paul[E[e].q] = E[e].rgt;
	} else tree_remove(s, e);
}

static void next_bucket(orc_sys* s)                         /* addNextPaulEvent 2287 */
{
	s->actual++;
	s->paulTime += s->dtPaul;
	if (s->actual == s->N) {
		s->actual = 0;
		int e = s->paul[s->N];
		s->paul[s->N] = NIL;
		while (e != NIL) { int n = s->ev[e].rgt; queue_add(s, e); e = n; }
	}
	int e = s->paul[s->actual];
	while (e != NIL) { int n = s->ev[e].rgt; tree_add(s, e); e = n; }
	s->paul[s->actual] = NIL;
}

static int next_event(orc_sys* s)                           /* findNextEvent 2313 */
{
	while (s->treeMin == NIL) next_bucket(s);
	return s->treeMin;
}

/* ------------------------------------------------------------------ */
/* cell list (EDMD.c:2053-2107)                                        */
/* ------------------------------------------------------------------ */
static void cell_add(orc_sys* s, int i)                     /* addToCell 2053 */
{
	int X = (int)(s->x[i] * s->cxf);
	int Y = (int)(s->y[i] * s->cyf);
	s->cx[i] = X; s->cy[i] = Y;
	s->prv[i] = NIL;
	s->nxt[i] = s->head[Y * s->Nxc + X];
	s->head[Y * s->Nxc + X] = i;
	if (s->nxt[i] != NIL) s->prv[s->nxt[i]] = i;
}
static void cell_remove(orc_sys* s, int i)                  /* removeFromCell 2083 */
{
	if (s->prv[i] == NIL) s->head[s->cy[i] * s->Nxc + s->cx[i]] = s->nxt[i];
	else s->nxt[s->prv[i]] = s->nxt[i];
	if (s->nxt[i] != NIL) s->prv[s->nxt[i]] = s->prv[i];
}

/* ------------------------------------------------------------------ */
/* free flight (EDMD.c:4954-5007)                                     */
/* ------------------------------------------------------------------ */
static void free_fly(orc_sys* s, int i)
{
	double dt = s->t - s->tl[i];
	s->tl[i] = s->t;
	s->x[i] += dt * s->vx[i];
	s->y[i] += dt * s->vy[i];
	if (s->grow) s->rad[i] += dt * s->vrd[i];               /* freeFlyGrow 4992 */
	pbc_post(s, &s->x[i], &s->y[i]);
}

/* ------------------------------------------------------------------ */
/* predictions                                                        */
/* ------------------------------------------------------------------ */
/* contact distance and its square, DIST / DIST2 (EDMD.c:35-43): the
 * reference's default NONADDITIVE 0 gives 2 sqrt(r1 r2); NONADDITIVE 1 gives
 * r1 + r2.  Same operation order as the macros. */
static int g_additive = 0;
int orc_set_contact(int additive)
{
	int old = g_additive;
	g_additive = additive != 0;
	return old;
}

static inline double contact(const orc_sys* s, double r1, double r2)
{
	return s->additive ? (r1) + (r2) : sqrt(4 * (r1) * (r2));
}

static inline double contact2(const orc_sys* s, double r1, double r2)
{
	return s->additive ? ((r1) + (r2)) * ((r1) + (r2)) : 4 * (r1) * (r2);
}

static double coll_time_normal(orc_sys* s, int a, int b)    /* collisionTimeNormal 2661 */
{
	s->npair++;
	double lat2 = s->t - s->tl[b];
	double dvx = s->vx[b] - s->vx[a];
	double dvy = s->vy[b] - s->vy[a];
	double dx = (s->x[b] + lat2 * s->vx[b]) - s->x[a];
	double dy = (s->y[b] + lat2 * s->vy[b]) - s->y[a];
	pbc(s, &dx, &dy);
	double bb = dx * dvx + dy * dvy;
	if (bb > 0) return NEVER;
	double v2 = dvx * dvx + dvy * dvy;
	double d2 = dx * dx + dy * dy - contact2(s, s->rad[a], s->rad[b]);
	double det = bb * bb - v2 * d2;
	if (d2 < -0.01) {
		fprintf(stderr, "oracle: overlap between %d and %d at t=%.17g\n", a, b, s->t);
		exit(3);
	}
	if (det < 0) return NEVER;
	return (-bb - sqrt(det)) / v2;
}

static double coll_time_grow(orc_sys* s, int a, int b)      /* collisionTimeGrow 2598 */
{
	s->npair++;
	double lat2 = s->t - s->tl[b];
	double dvx = s->vx[b] - s->vx[a];
	double dvy = s->vy[b] - s->vy[a];
	double dvr = s->vrd[a] + s->vrd[b];
	double dx = (s->x[b] + lat2 * s->vx[b]) - s->x[a];
	double dy = (s->y[b] + lat2 * s->vy[b]) - s->y[a];
	double dr = contact(s, s->rad[a], s->rad[b] + lat2 * s->vrd[b]);
	pbc(s, &dx, &dy);
	double bb = dx * dvx + dy * dvy - dvr * dr;
	double v2 = dvx * dvx + dvy * dvy;
	double d2 = dx * dx + dy * dy;
	double det = bb * bb - (v2 - dvr * dvr) * (d2 - dr * dr);
	if (det < 0) return NEVER;
	double plus = (-bb + sqrt(det)) / (v2 - dvr * dvr);
	double minus = (-bb - sqrt(det)) / (v2 - dvr * dvr);
	if (((minus > 0) && (plus > 0) && (minus < plus)) || ((minus > 0) && (plus < 0)))
		return minus;
	else if (((minus > 0) && (plus > 0.000000001) && (plus < minus)) || ((minus < 0) && (plus > 0.000000001)))
		return plus;
	if (d2 - dr * dr < -0.01) {
		fprintf(stderr, "oracle: overlap during growth between %d and %d\n", a, b);
		exit(3);
	}
	return NEVER;
}

static void add_collision(orc_sys* s, int i, int j, double tc)   /* addCollisionEvent 3286 */
{
	ev_t* e = &s->ev[s->N + i];
	e->j = j; e->type = EV_COLL; e->t = tc;
	e->collActual = s->coll[j];
	queue_add(s, s->N + i);
}

static void collision_event(orc_sys* s, int i)              /* collisionEventNormal 2829 / Grow 3104 */
{
	s->npred++;
	int partner = 0;
	double dt = s->grow ? 10000000 : NEVER;
	int X = s->cx[i], Y = s->cy[i];
	for (int jj = -1; jj <= 1; jj++)
		for (int kk = -1; kk <= 1; kk++) {
			int p2 = s->head[pbc_cy(s, Y + jj) * s->Nxc + pbc_cx(s, X + kk)];
			while (p2 != NIL) {
				if (p2 != i) {
					double d = s->grow ? coll_time_grow(s, i, p2) : coll_time_normal(s, i, p2);
					if (dt > d) { partner = p2; dt = d; }
				}
				p2 = s->nxt[p2];
			}
		}
	add_collision(s, i, partner, s->t + dt);
}

static void crossing_event(orc_sys* s, int i)               /* crossingEventNormal 2405 / Grow 2343 */
{
	double tx, ty; int xx, yy;
	if (s->vx[i] < 0) { tx = pbc_in_x(s, s->cx[i] * s->cxs - s->x[i]) / s->vx[i]; xx = 1; }
	else { tx = pbc_in_x(s, (1 + s->cx[i]) * s->cxs - s->x[i]) / s->vx[i]; xx = 2; }
	if (s->vy[i] < 0) { ty = pbc_in_y(s, s->cy[i] * s->cys - s->y[i]) / s->vy[i]; yy = 3; }
	else { ty = pbc_in_y(s, (1 + s->cy[i]) * s->cys - s->y[i]) / s->vy[i]; yy = 4; }
	ev_t* e = &s->ev[i];                                    /* addCrossingEvent 2487 */
	e->type = EV_CROSS;
	if (tx < ty) { e->j = xx; e->t = s->t + tx; }
	else { e->j = yy; e->t = s->t + ty; }
	queue_add(s, i);
}

/* ------------------------------------------------------------------ */
/* event handlers                                                     */
/* ------------------------------------------------------------------ */
static void do_crossing(orc_sys* s, int i, int dir)         /* doTheCrossing 2501 */
{
	free_fly(s, i);
	cell_remove(s, i);
	switch (dir) {
	case 1: if (s->cx[i] - 1 == -1) { s->cx[i] = s->Nxc - 1; s->crossX[i] -= 1; } else s->cx[i] -= 1; break;
	case 2: if (s->cx[i] + 1 == s->Nxc) { s->cx[i] = 0; s->crossX[i] += 1; } else s->cx[i] += 1; break;
	case 3: if (s->cy[i] - 1 == -1) { s->cy[i] = s->Nyc - 1; s->crossY[i] -= 1; } else s->cy[i] -= 1; break;
	case 4: if (s->cy[i] + 1 == s->Nyc) { s->cy[i] = 0; s->crossY[i] += 1; } else s->cy[i] += 1; break;
	}
	int c = s->cy[i] * s->Nxc + s->cx[i];
	s->prv[i] = NIL;
	s->nxt[i] = s->head[c];
	s->head[c] = i;
	if (s->nxt[i] != NIL) s->prv[s->nxt[i]] = i;
	crossing_event(s, i);
	queue_remove(s, s->N + i);
	collision_event(s, i);
}

static void do_collision(orc_sys* s, int i, int j, uint64_t collActual)  /* doTheCollisionNormal 3542 / Grow 3465 */
{
	free_fly(s, i);
	if (collActual != s->coll[j]) { s->nstale++; collision_event(s, i); return; }
	s->ncol++;
	free_fly(s, j);
	s->coll[i]++; s->coll[j]++;
	double dx = s->x[j] - s->x[i];
	double dy = s->y[j] - s->y[i];
	double dvx = s->vx[j] - s->vx[i];
	double dvy = s->vy[j] - s->vy[i];
	if (!s->grow) {                                         /* elastic branch 3802-3827 */
		double invMass = 1 / (s->m[i] + s->m[j]);
		pbc(s, &dx, &dy);
		double collKernel = invMass * (1 + s->res) * (dx * dvx + dy * dvy);
		double distSquared = contact2(s, s->rad[i], s->rad[j]);
		double f = collKernel / distSquared;
		double ct = s->m[i] * s->m[j] * f;
		s->collT[0] += ct * dx * dx;
		s->collT[1] += ct * dy * dy;
		s->collT[2] += ct * dx * dy;
		s->collT[3] += ct * dy * dx;
		s->vx[i] += f * s->m[j] * dx;
		s->vy[i] += f * s->m[j] * dy;
		s->vx[j] -= f * s->m[i] * dx;
		s->vy[j] -= f * s->m[i] * dy;
	} else {                                                /* growth rule 3479-3520 */
		double delta = 0.1 * 0;
		double res = 0.75 * 0 + 1;
		double dvr = s->vrd[i] + s->vrd[j];
		pbc(s, &dx, &dy);
		double dist = sqrt(dx * dx + dy * dy);
		double dxr = dx / dist, dyr = dy / dist;
		double invMass = 1 / (s->m[i] + s->m[j]);
		double collKernel = invMass * (1 + res) * (dxr * dvx + dyr * dvy - dvr);
		s->vx[i] += collKernel * s->m[j] * dxr - 2 * s->m[j] * invMass * delta * dxr;
		s->vy[i] += collKernel * s->m[j] * dyr - 2 * s->m[j] * invMass * delta * dyr;
		s->vx[j] -= collKernel * s->m[i] * dxr - 2 * s->m[i] * invMass * delta * dxr;
		s->vy[j] -= collKernel * s->m[i] * dyr - 2 * s->m[i] * invMass * delta * dyr;
	}
	queue_remove(s, i);
	queue_remove(s, j);
	crossing_event(s, i);
	crossing_event(s, j);
	queue_remove(s, s->N + j);
	collision_event(s, i);
	collision_event(s, j);
}

static void add_special(orc_sys* s, int slot, int type, double t)
{
	ev_t* e = &s->ev[slot];
	e->type = type; e->t = t; e->j = 0;
	queue_add(s, slot);
}

/* physicalQ (EDMD.c:5968-6013) */
void orc_physicalq(const orc_sys* s, double* E, double* px, double* py)
{
	double a = 0, b = 0, e = 0;
	for (int i = 0; i < s->N; i++) {
		a += s->vx[i] * s->m[i];
		b += s->vy[i] * s->m[i];
		double vx = s->vx[i];
		e += 0.5 * s->m[i] * (vx * vx + s->vy[i] * s->vy[i]);
	}
	*E = e; *px = a; *py = b;
}

static void normalize(orc_sys* s)                           /* normalizePhysicalQ 5723 */
{
	double E, px, py;
	orc_physicalq(s, &E, &px, &py);
	for (int i = 0; i < s->N; i++) {
		s->vx[i] -= px / (s->N * s->m[i]);
		s->vy[i] -= py / (s->N * s->m[i]);
	}
	orc_physicalq(s, &E, &px, &py);
	for (int i = 0; i < s->N; i++) {
		s->vx[i] /= sqrt(E / s->N / s->Einit);
		s->vy[i] /= sqrt(E / s->N / s->Einit);
	}
}

static void stop_grow(orc_sys* s)                           /* stopGrow 4740 */
{
	for (int i = 0; i < s->N; i++) {
		free_fly(s, i);
		s->coll[i] = 0;
		s->crossX[i] = 0; s->crossY[i] = 0;
	}
	s->ncol = 0; s->ncross = 0;
	s->grow = 0;
	normalize(s);
	for (int i = 0; i < s->N; i++) {
		s->coll[i]++;
		queue_remove(s, s->N + i);
		collision_event(s, i);
		queue_remove(s, i);
		crossing_event(s, i);
	}
}

static void take_thermo(orc_sys* s)                         /* takeAThermo 4679 + saveThermo 5232 */
{
	double E, px, py;
	orc_physicalq(s, &E, &px, &py);
	double area = s->Lx * s->Ly;
	double dT = s->t - s->lastScreen;
	s->lastScreen = s->t;
	double eX = 0, eY = 0, eXY = 0, eYX = 0;
	for (int i = 0; i < s->N; i++) {
		double vx = s->vx[i], vy = s->vy[i];
		eX += s->m[i] * vx * vx; eY += s->m[i] * vy * vy;
		eXY += s->m[i] * vx * vy; eYX += s->m[i] * vy * vx;
	}
	thermo_row r;
	r.t = s->t; r.ncol = (double)s->ncol; r.E = E / s->N;
	r.px = -1 * s->collT[0] / (area * dT) + eX / area;
	r.py = -1 * s->collT[1] / (area * dT) + eY / area;
	r.pxy = -1 * s->collT[2] / (area * dT) + eXY / area;
	r.pyx = -1 * s->collT[3] / (area * dT) + eYX / area;
	r.p = (-1 / (dT)) * (s->collT[0] + s->collT[1]) / (2 * area) + E / area;
	s->collT[0] = s->collT[1] = s->collT[2] = s->collT[3] = 0;
	double vxa = 0;
	for (int i = 0; i < s->N; i++) vxa += s->vx[i];
	vxa /= s->N;
	double v2 = 0, v4 = 0;
	for (int i = 0; i < s->N; i++) { double d = s->vx[i] - vxa; double d2 = d * d; v2 += d2; v4 += d2 * d2; }
	v2 /= s->N; v4 /= s->N;
	r.a2 = (v2 > 0.0) ? v4 / (3.0 * v2 * v2) - 1.0 : 0.0;
	if (s->t != 0) {
		if (s->nrows == s->caprows) {
			s->caprows = s->caprows ? 2 * s->caprows : 64;
			s->rows = (thermo_row*)realloc(s->rows, s->caprows * sizeof(thermo_row));
		}
		s->rows[s->nrows++] = r;
	}
}

/* ------------------------------------------------------------------ */
/* construction                                                       */
/* ------------------------------------------------------------------ */
void orc_default_params(orc_params* p)
{
	memset(p, 0, sizeof(*p));
	p->N = 500; p->phi = 0.38; p->xs = 0.3; p->q = 0.4; p->aspect = 1.0;
	p->Einit = 1; p->res = 1; p->tmax = 4000; p->dtime = 100; p->dtimeThermo = 100;
	p->firstScreen = 1; p->firstThermo = 1000; p->seed = 1; p->start = ORC_START_HEX;
}

static orc_sys* alloc_sys(int N)
{
	orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
	s->N = N;
	s->additive = g_additive;
#define A(f, T) s->f = (T*)calloc((size_t)N, sizeof(T))
	A(x, double); A(y, double); A(vx, double); A(vy, double); A(tl, double);
	A(rad, double); A(m, double); A(vrd, double);
	A(type, int32_t); A(cx, int32_t); A(cy, int32_t); A(prv, int32_t); A(nxt, int32_t);
	A(crossX, int32_t); A(crossY, int32_t); A(coll, uint64_t);
#undef A
	s->ev = (ev_t*)calloc((size_t)(2 * N + 10), sizeof(ev_t));
	s->paul = (int32_t*)malloc((size_t)(N + 1) * sizeof(int32_t));
	for (int k = 0; k <= N; k++) s->paul[k] = NIL;
	return s;
}

static void box_helper(orc_sys* s)                          /* boxConstantHelper 679 */
{
	s->halfLx = s->Lx / 2; s->halfLy = s->Ly / 2;
	s->Nyc = (int)(s->halfLy); s->Nxc = (int)(s->halfLx);
	s->cxs = s->Lx / s->Nxc; s->cys = s->Ly / s->Nyc;
	s->cxf = 1 / s->cxs; s->cyf = 1 / s->cys;
	s->dtPaul = 5.0 / (double)s->N;
}

static void lists_and_events(orc_sys* s)                    /* cellListInit 1906 + eventListInit 1935 */
{
	int N = s->N;
	s->head = (int32_t*)malloc((size_t)s->Nxc * s->Nyc * sizeof(int32_t));
	for (int c = 0; c < s->Nxc * s->Nyc; c++) s->head[c] = NIL;
	for (int i = 0; i < N; i++) { s->nxt[i] = NIL; s->prv[i] = NIL; cell_add(s, i); }
	for (int k = 0; k < 2 * N + 10; k++) { s->ev[k].lft = s->ev[k].rgt = s->ev[k].top = NIL; }
	s->root = 2 * N;
	s->ev[s->root].t = NEVER + 1;
	s->treeMin = NIL;
	if (s->grow) {
		double inv = 1 / s->vr;
		if (s->firstScreen < inv) s->firstScreen = inv + s->firstScreen;
		if (s->firstThermo < inv) s->firstThermo = inv + s->firstThermo;
	}
	add_special(s, 2 * N + 3, EV_THERMO, s->firstThermo + 0.000000001);
	if (s->grow) {
		s->tmax += 1 / s->vr;
		add_special(s, 2 * N + 5, EV_GROWSTOP, 1 / s->vr);
	}
	add_special(s, 2 * N + 1, EV_SCREEN, s->firstScreen);
	for (int i = 0; i < N; i++) {
		s->ev[i].i = i; s->ev[N + i].i = i;
		crossing_event(s, i);
		collision_event(s, i);
	}
}

orc_sys* orc_create(const orc_params* p)
{
	int N = p->N;
	double Lx, Ly;
	int Nx = 0, Ny = 0;
	orc_mt_seed(p->seed);                                   /* -v: init_genrand(version), EDMD.c:903-906 */
	if (p->start == ORC_START_HEX) {                        /* constantInit Hex branch 1024-1049 */
		Ny = sqrt(N) * p->aspect;
		if (Ny % 2 == 1) Ny += 1;
		Nx = N / Ny;
		N = Nx * Ny;
		Ly = sqrt(sqrt(3) / 2 * Ny / Nx * M_PI * N / p->phi);
		Lx = 2 / sqrt(3) * Nx / Ny * Ly;
	} else {                                                /* default branch 1107-1166 */
		double r2 = (1 + p->xs * (p->q * p->q - 1));
		Lx = sqrt(M_PI * N / (p->phi * p->aspect) * r2);
		Ly = Lx * p->aspect;
	}
	orc_sys* s = alloc_sys(N);
	s->Lx = Lx; s->Ly = Ly;
	s->res = p->res; s->Einit = p->Einit; s->tmax = p->tmax;
	s->dtime = p->dtime; s->dtimeThermo = p->dtimeThermo;
	s->firstScreen = p->firstScreen; s->firstThermo = p->firstThermo;
	box_helper(s);
	if (p->start == ORC_START_HEX) {                        /* particlesInit Hex 1582-1637 */
		int k = 0;
		double dx = Lx / Nx, dy = Ly / Ny;
		for (int i = 0; i < Nx; i++)
			for (int j = 0; j < Ny; j++) {
				s->x[k] = i * dx + (j % 2) * (dx / 2);
				s->y[k] = j * dy;
				s->type[k] = 1; s->rad[k] = 1; s->m[k] = 1;
				double U1 = drand_(0, 1), U2 = drand_(0, 1);
				s->vx[k] = sqrt(-2 * log(U1) / s->m[k] * s->Einit) * cos(2 * M_PI * U2);
				s->vy[k] = sqrt(-2 * log(U1) / s->m[k] * s->Einit) * sin(2 * M_PI * U2);
				k++;
			}
		normalize(s);
		s->grow = 0;
	} else {                                                /* particlesInit default 1690-1829 */
		double EinitGrow = 0.05;
		double vr;                                          /* optimizeGrowConstant 5766 */
		if (p->phi < 0.8) vr = 0.1; else vr = 0.1 * pow(0.8 / p->phi, 30);
		if (p->phi > 0.7) vr /= 8;
		s->vr = vr;
		int Nsmall = (int)(N * p->xs), Nbig = N - Nsmall;
		for (int i = 0; i < N; i++) {
			s->x[i] = drand_(0, Lx);
			s->y[i] = drand_(0, Ly);
			s->rad[i] = 0;
			if (i < Nbig) { s->type[i] = 1; s->m[i] = 1; s->vrd[i] = vr; }
			else { s->type[i] = 0; s->m[i] = pow(p->q, 3); s->m[i] = 1; s->vrd[i] = vr * p->q; }
			double U1 = drand_(0, 1), U2 = drand_(0, 1);
			s->vx[i] = sqrt(-2 * log(U1) / s->m[i] * EinitGrow) * cos(2 * M_PI * U2);
			s->vy[i] = sqrt(-2 * log(U1) / s->m[i] * EinitGrow) * sin(2 * M_PI * U2);
			(void)drand_(0, 1);                             /* charge draw, consumed */
		}
		s->grow = 1;
	}
	lists_and_events(s);
	return s;
}

orc_sys* orc_create_from_arrays(int N, double Lx, double Ly,
                                const double* x, const double* y,
                                const double* vx, const double* vy,
                                const double* rad, const double* m,
                                const int32_t* type, double res,
                                double firstScreen, double dtime,
                                double firstThermo, double dtimeThermo)
{
	orc_sys* s = alloc_sys(N);
	s->Lx = Lx; s->Ly = Ly; s->res = res; s->Einit = 1; s->tmax = 1e300;
	s->dtime = dtime; s->dtimeThermo = dtimeThermo;
	s->firstScreen = firstScreen; s->firstThermo = firstThermo;
	box_helper(s);
	memcpy(s->x, x, N * sizeof(double)); memcpy(s->y, y, N * sizeof(double));
	memcpy(s->vx, vx, N * sizeof(double)); memcpy(s->vy, vy, N * sizeof(double));
	memcpy(s->rad, rad, N * sizeof(double)); memcpy(s->m, m, N * sizeof(double));
	memcpy(s->type, type, N * sizeof(int32_t));
	s->grow = 0;
	lists_and_events(s);
	return s;
}

void orc_destroy(orc_sys* s)
{
	if (!s) return;
	free(s->x); free(s->y); free(s->vx); free(s->vy); free(s->tl); free(s->rad); free(s->m); free(s->vrd);
	free(s->type); free(s->cx); free(s->cy); free(s->prv); free(s->nxt); free(s->crossX); free(s->crossY);
	free(s->coll); free(s->head); free(s->ev); free(s->paul); free(s->rows);
	free(s);
}

/* ------------------------------------------------------------------ */
/* main loop (EDMD.c:523-618)                                         */
/* ------------------------------------------------------------------ */
int64_t orc_run(orc_sys* s, int64_t max_coll, double t_stop,
                orc_coll* co, int64_t ccap, orc_event* eo, int64_t ecap, int64_t* nev)
{
	int64_t logged = 0, ne = 0;
	while (s->t <= s->tmax && logged < max_coll) {
		int e = next_event(s);
		ev_t* E = &s->ev[e];
		if (E->t >= t_stop) break;
		s->t = E->t;
		queue_remove(s, e);
		int stale = 0;
		if (E->type == EV_COLL) {
			stale = (E->collActual != s->coll[E->j]);
			if (!stale) {
				if (co && logged < ccap) {
					co[logged].i = E->i; co[logged].j = E->j;
					co[logged].ci = s->cy[E->i] * s->Nxc + s->cx[E->i];
					co[logged].cj = s->cy[E->j] * s->Nxc + s->cx[E->j];
					co[logged].t = s->t;
				}
				logged++;
			}
		}
		if (eo && ne < ecap) {
			eo[ne].type = E->type; eo[ne].i = E->i; eo[ne].j = E->j;
			eo[ne].stale = stale; eo[ne].t = s->t;
		}
		ne++;
		switch (E->type) {
		case EV_COLL: do_collision(s, E->i, E->j, E->collActual); break;
		case EV_CROSS: s->ncross++; do_crossing(s, E->i, E->j); break;
		case EV_SCREEN:                                     /* takeAScreenshot 4657 */
			for (int i = 0; i < s->N; i++) free_fly(s, i);
			add_special(s, 2 * s->N + 1, EV_SCREEN, s->t + s->dtime);
			break;
		case EV_THERMO:
			take_thermo(s);
			add_special(s, 2 * s->N + 3, EV_THERMO, s->t + s->dtimeThermo);
			break;
		case EV_GROWSTOP: stop_grow(s); break;
		}
		if (E->type == EV_GROWSTOP && s->stop_at_grow) break;
	}
	if (nev) *nev = ne;
	return logged;
}

void orc_set_stop_at_grow(orc_sys* s, int on) { s->stop_at_grow = on; }

void orc_sync_all(orc_sys* s) { for (int i = 0; i < s->N; i++) free_fly(s, i); }

int    orc_N(const orc_sys* s) { return s->N; }
double orc_time(const orc_sys* s) { return s->t; }
int    orc_growing(const orc_sys* s) { return s->grow; }
double orc_vr(const orc_sys* s) { return s->vr; }
void   orc_box(const orc_sys* s, double* Lx, double* Ly, int* nx, int* ny)
{
	*Lx = s->Lx; *Ly = s->Ly; *nx = s->Nxc; *ny = s->Nyc;
}
void orc_counters(const orc_sys* s, uint64_t* ncol, uint64_t* ncross, uint64_t* nstale,
                  uint64_t* npair, uint64_t* npred)
{
	*ncol = s->ncol; *ncross = s->ncross; *nstale = s->nstale; *npair = s->npair; *npred = s->npred;
}
void orc_state(const orc_sys* s, double* x, double* y, double* vx, double* vy, double* tl,
               double* rad, double* m, int32_t* type, int32_t* cell, uint64_t* coll)
{
	for (int i = 0; i < s->N; i++) {
		if (x) x[i] = s->x[i];
		if (y) y[i] = s->y[i];
		if (vx) vx[i] = s->vx[i];
		if (vy) vy[i] = s->vy[i];
		if (tl) tl[i] = s->tl[i];
		if (rad) rad[i] = s->rad[i];
		if (m) m[i] = s->m[i];
		if (type) type[i] = s->type[i];
		if (cell) cell[i] = s->cy[i] * s->Nxc + s->cx[i];
		if (coll) coll[i] = s->coll[i];
	}
}
void orc_virial(orc_sys* s, double out[4], int reset)
{
	for (int k = 0; k < 4; k++) { out[k] = s->collT[k]; if (reset) s->collT[k] = 0; }
}
int orc_thermo_rows(const orc_sys* s, double* out, int cap)
{
	int n = s->nrows < cap ? s->nrows : cap;
	for (int r = 0; r < n; r++) memcpy(out + 9 * r, &s->rows[r], 9 * sizeof(double));
	return s->nrows;
}

/* g(r) (pcf.c:61-120): O(N^2) histogram with dr bins up to max_r,
 * normalised by 2*pi*r*dr * rho * N with r at the bin centre. */
int orc_pcf(const orc_sys* s, double dr, double max_r, double* g, int nbins)
{
	int nb = (int)(max_r / dr);
	if (nb > nbins) nb = nbins;
	for (int b = 0; b < nb; b++) g[b] = 0;
	for (int i = 0; i < s->N; i++)
		for (int j = 0; j < s->N; j++) {
			if (i == j) continue;
			double dx = s->x[j] - s->x[i], dy = s->y[j] - s->y[i];
			pbc(s, &dx, &dy);
			double r = sqrt(dx * dx + dy * dy);
			if (r < max_r) { int b = (int)(r / dr); if (b >= 0 && b < nb) g[b] += 1.0; }
		}
	double rho = s->N / (s->Lx * s->Ly);
	for (int b = 0; b < nb; b++) {
		double r = (b + 0.5) * dr;
		double norm = 2 * M_PI * r * dr * rho * s->N;
		g[b] = norm > 0 ? g[b] / norm : 0.0;
	}
	return nb;
}
