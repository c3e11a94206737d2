/*
 * edmd_main.c -- drop-in command-line driver of the GB300 hard-disk engine.
 *
 * Keeps the no-graphics reference's command line and output files
 * (src/EDMD.c main 498-661, constantInit 745-1219, customName 6015-6116,
 * saveTXT 5012-5153, saveThermo 5232-5697) and replaces its event loop with
 * the GPU engine behind include/edmd_gpu.h.  Screenshots (ovito/LAMMPS text
 * dumps) and thermo rows are written exactly as the reference writes them.
 *
 * Reference options kept: -N/--number, -p/--phi, -x/--xs, -q/--sizeratio,
 * -a/--aspect, -t/--time, -D/--dt, -o/--dtimeThermo, -E/--initial-energy,
 * -r/--res, -v/--version (seed and file version), -l/--load (.txt or a dump
 * ending in 'p').  Added: --hex (triangular-lattice start, the reference's
 * Hex = 1 global), --max-coll n (stop after n accepted collisions),
 * --quiet, --additive (contact distance r1 + r2: the reference built with
 * NONADDITIVE 1, src/EDMD.c:35-43), --engine auto|warp|round.
 *
 * Engines.  "warp" runs every phase in the serial-exact engine, which makes
 * the thermo rows itself.  "round" runs the growth phase there and the
 * constant-radius phase in the round-parallel engine (edmd_advance_rounds,
 * exact mode), which stops at each screenshot and thermo time; the rows are
 * then computed here from the state and the collision virial with the same
 * operations in the same order.  Positions, velocities, collision counts and
 * dump files are the same as the serial engine's; the virial sums of a round
 * are added in another order, so a pressure term can differ in its last
 * bits (about 1e-16 relative), far below the printed digits.  Past tmax the
 * round call may process a few more disk events than the serial loop's one
 * (no file records them; only the final counters printed to stdout see
 * them).  "auto" takes rounds from ROUND_MIN_N disks.
 */
#include "../../include/edmd_gpu.h"
#include "../../include/edmd_host.h"

#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

typedef struct {
	int N; double phi, xs, q, aspect, tmax, dtime, dtimeThermo, Einit, res;
	unsigned seed; int version; int hex; int load; char loadfile[512];
	long long max_coll; int quiet; int additive; int engine;
} opts;

enum { ENG_AUTO = 0, ENG_WARP = 1, ENG_ROUND = 2 };
/* --engine auto runs the constant-radius phase in rounds from this many disks */
#define ROUND_MIN_N 1000
/* window radius of the rounds: 3 up to this many disks (measured ~1.5x the
 * collisions a round of 4 gives, no replays), 4 above (larger systems gain
 * nothing from 3, and its rarer causality violations replay whole calls) */
#define ROUND_R3_MAX_N 20000

static void die(const char* m, edmd_ctx* c)
{
	fprintf(stderr, "edmd: %s%s%s\n", m, c ? ": " : "", c ? edmd_last_error(c) : "");
	exit(3);
}

/* -l file.txt: "N Lx [Ly]" then "type x y rad m" per disk, velocities drawn
 * (src/EDMD.c:979-986, 1366-1386) */
static int load_txt(const char* fn, opts* o, double** arr, int32_t** type, double* Lx, double* Ly)
{
	FILE* f = fopen(fn, "r");
	if (!f) return -1;
	char buf[256];
	do { if (!fgets(buf, sizeof buf, f)) { fclose(f); return -1; } } while (buf[0] == '#');
	int N; double a, b;
	int nv = sscanf(buf, "%d %lf %lf", &N, &a, &b);
	if (nv < 2) { fclose(f); return -1; }
	*Lx = a; *Ly = nv == 2 ? a : b;
	for (int k = 0; k < 6; k++) arr[k] = calloc(N, sizeof(double));
	*type = calloc(N, sizeof(int32_t));
	for (int i = 0; i < N; i++) {
		do { if (!fgets(buf, sizeof buf, f)) { fclose(f); return -1; } } while (buf[0] == '#');
		int t;
		sscanf(buf, "%d %lf %lf %lf %lf", &t, &arr[0][i], &arr[1][i], &arr[4][i], &arr[5][i]);
		(*type)[i] = t;
		double U1 = edmd_mt_double(), U2 = edmd_mt_double();
		arr[2][i] = sqrt(-2 * log(U1) / arr[5][i] * o->Einit) * cos(2 * M_PI * U2);
		arr[3][i] = sqrt(-2 * log(U1) / arr[5][i] * o->Einit) * sin(2 * M_PI * U2);
	}
	fclose(f);
	edmd_normalize(N, o->Einit, arr[5], arr[2], arr[3]);
	return N;
}

/* -l file.dump: last frame of a LAMMPS text dump, velocities kept
 * (src/EDMD.c:987-995, 1387-1451 via parser.c) */
static int load_dump(const char* fn, double** arr, int32_t** type, double* Lx, double* Ly)
{
	FILE* f = fopen(fn, "r");
	if (!f) return -1;
	char line[1024];
	long last = -1, pos = 0;
	while (fgets(line, sizeof line, f)) {
		if (strncmp(line, "ITEM: TIMESTEP", 14) == 0) last = pos;
		pos = ftell(f);
	}
	if (last < 0) { fclose(f); return -1; }
	fseek(f, last, SEEK_SET);
	int N = 0;
	double lo, hi;
	int col[8] = {-1, -1, -1, -1, -1, -1, -1, -1};   /* x y vx vy radius m type id */
	while (fgets(line, sizeof line, f)) {
		if (strncmp(line, "ITEM: NUMBER OF ATOMS", 21) == 0) {
			if (!fgets(line, sizeof line, f)) break;
			N = atoi(line);
		} else if (strncmp(line, "ITEM: BOX BOUNDS", 16) == 0) {
			if (!fgets(line, sizeof line, f)) break;
			sscanf(line, "%lf %lf", &lo, &hi); *Lx = hi - lo;
			if (!fgets(line, sizeof line, f)) break;
			sscanf(line, "%lf %lf", &lo, &hi); *Ly = hi - lo;
		} else if (strncmp(line, "ITEM: ATOMS", 11) == 0) {
			const char* names[8] = {"x", "y", "vx", "vy", "radius", "m", "type", "id"};
			char* tok = strtok(line + 11, " \n");
			int k = 0;
			while (tok) {
				for (int c = 0; c < 8; c++) if (strcmp(tok, names[c]) == 0) col[c] = k;
				k++;
				tok = strtok(NULL, " \n");
			}
			break;
		}
	}
	if (N <= 0 || col[0] < 0 || col[1] < 0) { fclose(f); return -1; }
	for (int k = 0; k < 6; k++) arr[k] = calloc(N, sizeof(double));
	*type = calloc(N, sizeof(int32_t));
	for (int r = 0; r < N; r++) {
		if (!fgets(line, sizeof line, f)) { fclose(f); return -1; }
		double v[32]; int nv = 0;
		char* tok = strtok(line, " \n");
		while (tok && nv < 32) { v[nv++] = atof(tok); tok = strtok(NULL, " \n"); }
		int i = col[7] >= 0 ? (int)v[col[7]] : r;
		if (i < 0 || i >= N) i = r;
		double x = v[col[0]], y = v[col[1]];
		if (x < 0) x += *Lx; else if (x >= *Lx) x -= *Lx;     /* PBCpostX/Y, 1405-1406 */
		if (y < 0) y += *Ly; else if (y >= *Ly) y -= *Ly;
		arr[0][i] = x; arr[1][i] = y;
		arr[2][i] = col[2] >= 0 ? v[col[2]] : 0; arr[3][i] = col[3] >= 0 ? v[col[3]] : 0;
		arr[4][i] = col[4] >= 0 ? v[col[4]] : 1; arr[5][i] = col[5] >= 0 ? v[col[5]] : 1;
		(*type)[i] = col[6] >= 0 ? (int)v[col[6]] : 1;
	}
	fclose(f);
	return N;
}

/* one saveThermo row (EDMD.c:5409-5577 with Nthermo = 1) */
static void put_row(FILE* f, const double* r)
{
	fprintf(f, "%lf ", r[0]);
	fprintf(f, "%ld ", (long)r[1]);
	fprintf(f, "%lf ", r[2]);
	fprintf(f, "%lf %lf %lf %.10lf %.10lf ", r[3], r[4], r[5], r[6], r[7]);
	fprintf(f, "%lf ", r[8]);
	fprintf(f, "\n");
}

/* one frame of saveTXT (EDMD.c:5012-5153), as takeAScreenshot writes it */
static void put_frame(FILE* f, double t, int N, double Lx, double Ly, const int32_t* type, const double* x,
                      const double* y, const double* vx, const double* vy, const double* rad, const double* m)
{
	fprintf(f, "ITEM: TIMESTEP\n%lf\nITEM: NUMBER OF ATOMS\n%d\nITEM: BOX BOUNDS pp pp pp\n"
	           "0 %lf\n0 %lf\n0 0\nITEM: ATOMS id type x y vx vy radius m coll", t, N, Lx, Ly);
	fprintf(f, "\n");
	for (int i = 0; i < N; i++) {
		fprintf(f, "%d %d %.3lf %lf %lf %lf %lf %lf %d", i, type[i], x[i], y[i], vx[i], vy[i], rad[i], m[i], type[i]);
		fprintf(f, "\n");
	}
	fflush(f);
}

/* takeAThermo + physicalQ + saveThermo (EDMD.c:4679-4705, 5968-6013,
 * 5232-5697 with Nthermo = 1) at time t: the operations of the serial
 * engines' in-kernel rows, in the same order (sums over disks in index
 * order).  collT holds collTermX, Y, XY, YX since the previous row; *last is
 * lastScreen, the time of the previous row (0 before the first). */
static void thermo_row(double* row, double t, double* last, uint64_t ncol, int N, double Lx, double Ly,
                       const double* vx, const double* vy, const double* m, const double collT[4])
{
	double E = 0;
	for (int i = 0; i < N; i++) {
		double v = vx[i];
		E += 0.5 * m[i] * (v * v + vy[i] * vy[i]);
	}
	double area = Lx * Ly;
	double dT = t - *last;
	*last = t;
	double e4[4] = {0, 0, 0, 0};
	for (int i = 0; i < N; i++) {
		e4[0] += m[i] * vx[i] * vx[i];
		e4[1] += m[i] * vy[i] * vy[i];
		e4[2] += m[i] * vx[i] * vy[i];
		e4[3] += m[i] * vy[i] * vx[i];
	}
	row[0] = t;
	row[1] = (double)ncol;
	row[2] = E / N;
	for (int k = 0; k < 4; k++) row[4 + k] = -1 * collT[k] / (area * dT) + e4[k] / area;
	row[3] = (-1 / (dT)) * (collT[0] + collT[1]) / (2 * area) + E / area;
	double vxa = 0;
	for (int i = 0; i < N; i++) vxa += vx[i];
	vxa /= N;
	double v2 = 0, v4 = 0;
	for (int i = 0; i < N; i++) {
		double dd = vx[i] - vxa;
		double d2 = dd * dd;
		v2 += d2;
		v4 += d2 * d2;
	}
	v2 /= N;
	v4 /= N;
	row[8] = (v2 > 0.0) ? v4 / (3.0 * v2 * v2) - 1.0 : 0.0;
}

/* The constant-radius phase in the round-parallel engine: advance to each
 * screenshot or thermo time in turn (screenshot times firstScreen + k dtime,
 * thermo times firstThermo + 1e-9 + k dtimeThermo, accumulated by repeated
 * addition as addEventThermo / takeAScreenshot do) and write the frame or
 * the row there.  The serial loop ends after the first event later than
 * tmax; when that event is a screenshot or thermo event, its frame or row
 * is written here too. */
static edmd_counters round_phase(edmd_ctx* ctx, const edmd_system_desc* d, const opts* o, int N, double Lx,
                                 double Ly, const int32_t* type, long long coll_left, uint64_t ncol_seen,
                                 FILE* dump, FILE* thermo, double* sx, double* sy, double* svx, double* svy,
                                 double* srad, double* sm)
{
	double ts = d->first_screen, tt = d->first_thermo + 0.000000001, last_th = 0;
	double tend = nextafter(d->tmax, INFINITY);
	const int32_t radius = N <= ROUND_R3_MAX_N ? 3 : 4;
	edmd_counters cnt;
	for (;;) {
		int th = tt < ts;                               /* the thermo time comes first */
		double tb = th ? tt : nextafter(ts, INFINITY);  /* a screenshot is passed, then the call stops */
		int64_t nr = 0, nv = 0;
		int last = tb > tend;
		/* after tmax: finish the events at or before it; the first event
		 * after it is the loop's last (while (t <= tmax), EDMD.c:523) */
		int rc = edmd_advance_rounds(ctx, coll_left, last ? tend : tb, EDMD_F_EXACT, radius, (int64_t)1 << 60, NULL,
		                             &nr, &nv);
		if (rc != EDMD_OK) die("round advance failed", ctx);
		edmd_get_counters(ctx, 0, &cnt);
		coll_left -= (long long)(cnt.ncol_total - ncol_seen);
		ncol_seen = cnt.ncol_total;
		if (cnt.stop_reason == EDMD_STOP_COLL || coll_left <= 0) break;
		if (last) {
			/* is the barrier that first event?  Only if no disk event comes before it */
			uint64_t ev0 = cnt.ncol + cnt.ncross + cnt.nstale;
			rc = edmd_advance_rounds(ctx, coll_left, tb, EDMD_F_EXACT, radius, (int64_t)1 << 60, NULL, &nr, &nv);
			if (rc != EDMD_OK) die("round advance failed", ctx);
			edmd_get_counters(ctx, 0, &cnt);
			if (cnt.ncol + cnt.ncross + cnt.nstale != ev0) break;
		}
		if (th) {
			double collT[4], row[9];
			edmd_get_state(ctx, 0, NULL, NULL, svx, svy, NULL, sm, NULL, NULL);
			edmd_get_virial(ctx, 0, collT, 1);
			thermo_row(row, tt, &last_th, cnt.ncol, N, Lx, Ly, svx, svy, sm, collT);
			put_row(thermo, row);
			fflush(thermo);
			tt = tt + o->dtimeThermo;
		} else {
			edmd_get_state(ctx, 0, sx, sy, svx, svy, srad, sm, NULL, NULL);
			put_frame(dump, ts, N, Lx, Ly, type, sx, sy, svx, svy, srad, sm);
			if (!o->quiet) printf("\rt = %.2e / %.2e  ncol = %.2e", ts, o->tmax, (double)cnt.ncol);
			ts = ts + o->dtime;
		}
		if (last) break;
	}
	return cnt;
}

int main(int argc, char* argv[])
{
	opts o = {500, 0.38, 0.3, 0.4, 1.0, 4000, 100, 100, 1, 1, 0, 1, 0, 0, "", -1, 0, 0, ENG_AUTO};
	int seeded = 0;
	static struct option lo[] = {
		{"load", 1, 0, 'l'}, {"number", 1, 0, 'N'}, {"phi", 1, 0, 'p'}, {"res", 1, 0, 'r'},
		{"time", 1, 0, 't'}, {"dt", 1, 0, 'D'}, {"initial-energy", 1, 0, 'E'}, {"xs", 1, 0, 'x'},
		{"sizeratio", 1, 0, 'q'}, {"aspect", 1, 0, 'a'}, {"dtimeThermo", 1, 0, 'o'},
		{"version", 1, 0, 'v'}, {"hex", 0, 0, 1000}, {"max-coll", 1, 0, 1001}, {"quiet", 0, 0, 1002},
		{"additive", 0, 0, 1003}, {"engine", 1, 0, 1004}, {0, 0, 0, 0}};
	int c;
	while ((c = getopt_long(argc, argv, "l:N:p:r:t:D:E:x:q:a:o:v:", lo, NULL)) != -1) {
		switch (c) {
		case 'l': {
			snprintf(o.loadfile, sizeof o.loadfile, "%s", optarg);
			size_t n = strlen(o.loadfile);
			o.load = (n > 0 && o.loadfile[n - 1] == 'p') ? 2 : 1;
			break;
		}
		case 'N': o.load = 0; o.N = atoi(optarg); break;
		case 'p': o.load = 0; o.phi = atof(optarg); break;
		case 'x': o.load = 0; o.xs = atof(optarg); break;
		case 'a': o.load = 0; o.aspect = atof(optarg); break;
		case 'q': o.load = 0; o.q = atof(optarg); break;
		case 'r': o.res = atof(optarg); break;
		case 't': o.tmax = atof(optarg); break;
		case 'D': o.dtime = atof(optarg); break;
		case 'E': o.Einit = atof(optarg); break;
		case 'o': o.dtimeThermo = atof(optarg); break;
		case 'v': o.version = atoi(optarg); o.seed = (unsigned)o.version; seeded = 1; break;
		case 1000: o.hex = 1; break;
		case 1001: o.max_coll = atoll(optarg); break;
		case 1002: o.quiet = 1; break;
		case 1003: o.additive = 1; break;
		case 1004:
			if (strcmp(optarg, "auto") == 0) o.engine = ENG_AUTO;
			else if (strcmp(optarg, "warp") == 0) o.engine = ENG_WARP;
			else if (strcmp(optarg, "round") == 0) o.engine = ENG_ROUND;
			else { fprintf(stderr, "edmd: --engine auto|warp|round\n"); return 1; }
			break;
		default: fprintf(stderr, "edmd: unknown option\n"); return 1;
		}
	}
	if (!seeded) o.seed = (unsigned)time(NULL);            /* init_genrand(time(NULL)), EDMD.c:500 */
	edmd_mt_seed(o.seed);

	/* ---- constantInit + particlesInit on the host */
	int N = o.N, Nsmall = 0;
	double Lx = 0, Ly = 0, vr_base = 0;
	double* a[7] = {0};
	int32_t* type = NULL;
	if (o.load == 1) {
		N = load_txt(o.loadfile, &o, a, &type, &Lx, &Ly);
		if (N <= 0) die("cannot read the load file", NULL);
	} else if (o.load == 2) {
		N = load_dump(o.loadfile, a, &type, &Lx, &Ly);
		if (N <= 0) die("cannot read the dump file", NULL);
	} else {
		for (int k = 0; k < 7; k++) a[k] = calloc(N, sizeof(double));
		type = calloc(N, sizeof(int32_t));
		if (o.hex) {
			N = edmd_init_hex(N, o.phi, o.aspect, o.Einit, o.seed, a[0], a[1], a[2], a[3], a[4], a[5], type, &Lx, &Ly);
			if (N <= 0) die("bad lattice parameters", NULL);
		} else {
			edmd_init_grow(N, o.phi, o.xs, o.q, o.aspect, o.seed, a[0], a[1], a[2], a[3], a[4], a[5], a[6], type,
			               &Lx, &Ly, &vr_base);
			Nsmall = (int)(N * o.xs);
		}
	}
	double sizeratio = o.q;
	if (o.load) {                                           /* EDMD.c:1384, 1441 */
		int Nbig = 0;
		for (int i = 0; i < N; i++) Nbig += type[i];
		Nsmall = N - Nbig;
		sizeratio = a[4][N - 1];
		o.phi = M_PI * (sizeratio * sizeratio * Nsmall + Nbig) / (Lx * Ly);
	}

	/* ---- customName (EDMD.c:6015-6116): dump/ and versioned file names */
	mkdir("dump/", 0777);
	char base[400], fileName[480], thermoName[480];
	snprintf(base, sizeof base, "dump/N_%dres_%.3lfphi_%.6lfq_%.3lfrat_%.3lfLx_%.3lfLy_%.3lfv_",
	         N, o.res, o.phi, (double)Nsmall / N, sizeratio, Lx, Ly);
	int version = o.version;
	for (;;) {
		snprintf(fileName, sizeof fileName, "%s%d.dump", base, version);
		if (access(fileName, F_OK) != 0) break;
		version += 1;
	}
	snprintf(thermoName, sizeof thermoName, "%s%d.thermo", base, version);

	/* ---- engine (cellListInit + eventListInit) */
	edmd_system_desc d;
	edmd_default_desc(&d, N, Lx, Ly, o.load ? 0 : vr_base, o.tmax, o.dtime, o.dtimeThermo);
	d.res = o.res; d.Einit = o.Einit;
	d.contact = o.additive ? EDMD_CONTACT_ADDITIVE : EDMD_CONTACT_NONADDITIVE;
	edmd_ctx* ctx = NULL;
	int rc = edmd_create(1, &d, a[0], a[1], a[2], a[3], a[4], a[5], vr_base > 0 ? a[6] : NULL, 0, &ctx);
	if (rc != EDMD_OK) die(rc == EDMD_ERR_NODEV ? "no CUDA device" : "engine creation failed", ctx);

	FILE* dump = fopen(fileName, "w");
	FILE* thermo = fopen(thermoName, "w");
	if (!dump || !thermo) die("cannot open output files", NULL);
	fprintf(thermo, "t Ncol E p px py pxy pyx a2 \n");    /* initThermo 1220-1290 */

	/* ---- main loop (EDMD.c:523-618) */
	double* sx = malloc(N * 8), *sy = malloc(N * 8), *svx = malloc(N * 8), *svy = malloc(N * 8);
	double* srad = malloc(N * 8), *sm = malloc(N * 8);
	static double rows[9 * 1024];
	long long coll_left = o.max_coll < 0 ? (long long)4e18 : o.max_coll;
	uint64_t ncol_seen = 0;
	int rounds = o.engine == ENG_ROUND || (o.engine == ENG_AUTO && N >= ROUND_MIN_N);
	if ((int)(Lx / 2) < 3 || (int)(Ly / 2) < 3) rounds = 0;  /* the round engine needs 3x3 cells */
	edmd_counters cnt;
	memset(&cnt, 0, sizeof cnt);
	/* serial engine: every phase, or the growth phase before the rounds.
	 * Each call stops at a screenshot, at the growth stop (before rounds),
	 * or after at most 1000 thermo periods, so the 1024-row buffer the
	 * engine keeps per system never overflows between drains. */
	int growing = vr_base > 0 && !o.load;
	for (; !rounds || growing;) {
		double tchunk = o.dtimeThermo > 0 ? cnt.t + 1000 * o.dtimeThermo : INFINITY;
		uint32_t fl = EDMD_F_STOP_AT_SCREEN | (rounds ? EDMD_F_STOP_AT_GROW : 0);
		rc = edmd_advance(ctx, coll_left, tchunk, fl, (int64_t)1 << 60, NULL);
		if (rc != EDMD_OK) die("advance failed", ctx);
		edmd_get_counters(ctx, 0, &cnt);
		coll_left -= (long long)(cnt.ncol_total - ncol_seen);
		ncol_seen = cnt.ncol_total;
		int32_t nr = 0;
		rc = edmd_take_thermo(ctx, 0, rows, 1024, &nr);
		if (rc != EDMD_OK) die("thermo rows", ctx);
		for (int k = 0; k < nr; k++) put_row(thermo, rows + 9 * k);
		fflush(thermo);
		if (cnt.stop_reason == EDMD_STOP_SCREEN) {
			edmd_get_state(ctx, 0, sx, sy, svx, svy, srad, sm, NULL, NULL);
			put_frame(dump, cnt.t, N, Lx, Ly, type, sx, sy, svx, svy, srad, sm);
			if (!o.quiet)
				printf("\rt = %.2e / %.2e  ncol = %.2e", cnt.t, o.tmax, (double)cnt.ncol);
			if (coll_left > 0) continue;
		}
		if (cnt.stop_reason == EDMD_STOP_TIME && coll_left > 0) continue;
		break;   /* t > tmax, the growth stop (rounds follow) or the collision budget is spent */
	}
	if (rounds && coll_left > 0 && (!growing || cnt.stop_reason == EDMD_STOP_GROW))
		cnt = round_phase(ctx, &d, &o, N, Lx, Ly, type, coll_left, ncol_seen, dump, thermo,
		                  sx, sy, svx, svy, srad, sm);
	if (!o.quiet) printf("\rt = %.2e  ncol = %lu  ncross = %lu\n", cnt.t, (unsigned long)cnt.ncol, (unsigned long)cnt.ncross);
	fclose(dump);
	fclose(thermo);
	edmd_destroy(ctx);
	return 1;   /* the reference's main returns 1 */
}
