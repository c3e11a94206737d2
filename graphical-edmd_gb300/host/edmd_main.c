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
 * NONADDITIVE 1, src/EDMD.c:35-43).
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
	long long max_coll; int quiet; int additive;
} opts;

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

int main(int argc, char* argv[])
{
	opts o = {500, 0.38, 0.3, 0.4, 1.0, 4000, 100, 100, 1, 1, 0, 1, 0, 0, "", -1, 0, 0};
	int seeded = 0;
	static struct option lo[] = {
		{"load", 1, 0, 'l'}, {"number", 1, 0, 'N'}, {"phi", 1, 0, 'p'}, {"res", 1, 0, 'r'},
		{"time", 1, 0, 't'}, {"dt", 1, 0, 'D'}, {"initial-energy", 1, 0, 'E'}, {"xs", 1, 0, 'x'},
		{"sizeratio", 1, 0, 'q'}, {"aspect", 1, 0, 'a'}, {"dtimeThermo", 1, 0, 'o'},
		{"version", 1, 0, 'v'}, {"hex", 0, 0, 1000}, {"max-coll", 1, 0, 1001}, {"quiet", 0, 0, 1002},
		{"additive", 0, 0, 1003}, {0, 0, 0, 0}};
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
	if (rc != EDMD_OK) die("engine creation failed", ctx);

	FILE* dump = fopen(fileName, "w");
	FILE* thermo = fopen(thermoName, "w");
	if (!dump || !thermo) die("cannot open output files", NULL);
	fprintf(thermo, "t Ncol E p px py pxy pyx a2 \n");    /* initThermo 1220-1290 */

	/* ---- main loop: advance to each screenshot, dump, repeat (EDMD.c:523-618) */
	double* sx = malloc(N * 8), *sy = malloc(N * 8), *svx = malloc(N * 8), *svy = malloc(N * 8);
	double* srad = malloc(N * 8), *sm = malloc(N * 8);
	static double rows[9 * 1024];
	int32_t rows_done = 0;
	long long coll_left = o.max_coll < 0 ? (long long)4e18 : o.max_coll;
	uint64_t ncol_seen = 0;
	for (;;) {
		rc = edmd_advance(ctx, coll_left, INFINITY, EDMD_F_STOP_AT_SCREEN, (int64_t)1 << 60, NULL);
		if (rc != EDMD_OK) die("advance failed", ctx);
		edmd_counters cnt;
		edmd_get_counters(ctx, 0, &cnt);
		coll_left -= (long long)(cnt.ncol_total - ncol_seen);
		ncol_seen = cnt.ncol_total;
		/* thermo rows produced so far (saveThermo row format, 5409-5577) */
		int32_t nr = 0;
		edmd_get_thermo(ctx, 0, rows, 1024, &nr);
		if (nr > 1024) nr = 1024;
		for (; rows_done < nr; rows_done++) {
			double* r = rows + 9 * rows_done;
			fprintf(thermo, "%lf ", r[0]);
			fprintf(thermo, "%ld ", (long)r[1]);
			fprintf(thermo, "%lf ", r[2]);
			fprintf(thermo, "%lf %lf %lf %.10lf %.10lf ", r[3], r[4], r[5], r[6], r[7]);
			fprintf(thermo, "%lf ", r[8]);
			fprintf(thermo, "\n");
		}
		fflush(thermo);
		if (cnt.stop_reason == EDMD_STOP_SCREEN) {          /* takeAScreenshot -> saveTXT */
			edmd_get_state(ctx, 0, sx, sy, svx, svy, srad, sm, NULL, NULL);
			fprintf(dump, "ITEM: TIMESTEP\n%lf\nITEM: NUMBER OF ATOMS\n%d\nITEM: BOX BOUNDS pp pp pp\n"
			              "0 %lf\n0 %lf\n0 0\nITEM: ATOMS id type x y vx vy radius m coll", cnt.t, N, Lx, Ly);
			fprintf(dump, "\n");
			for (int i = 0; i < N; i++) {
				fprintf(dump, "%d %d %.3lf %lf %lf %lf %lf %lf %d", i, type[i], sx[i], sy[i], svx[i], svy[i],
				        srad[i], sm[i], type[i]);
				fprintf(dump, "\n");
			}
			fflush(dump);
			if (!o.quiet)
				printf("\rt = %.2e / %.2e  ncol = %.2e", cnt.t, o.tmax, (double)cnt.ncol);
			if (coll_left > 0) continue;
		}
		break;   /* t > tmax or the collision budget is spent */
	}
	edmd_counters cnt;
	edmd_get_counters(ctx, 0, &cnt);
	if (!o.quiet) printf("\rt = %.2e  ncol = %lu  ncross = %lu\n", cnt.t, (unsigned long)cnt.ncol, (unsigned long)cnt.ncross);
	fclose(dump);
	fclose(thermo);
	edmd_destroy(ctx);
	return 1;   /* the reference's main returns 1 */
}
