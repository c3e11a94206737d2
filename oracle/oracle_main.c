/*
 * oracle_main.c -- command-line front end of the CPU oracle.
 * TEST INFRASTRUCTURE ONLY.  Prints the same trace format as
 * ref_harness.c so the two can be compared line by line.
 *
 * usage: oracle_trace [--hex] [-N n] [--phi f] [-x f] [-q f] [-a f]
 *                     [-E f] [-r f] [-t f] [-D f] [-o f] [-v seed]
 * env:   MAXCOLL, TSTOP, TRACE_OUT, EVENTS (as ref_harness.c)
 */
#include "edmd_oracle.h"
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int main(int argc, char* argv[])
{
	orc_params p;
	orc_default_params(&p);
	p.start = ORC_START_GROW;
	long maxcoll = getenv("MAXCOLL") ? atol(getenv("MAXCOLL")) : 10000;
	double tstop = getenv("TSTOP") ? atof(getenv("TSTOP")) : 1e300;
	FILE* tr = getenv("TRACE_OUT") ? fopen(getenv("TRACE_OUT"), "w") : stdout;
	int log_events = getenv("EVENTS") != NULL;
	int a = 1;
	if (argc > 1 && strcmp(argv[1], "--hex") == 0) { p.start = ORC_START_HEX; a = 2; }
	static struct option lo[] = {
		{"number", 1, 0, 'N'}, {"phi", 1, 0, 'p'}, {"xs", 1, 0, 'x'}, {"sizeratio", 1, 0, 'q'},
		{"aspect", 1, 0, 'a'}, {"initial-energy", 1, 0, 'E'}, {"res", 1, 0, 'r'},
		{"time", 1, 0, 't'}, {"dt", 1, 0, 'D'}, {"dtimeThermo", 1, 0, 'o'}, {"version", 1, 0, 'v'},
		{0, 0, 0, 0}};
	int c;
	argv[a - 1] = argv[0];
	while ((c = getopt_long(argc - a + 1, argv + a - 1, "N:p:x:q:a:E:r:t:D:o:v:", lo, NULL)) != -1) {
		switch (c) {
		case 'N': p.N = atoi(optarg); break;
		case 'p': p.phi = atof(optarg); break;
		case 'x': p.xs = atof(optarg); break;
		case 'q': p.q = atof(optarg); break;
		case 'a': p.aspect = atof(optarg); break;
		case 'E': p.Einit = atof(optarg); break;
		case 'r': p.res = atof(optarg); break;
		case 't': p.tmax = atof(optarg); break;
		case 'D': p.dtime = atof(optarg); break;
		case 'o': p.dtimeThermo = atof(optarg); break;
		case 'v': p.seed = (uint32_t)atoi(optarg); break;
		}
	}
	orc_sys* s = orc_create(&p);
	int N = orc_N(s), nx, ny;
	double Lx, Ly;
	orc_box(s, &Lx, &Ly, &nx, &ny);
	fprintf(tr, "# N %d Lx %a Ly %a Nxc %d Nyc %d\n", N, Lx, Ly, nx, ny);
	double *x = malloc(N * 8), *y = malloc(N * 8), *vx = malloc(N * 8), *vy = malloc(N * 8);
	double *rad = malloc(N * 8), *m = malloc(N * 8);
	int32_t *type = malloc(N * 4), *cell = malloc(N * 4);
	uint64_t* coll = malloc(N * 8);
	orc_state(s, x, y, vx, vy, NULL, rad, m, type, cell, coll);
	for (int i = 0; i < N; i++)
		fprintf(tr, "I %d %a %a %a %a %a %a %d\n", i, x[i], y[i], vx[i], vy[i], rad[i], m[i], type[i]);
	long chunk = 1 << 16;
	orc_coll* co = malloc(chunk * sizeof(orc_coll));
	orc_event* eo = log_events ? malloc(chunk * 4 * sizeof(orc_event)) : NULL;
	long logged = 0, nevt = 0;
	for (;;) {
		long want = maxcoll - logged < chunk ? maxcoll - logged : chunk;
		int64_t ne = 0;
		double t0 = orc_time(s);
		(void)t0;
		long got = (long)orc_run(s, want, tstop, co, chunk, eo, log_events ? chunk * 4 : 0, &ne);
		if (log_events && ne > chunk * 4) { fprintf(stderr, "event buffer too small\n"); return 2; }
		/* interleave is not needed: collisions and events are printed per chunk */
		for (long k = 0; k < got; k++)
			fprintf(tr, "C %ld %d %d %d %d %a\n", logged + k, co[k].i, co[k].j, co[k].ci, co[k].cj, co[k].t);
		if (log_events)
			for (long k = 0; k < ne; k++)
				fprintf(tr, "E %ld %d %d %d %d %a\n", nevt + k, eo[k].type, eo[k].i, eo[k].j, eo[k].stale, eo[k].t);
		logged += got; nevt += ne;
		if (got < want || logged >= maxcoll) break;
	}
	double v[4];
	orc_virial(s, v, 0);
	fprintf(tr, "V %a %a %a %a\n", v[0], v[1], v[2], v[3]);
	uint64_t ncol, ncross, nstale, npair, npred;
	orc_counters(s, &ncol, &ncross, &nstale, &npair, &npred);
	fprintf(tr, "T %a %lu %lu\n", orc_time(s), (unsigned long)ncol, (unsigned long)ncross);
	orc_sync_all(s);
	orc_state(s, x, y, vx, vy, NULL, rad, m, type, cell, coll);
	for (int i = 0; i < N; i++)
		fprintf(tr, "S %d %a %a %a %a %a %d %lu\n", i, x[i], y[i], vx[i], vy[i], rad[i], cell[i], (unsigned long)coll[i]);
	fprintf(stderr, "oracle: N=%d t=%.6f ncol=%lu ncross=%lu stale=%lu pair=%lu pred=%lu\n", N, orc_time(s),
	        (unsigned long)ncol, (unsigned long)ncross, (unsigned long)nstale, (unsigned long)npair, (unsigned long)npred);
	orc_destroy(s);
	if (tr != stdout) fclose(tr);
	return 0;
}
