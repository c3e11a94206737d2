/*
 * ref_harness.c -- drives the reference's OWN unmodified C (src/EDMD.c and
 * the satellites its Makefile compiles) and writes a collision trace.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle ref` from the sources
 * where they lie under the reference checkout (REF=...); the binary goes to
 * oracle/_ref/ and is used to pin the oracle restatement and to generate the
 * golden fixtures under tests/golden/.  Nothing of the reference is copied:
 * this file #includes EDMD.c and re-runs the body of its main loop
 * (src/EDMD.c:523-618) with a logging hook and a collision-count stop.
 *
 * usage: ref_trace [--hex] <reference CLI flags ...>
 * env:   MAXCOLL (default 10000), TSTOP (default inf),
 *        TRACE_OUT (default stdout), DUMP_OUT, THERMO_OUT (default /dev/null),
 *        EVENTS=1 (also log every popped event)
 */
#define main edmd_reference_main
#include "EDMD.c"
#undef main

int main(int argc, char* argv[])
{
	long maxcoll = getenv("MAXCOLL") ? atol(getenv("MAXCOLL")) : 10000;
	double tstop = getenv("TSTOP") ? atof(getenv("TSTOP")) : 1e300;
	FILE* tr = getenv("TRACE_OUT") ? fopen(getenv("TRACE_OUT"), "w") : stdout;
	int log_events = getenv("EVENTS") != NULL;
	int a = 1;
	if (argc > 1 && strcmp(argv[1], "--hex") == 0) { Hex = 1; a = 2; }
	argv[a - 1] = argv[0];
	init_genrand(5489UL);
	constantInit(argc - a + 1, argv + a - 1);
	particlesInit();
	cellListInit();
	eventListInit();
	physicalQ();
	fichier = fopen(getenv("DUMP_OUT") ? getenv("DUMP_OUT") : "/dev/null", "w");
	snprintf(thermoName, sizeof(thermoName), "%s", getenv("THERMO_OUT") ? getenv("THERMO_OUT") : "/dev/null");
	initThermo();
	fprintf(tr, "# N %d Lx %a Ly %a Nxc %d Nyc %d\n", N, Lx, Ly, Nxcells, Nycells);
	for (int i = 0; i < N; i++)
		fprintf(tr, "I %d %a %a %a %a %a %a %d\n", i, particles[i].x, particles[i].y,
		        particles[i].vx, particles[i].vy, particles[i].rad, particles[i].m, particles[i].type);
	long logged = 0, nev = 0;
	while (t <= tmax && logged < maxcoll) {
		nextEvent = findNextEvent();
		if (nextEvent->t >= tstop) break;
		t = nextEvent->t;
		removeEventFromQueue(nextEvent);
		int stale = 0;
		if (nextEvent->type == COLLISION) {
			particle* pi = particles + nextEvent->i;
			particle* pj = particles + nextEvent->j;
			stale = nextEvent->collActual != pj->coll;
			if (!stale) {
				fprintf(tr, "C %ld %d %d %d %d %a\n", logged, nextEvent->i, nextEvent->j,
				        pi->cell[1] * Nxcells + pi->cell[0], pj->cell[1] * Nxcells + pj->cell[0], t);
				logged++;
			}
		}
		if (log_events)
			fprintf(tr, "E %ld %d %d %d %d %a\n", nev, (int)nextEvent->type, nextEvent->i, nextEvent->j, stale, t);
		nev++;
		switch (nextEvent->type) {
		case COLLISION: doTheCollision(); break;
		case CELLCROSS: ncross++; doTheCrossing(); break;
		case SCREENSHOT: takeAScreenshot(); break;
		case THERMO: takeAThermo(); break;
		case GROWSTOP: stopGrow(); break;
		default: break;
		}
	}
	fprintf(tr, "V %a %a %a %a\n", collTermX, collTermY, collTermXY, collTermYX);
	fprintf(tr, "T %a %lu %lu\n", t, ncol, ncross);
	for (int i = 0; i < N; i++) freeFly(particles + i);
	for (int i = 0; i < N; i++)
		fprintf(tr, "S %d %a %a %a %a %a %d %lu\n", i, particles[i].x, particles[i].y,
		        particles[i].vx, particles[i].vy, particles[i].rad,
		        particles[i].cell[1] * Nxcells + particles[i].cell[0], particles[i].coll);
	fclose(fichier);
	fclose(thermo);
	if (tr != stdout) fclose(tr);
	return 0;
}
