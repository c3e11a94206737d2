/*
 * edmd_init.c -- host-side initial conditions of the drop-in (C, no GPU).
 *
 * Restates the reference's box sizing and start modes so the GPU engine is
 * fed exactly the state the reference would build from the same command line:
 *   MT19937            src/mersenne.c:68-81, 113-148, 185-189
 *   drand              src/EDMD.c:5699-5701
 *   Hex box sizing     src/EDMD.c:1024-1049 (constantInit)
 *   random box sizing  src/EDMD.c:1107-1166
 *   Hex lattice start  src/EDMD.c:1582-1637 (particlesInit)
 *   growth start       src/EDMD.c:1690-1829, optimizeGrowConstant 5766-5799
 *   normalizePhysicalQ src/EDMD.c:5723-5764
 * Built with -ffp-contract=off; the Box-Muller draws go through libm.
 */
#include "../../include/edmd_host.h"

#include <math.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define MT_N 624
#define MT_M 397
static uint32_t mt[MT_N];
static int mti = MT_N + 1;

void edmd_mt_seed(uint32_t s)
{
	mt[0] = s;
	for (mti = 1; mti < MT_N; mti++)
		mt[mti] = 1812433253u * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) + (uint32_t)mti;
}

uint32_t edmd_mt_u32(void)
{
	uint32_t y;
	if (mti >= MT_N) {
		if (mti == MT_N + 1) edmd_mt_seed(5489u);
		for (int k = 0; k < MT_N; k++) {
			y = (mt[k] & 0x80000000u) | (mt[(k + 1) % MT_N] & 0x7fffffffu);
			mt[k] = mt[(k + MT_M) % MT_N] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
		}
		mti = 0;
	}
	y = mt[mti++];
	y ^= (y >> 11);
	y ^= (y << 7) & 0x9d2c5680u;
	y ^= (y << 15) & 0xefc60000u;
	y ^= (y >> 18);
	return y;
}

double edmd_mt_double(void) { return edmd_mt_u32() * (1.0 / 4294967296.0); }
static double drand_(double lo, double hi) { return (edmd_mt_double() * (hi - lo)) + lo; }

int edmd_hex_size(int N, double phi, double aspect, int* Nout, double* Lx, double* Ly)
{
	int Ny = sqrt(N) * aspect;
	if (Ny % 2 == 1) Ny += 1;
	if (Ny <= 0) return -1;
	int Nx = N / Ny;
	N = Nx * Ny;
	if (N <= 0) return -1;
	*Ly = sqrt(sqrt(3) / 2 * Ny / Nx * M_PI * N / phi);
	*Lx = 2 / sqrt(3) * Nx / Ny * *Ly;
	*Nout = N;
	return 0;
}

void edmd_random_size(int N, double phi, double xs, double q, double aspect, double* Lx, double* Ly)
{
	double r2 = (1 + xs * (q * q - 1));
	*Lx = sqrt(M_PI * N / (phi * aspect) * r2);
	*Ly = *Lx * aspect;
}

double edmd_grow_rate(double phi)
{
	double vr;
	if (phi < 0.8) vr = 0.1;
	else vr = 0.1 * pow(0.8 / phi, 30);
	if (phi > 0.7) vr /= 8;
	return vr;
}

void edmd_normalize(int N, double Einit, const double* m, double* vx, double* vy)
{
	double px = 0, py = 0, E = 0;
	for (int i = 0; i < N; i++) {
		px += vx[i] * m[i]; py += vy[i] * m[i];
		double v = vx[i];
		E += 0.5 * m[i] * (v * v + vy[i] * vy[i]);
	}
	for (int i = 0; i < N; i++) {
		vx[i] -= px / (N * m[i]);
		vy[i] -= py / (N * m[i]);
	}
	px = py = E = 0;
	for (int i = 0; i < N; i++) {
		double v = vx[i];
		E += 0.5 * m[i] * (v * v + vy[i] * vy[i]);
	}
	for (int i = 0; i < N; i++) {
		vx[i] /= sqrt(E / N / Einit);
		vy[i] /= sqrt(E / N / Einit);
	}
}

int edmd_init_hex(int N, double phi, double aspect, double Einit, uint32_t seed,
                  double* x, double* y, double* vx, double* vy, double* rad, double* m,
                  int32_t* type, double* Lx_out, double* Ly_out)
{
	int Nr;
	double Lx, Ly;
	if (edmd_hex_size(N, phi, aspect, &Nr, &Lx, &Ly)) return -1;
	int Ny = sqrt(N) * aspect;
	if (Ny % 2 == 1) Ny += 1;
	int Nx = N / Ny;
	edmd_mt_seed(seed);
	double dx = Lx / Nx, dy = Ly / Ny;
	int k = 0;
	for (int i = 0; i < Nx; i++)
		for (int j = 0; j < Ny; j++) {
			x[k] = i * dx + (j % 2) * (dx / 2);
			y[k] = j * dy;
			type[k] = 1; rad[k] = 1; m[k] = 1;
			double U1 = drand_(0, 1), U2 = drand_(0, 1);
			vx[k] = sqrt(-2 * log(U1) / m[k] * Einit) * cos(2 * M_PI * U2);
			vy[k] = sqrt(-2 * log(U1) / m[k] * Einit) * sin(2 * M_PI * U2);
			k++;
		}
	edmd_normalize(Nr, Einit, m, vx, vy);
	*Lx_out = Lx; *Ly_out = Ly;
	return Nr;
}

int edmd_init_grow(int N, double phi, double xs, double q, double aspect, uint32_t seed,
                   double* x, double* y, double* vx, double* vy, double* rad, double* m,
                   double* vr_out, int32_t* type, double* Lx_out, double* Ly_out, double* vr_base)
{
	double Lx, Ly;
	edmd_random_size(N, phi, xs, q, aspect, &Lx, &Ly);
	double EinitGrow = 0.05;
	double vr = edmd_grow_rate(phi);
	edmd_mt_seed(seed);
	int Nsmall = (int)(N * xs), Nbig = N - Nsmall;
	for (int i = 0; i < N; i++) {
		x[i] = drand_(0, Lx);
		y[i] = drand_(0, Ly);
		rad[i] = 0;
		if (i < Nbig) { type[i] = 1; m[i] = 1; vr_out[i] = vr; }
		else { type[i] = 0; m[i] = 1; vr_out[i] = vr * q; }
		double U1 = drand_(0, 1), U2 = drand_(0, 1);
		vx[i] = sqrt(-2 * log(U1) / m[i] * EinitGrow) * cos(2 * M_PI * U2);
		vy[i] = sqrt(-2 * log(U1) / m[i] * EinitGrow) * sin(2 * M_PI * U2);
		(void)drand_(0, 1);   /* charge draw of the reference, consumed */
	}
	*Lx_out = Lx; *Ly_out = Ly; *vr_base = vr;
	return N;
}

/* system descriptor with the reference's defaults for sampling times:
 * firstScreen 1, firstThermo 1000, dtime 100, dtimeThermo 100, tmax 4000
 * (src/EDMD.c:243-249), shifted by 1/vr for a growth start
 * (eventListInit src/EDMD.c:1958-1978). */
void edmd_default_desc(edmd_system_desc* d, int N, double Lx, double Ly, double vr_base,
                       double tmax, double dtime, double dtime_thermo)
{
	memset(d, 0, sizeof(*d));
	d->N = N; d->Lx = Lx; d->Ly = Ly; d->res = 1; d->Einit = 1;
	d->first_screen = 1; d->first_thermo = 1000;
	d->dtime = dtime; d->dtime_thermo = dtime_thermo;
	d->tmax = tmax;
	d->t_growstop = -1;
	if (vr_base > 0) {
		double inv = 1 / vr_base;
		if (d->first_screen < inv) d->first_screen = inv + d->first_screen;
		if (d->first_thermo < inv) d->first_thermo = inv + d->first_thermo;
		d->tmax += 1 / vr_base;
		d->t_growstop = 1 / vr_base;
	}
}
