/*
 * edmd_host.h -- host-side (CPU) pieces of the drop-in that feed the engine.
 *
 * These replace the reference's setup path, which stays on the host because it
 * draws from MT19937 and libm (log/cos/sin) exactly once per run:
 *   edmd_mt_*          src/mersenne.c:68-189 (init_genrand, genrand)
 *   edmd_hex_size      src/EDMD.c:1024-1049 (constantInit, Hex branch)
 *   edmd_random_size   src/EDMD.c:1107-1166 (constantInit, default branch)
 *   edmd_grow_rate     src/EDMD.c:5766-5799 (optimizeGrowConstant)
 *   edmd_init_hex      src/EDMD.c:1582-1637 (particlesInit, Hex branch)
 *   edmd_init_grow     src/EDMD.c:1690-1829 (particlesInit, default branch)
 *   edmd_normalize     src/EDMD.c:5723-5764 (normalizePhysicalQ)
 *   edmd_default_desc  src/EDMD.c:243-249 defaults, 1958-1978 growth shifts
 */
#ifndef EDMD_HOST_H
#define EDMD_HOST_H

#include <stdint.h>
#include "edmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

void     edmd_mt_seed(uint32_t s);
uint32_t edmd_mt_u32(void);
double   edmd_mt_double(void);

int    edmd_hex_size(int N, double phi, double aspect, int* Nout, double* Lx, double* Ly);
void   edmd_random_size(int N, double phi, double xs, double q, double aspect, double* Lx, double* Ly);
double edmd_grow_rate(double phi);
void   edmd_normalize(int N, double Einit, const double* m, double* vx, double* vy);

/* Returns the rounded N (Nx*Ny); arrays must hold the requested N. */
int edmd_init_hex(int N, double phi, double aspect, double Einit, uint32_t seed,
                  double* x, double* y, double* vx, double* vy, double* rad, double* m,
                  int32_t* type, double* Lx, double* Ly);

/* Random positions, zero radii, growth rates in vr (big: vr_base, small:
 * vr_base*q); *vr_base receives optimizeGrowConstant's rate. */
int edmd_init_grow(int N, double phi, double xs, double q, double aspect, uint32_t seed,
                   double* x, double* y, double* vx, double* vy, double* rad, double* m,
                   double* vr, int32_t* type, double* Lx, double* Ly, double* vr_base);

void edmd_default_desc(edmd_system_desc* d, int N, double Lx, double Ly, double vr_base,
                       double tmax, double dtime, double dtime_thermo);

#ifdef __cplusplus
}
#endif
#endif
