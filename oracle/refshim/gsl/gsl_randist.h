/*
 * ORACLE shim -- test infrastructure only.  gsl_ran_flat / gsl_ran_gaussian
 * (called at shared/particle.h:154, 202, 273, 568) mapped onto the Philox
 * stream: flat uses the Vicsek-noise stream, gaussian the rotational-noise
 * stream, with the same uniform -> double and Box-Muller mappings as
 * oracle/spp_oracle64.c.
 */
#ifndef ORACLE_SHIM_GSL_RANDIST_H
#define ORACLE_SHIM_GSL_RANDIST_H
#include <math.h>
#include "gsl_rng.h"

static inline double gsl_ran_flat(const gsl_rng*, double a, double b) {
  double u = spp_u01_d(shim_next_bits(SPP_RNG_VICSEK).v[0]);
  return a * (1 - u) + b * u; /* GSL's gsl_ran_flat formula */
}
static inline double gsl_ran_gaussian(const gsl_rng*, double sigma) {
  spp_u32x4 d = shim_next_bits(SPP_RNG_ROT_NOISE);
  double u1 = spp_u01_open0_d(d.v[0]);
  double u2 = spp_u01_d(d.v[1]);
  return sigma * (sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2));
}
#endif
