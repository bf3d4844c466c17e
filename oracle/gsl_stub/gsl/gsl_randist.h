/*
 * GSL random-distribution API subset used by the halo finder's subgrid
 * cycle (get_halos.c:353): Poisson deviates.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  gsl_stub.c restates the published
 * method for means up to 10: Knuth's product of uniforms (TAOCP vol. 2,
 * 3.4.1, algorithm Q); a larger mean aborts (its gamma/binomial split is not
 * restated).
 */
#ifndef SF21_ORACLE_GSL_RANDIST_STUB_H
#define SF21_ORACLE_GSL_RANDIST_STUB_H
#include "gsl/gsl_rng.h"

unsigned int gsl_ran_poisson(const gsl_rng *r, double mu);
#endif
