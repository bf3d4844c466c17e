/*
 * GSL random-number API subset used by the halo finder (get_halos.c:70-71,
 * 353): the gsl_rng_taus generator and its uniform deviate.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY (GSL is not installed here).  gsl_stub.c
 * restates the published generator: L'Ecuyer's maximally equidistributed
 * combined Tausworthe generator (Math. Comp. 65 (1996) 203-213, "taus88"),
 * with GSL's seeding by the 69069 linear congruential sequence.  Parity of
 * this part is unpinned against a real GSL build (none is available).
 */
#ifndef SF21_ORACLE_GSL_RNG_STUB_H
#define SF21_ORACLE_GSL_RNG_STUB_H

typedef struct {
  const char *name;
} gsl_rng_type;

typedef struct {
  const gsl_rng_type *type;
  unsigned long s1, s2, s3;
} gsl_rng;

extern const gsl_rng_type *gsl_rng_taus;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long int seed);
void gsl_rng_free(gsl_rng *r);
unsigned long gsl_rng_get(const gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
#endif
