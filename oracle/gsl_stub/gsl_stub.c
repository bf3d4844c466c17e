/*
 * Aborting bodies for the GSL symbols declared in gsl/gsl_integration.h.
 * ORACLE / TEST INFRASTRUCTURE ONLY: the HII stage never reaches them
 * (only sigmaR, auxiliary.c:377-398, integrates with GSL).
 */
#include <stdio.h>
#include <stdlib.h>

#include "gsl/gsl_integration.h"

static void sf21_gsl_absent(const char *fn) {
  fprintf(stderr, "GSL stub: %s called, but GSL is not part of the HII path\n", fn);
  abort();
}
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n) {
  (void)n;
  sf21_gsl_absent("gsl_integration_workspace_alloc");
  return NULL;
}
void gsl_integration_workspace_free(gsl_integration_workspace *w) {
  (void)w;
  sf21_gsl_absent("gsl_integration_workspace_free");
}
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs,
                        double epsrel, size_t limit, int key,
                        gsl_integration_workspace *workspace, double *result,
                        double *abserr) {
  (void)f; (void)a; (void)b; (void)epsabs; (void)epsrel; (void)limit; (void)key;
  (void)workspace; (void)result; (void)abserr;
  sf21_gsl_absent("gsl_integration_qag");
  return -1;
}
