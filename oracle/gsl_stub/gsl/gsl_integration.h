/*
 * GSL integration API subset: types and prototypes only.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY.  GSL is not installed here (the
 * reference's makefile links -lgsl with no version).  The reference's
 * auxiliary.c:18 includes this header for sigmaR() (auxiliary.c:377-398),
 * which integrates with gsl_integration_qag and the 15-point Gauss-Kronrod
 * rule; the halo finder reaches it through sigma() (get_halos.c:213, 304,
 * 335).  gsl_stub.c restates that published algorithm (QUADPACK QAG/QK15,
 * Piessens et al. 1983).
 */
#ifndef SF21_ORACLE_GSL_INTEGRATION_STUB_H
#define SF21_ORACLE_GSL_INTEGRATION_STUB_H
#include <stddef.h>

typedef struct {
  double (*function)(double x, void *params);
  void *params;
} gsl_function;

typedef struct gsl_integration_workspace_s gsl_integration_workspace;

enum { GSL_INTEG_GAUSS15 = 1, GSL_INTEG_GAUSS21 = 2, GSL_INTEG_GAUSS31 = 3,
       GSL_INTEG_GAUSS41 = 4, GSL_INTEG_GAUSS51 = 5, GSL_INTEG_GAUSS61 = 6 };

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qag(const gsl_function *f, double a, double b,
                        double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace *workspace, double *result,
                        double *abserr);
#endif
