/*
 * Included by get_SFR.c:21, which calls nothing from it.
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 */
#ifndef SF21_ORACLE_GSL_SPLINE_STUB_H
#define SF21_ORACLE_GSL_SPLINE_STUB_H
#endif
