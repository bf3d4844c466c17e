/*
 * Included by get_halos.c:24, which calls nothing from it.
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 */
#ifndef SF21_ORACLE_GSL_SF_ERF_STUB_H
#define SF21_ORACLE_GSL_SF_ERF_STUB_H
#endif
