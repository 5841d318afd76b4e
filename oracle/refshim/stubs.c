/* Abort-on-call stand-ins for the external solver libraries the reference links
 * (Makefile:7): UMFPACK, LAPACK dgesv/dgetrf/dgetrs and CBLAS dgemv. The
 * skyline path (SLVFLAG == 0) never reaches them. Test infrastructure only. */
#include <stdio.h>
#include <stdlib.h>

static void stub_called(const char *name)
{
    fprintf(stderr, "reference stub %s called: SLVFLAG != 0 is not supported\n", name);
    abort();
}

int umfpack_di_symbolic(void) { stub_called("umfpack_di_symbolic"); return 0; }
int umfpack_di_numeric(void) { stub_called("umfpack_di_numeric"); return 0; }
int umfpack_di_solve(void) { stub_called("umfpack_di_solve"); return 0; }
void umfpack_di_free_symbolic(void) { stub_called("umfpack_di_free_symbolic"); }
void umfpack_di_free_numeric(void) { stub_called("umfpack_di_free_numeric"); }
void dgesv_(void) { stub_called("dgesv_"); }
void dgetrf_(void) { stub_called("dgetrf_"); }
void dgetrs_(void) { stub_called("dgetrs_"); }
void cblas_dgemv(void) { stub_called("cblas_dgemv"); }
