/* Declarations that let the reference's solve.c compile without SuiteSparse.
 * The UMFPACK / LAPACK / CBLAS branches are reached only with SLVFLAG != 0,
 * which no model used here selects; stubs.c aborts if one is ever called.
 * Test infrastructure only. */
#define UMFPACK_A 0
int umfpack_di_symbolic(int, int, const int *, const int *, const double *, void **,
                        const double *, double *);
int umfpack_di_numeric(const int *, const int *, const double *, void *, void **,
                       const double *, double *);
void umfpack_di_free_symbolic(void **);
void umfpack_di_free_numeric(void **);
int umfpack_di_solve(int, const int *, const int *, const double *, double *,
                     const double *, void *, const double *, double *);
