/* Link-time wrapper (-Wl,--wrap=test) around the reference's convergence test
 * (misc.c:187-250). When CUBEN_TESTLOG names a file it appends, per call, the
 * three criteria the test evaluates and the true relative residual
 * |qtot - f| / |qtot|, all in FP64 binary (5 doubles + int32 convchk + pad).
 * Test infrastructure only. */
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <math.h>

extern long NEQ;
int __real_test(double *pd_temp, double *pdd, double *pf_temp, double *pfp, double *pqtot,
                double *pf_ip, double *pintener1, int *pconvchk, double *ptoldisp,
                double *ptolforc, double *ptolener);

static FILE *log_fp = NULL;

int __wrap_test(double *pd_temp, double *pdd, double *pf_temp, double *pfp, double *pqtot,
                double *pf_ip, double *pintener1, int *pconvchk, double *ptoldisp,
                double *ptolforc, double *ptolener)
{
    int rc = __real_test(pd_temp, pdd, pf_temp, pfp, pqtot, pf_ip, pintener1, pconvchk,
                         ptoldisp, ptolforc, ptolener);
    const char *path = getenv("CUBEN_TESTLOG");
    if (!path) return rc;
    if (!log_fp) log_fp = fopen(path, "wb");
    if (!log_fp) return rc;
    double sdd = 0, sdt = 0, sr = 0, srp = 0, sen = 0, sq = 0;
    for (long i = 0; i < NEQ; ++i) {
        double r = pqtot[i] - pf_temp[i], rp = pqtot[i] - pfp[i];
        sdd += pdd[i] * pdd[i];
        sdt += pd_temp[i] * pd_temp[i];
        sr += r * r;
        srp += rp * rp;
        sen += pdd[i] * (pqtot[i] - pf_ip[i]);
        sq += pqtot[i] * pqtot[i];
    }
    double rec[5] = {sqrt(sdd) / sqrt(sdt), sqrt(sr) / sqrt(srp), fabs(sen / *pintener1),
                     sqrt(sr) / sqrt(sq), 0.0};
    int32_t cc[2] = {*pconvchk, rc};
    fwrite(rec, sizeof rec, 1, log_fp);
    fwrite(cc, sizeof cc, 1, log_fp);
    fflush(log_fp);
    return rc;
}
