/* Strict-mode forwarders: the reference's unmodified objects, linked with
 * -Wl,--wrap=<name> for every hot-path entry point, call __wrap_<name>,
 * which forwards to the library's <name> (libcubens_dropin.so, opened at run
 * time because the reference objects define the same names). The library
 * path is $CUBENS_DROPIN, else libcubens_dropin.so on the loader's search
 * path. The program must export CU-BENs' globals (NJ, NEQ, ...) for the
 * library to bind them: link with -rdynamic. Generated from the prototypes of
 * include/cubens_gb300_dropin.h; test infrastructure only. */
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>

#include "cubens_gb300_dropin.h"

static void *resolve(const char *name)
{
    static void *lib = NULL;
    if (!lib) {
        const char *path = getenv("CUBENS_DROPIN");
        lib = dlopen(path ? path : "libcubens_dropin.so", RTLD_NOW | RTLD_GLOBAL);
        if (!lib) {
            fprintf(stderr, "strict mode: cannot open the drop-in library: %s\n", dlerror());
            exit(3);
        }
    }
    void *f = dlsym(lib, name);
    if (!f) {
        fprintf(stderr, "strict mode: the drop-in library has no %s\n", name);
        exit(3);
    }
    return f;
}

void __wrap_updatc(double *px_temp, double *px_ip, double *pxfr_temp, double *pdd, double *pdefllen_i, double *pdeffarea_i, double *pdefslen_i, double *poffset, int *posflag, double *pauxpt, double *pc1_i, double *pc2_i, double *pc3_i, long *pminc, long *pjcode)
{
    static __typeof__(updatc) *f = NULL;
    if (!f) f = (__typeof__(updatc) *)resolve("updatc");
    f(px_temp, px_ip, pxfr_temp, pdd, pdefllen_i, pdeffarea_i, pdefslen_i, poffset, posflag, pauxpt, pc1_i, pc2_i, pc3_i, pminc, pjcode);
}

void __wrap_stiff_tr(double *pss, double *pemod, double *pcarea, double *plength, double *pdefllen_ip, double *pyield, double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pef_ip, long *pmaxa, long *pmcode)
{
    static __typeof__(stiff_tr) *f = NULL;
    if (!f) f = (__typeof__(stiff_tr) *)resolve("stiff_tr");
    f(pss, pemod, pcarea, plength, pdefllen_ip, pyield, pc1_ip, pc2_ip, pc3_ip, pef_ip, pmaxa, pmcode);
}

void __wrap_forces_tr(double *pf_temp, double *pef_i, double *pd, double *pemod, double *pcarea, double *pllength, double *pdefllen_i, double *pyield, double *pc1_i, double *pc2_i, double *pc3_i, long *pmcode)
{
    static __typeof__(forces_tr) *f = NULL;
    if (!f) f = (__typeof__(forces_tr) *)resolve("forces_tr");
    f(pf_temp, pef_i, pd, pemod, pcarea, pllength, pdefllen_i, pyield, pc1_i, pc2_i, pc3_i, pmcode);
}

void __wrap_stiff_fr(double *pss, double *pemod, double *pgmod, double *pcarea, double *poffset, int *posflag, double *pllength, double *pdefllen_ip, double *pistrong, double *piweak, double *pipolar, double *piwarp, int *pyldflag, double *pyield, double *pzstrong, double *pzweak, double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pef_ip, double *pefFE_ip, int *pmendrel, long *pmaxa, long *pmcode)
{
    static __typeof__(stiff_fr) *f = NULL;
    if (!f) f = (__typeof__(stiff_fr) *)resolve("stiff_fr");
    f(pss, pemod, pgmod, pcarea, poffset, posflag, pllength, pdefllen_ip, pistrong, piweak, pipolar, piwarp, pyldflag, pyield, pzstrong, pzweak, pc1_ip, pc2_ip, pc3_ip, pef_ip, pefFE_ip, pmendrel, pmaxa, pmcode);
}

int __wrap_forces_fr(double *pf_temp, double *pef_ip, double *pef_i, double *pefFE_ref, double *pefFE_ip, double *pefFE_i, int *pyldflag, double *pdd, double *pemod, double *pgmod, double *pcarea, double *poffset, int *posflag, double *pllength, double *pdefllen_ip, double *pistrong, double *piweak, double *pipolar, double *piwarp, double *pyield, double *pzstrong, double *pzweak, double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pc1_i, double *pc2_i, double *pc3_i, int *pmendrel, long *pmcode, double *pdlpf, int *pitecnt)
{
    static __typeof__(forces_fr) *f = NULL;
    if (!f) f = (__typeof__(forces_fr) *)resolve("forces_fr");
    return f(pf_temp, pef_ip, pef_i, pefFE_ref, pefFE_ip, pefFE_i, pyldflag, pdd, pemod, pgmod, pcarea, poffset, posflag, pllength, pdefllen_ip, pistrong, piweak, pipolar, piwarp, pyield, pzstrong, pzweak, pc1_ip, pc2_ip, pc3_ip, pc1_i, pc2_i, pc3_i, pmendrel, pmcode, pdlpf, pitecnt);
}

void __wrap_mass_fr(double *psm, double *pcarea, double *pllength, double *pistrong, double *piweak, double *pipolar, double *piwarp, double *pdens, int *posflag, double *poffset, double *px, double *pxfr, long *pminc, long *pmcode, double *pjac)
{
    static __typeof__(mass_fr) *f = NULL;
    if (!f) f = (__typeof__(mass_fr) *)resolve("mass_fr");
    f(psm, pcarea, pllength, pistrong, piweak, pipolar, piwarp, pdens, posflag, poffset, px, pxfr, pminc, pmcode, pjac);
}

void __wrap_stiff_sh(double *pss, double *pemod, double *pnu, double *px_temp, double *pxlocal, double *pthick, double *pfarea, double *pdeffarea_ip, double *pslength, double *pdefslen_ip, double *pyield, double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pef_ip, double *pd_temp, double *pchi_temp, double *pefN_temp, double *pefM_temp, long *pmaxa, long *pminc, long *pmcode)
{
    static __typeof__(stiff_sh) *f = NULL;
    if (!f) f = (__typeof__(stiff_sh) *)resolve("stiff_sh");
    f(pss, pemod, pnu, px_temp, pxlocal, pthick, pfarea, pdeffarea_ip, pslength, pdefslen_ip, pyield, pc1_ip, pc2_ip, pc3_ip, pef_ip, pd_temp, pchi_temp, pefN_temp, pefM_temp, pmaxa, pminc, pmcode);
}

int __wrap_forces_sh(double *pf_temp, double *pef_ip, double *pef_i, double *pefN_temp, double *pefM_temp, double *pdd, double *pd_temp, double *pchi_temp, double *px_temp, double *px_ip, double *pemod, double *pnu, double *pxlocal, double *pthick, double *pfarea, double *pdeffarea_ip, double *pslength, double *pdefslen_ip, double *pyield, double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pc1_i, double *pc2_i, double *pc3_i, long *pminc, long *pmcode, long *pjcode)
{
    static __typeof__(forces_sh) *f = NULL;
    if (!f) f = (__typeof__(forces_sh) *)resolve("forces_sh");
    return f(pf_temp, pef_ip, pef_i, pefN_temp, pefM_temp, pdd, pd_temp, pchi_temp, px_temp, px_ip, pemod, pnu, pxlocal, pthick, pfarea, pdeffarea_ip, pslength, pdefslen_ip, pyield, pc1_ip, pc2_ip, pc3_ip, pc1_i, pc2_i, pc3_i, pminc, pmcode, pjcode);
}

int __wrap_solve(long *pjcode_fsi, double *pss, double *pss_fsi, double *psm, double *psm_fsi, double *psd_fsi, double *pr, double *pdd, long *pmaxa, double *pssd, int *pdet, double *pum, double *pvm, double *pam, double *puc, double *pvc, double *pac, double *pqdyn, double *ptstps, double *pKeff, double *pReff, double *pMeff, int *pAp, int *pAi, double *pAx, double alpham, double alphaf, int *pipiv, int fact, double ddt, double *ppdisp, long *pkht, int *piter, int *pii, int *pij, int tstp)
{
    static __typeof__(solve) *f = NULL;
    if (!f) f = (__typeof__(solve) *)resolve("solve");
    return f(pjcode_fsi, pss, pss_fsi, psm, psm_fsi, psd_fsi, pr, pdd, pmaxa, pssd, pdet, pum, pvm, pam, puc, pvc, pac, pqdyn, ptstps, pKeff, pReff, pMeff, pAp, pAi, pAx, alpham, alphaf, pipiv, fact, ddt, ppdisp, pkht, piter, pii, pij, tstp);
}

int __wrap_skyfact(long *pmaxa, double *pss_temp, double *pssd, double *pdd, int fact, int *pdet)
{
    static __typeof__(skyfact) *f = NULL;
    if (!f) f = (__typeof__(skyfact) *)resolve("skyfact");
    return f(pmaxa, pss_temp, pssd, pdd, fact, pdet);
}

int __wrap_skysolve(long *pmaxa, double *pss, double *pssd, double *pdd, int fact, int *pdet)
{
    static __typeof__(skysolve) *f = NULL;
    if (!f) f = (__typeof__(skysolve) *)resolve("skysolve");
    return f(pmaxa, pss, pssd, pdd, fact, pdet);
}

int __wrap_quad(double *pa, double *pb, double *pc, double *pdt, double *pdp, double *pddr, double *pddq, double *pdd, double *pdlpf, double *plpft)
{
    static __typeof__(quad) *f = NULL;
    if (!f) f = (__typeof__(quad) *)resolve("quad");
    return f(pa, pb, pc, pdt, pdp, pddr, pddq, pdd, pdlpf, plpft);
}

int __wrap_test(double *pd_temp, double *pdd, double *pf_temp, double *pfp, double *pqtot, double *pf_ip, double *pintener1, int *pconvchk, double *ptoldisp, double *ptolfor, double *ptolener)
{
    static __typeof__(test) *f = NULL;
    if (!f) f = (__typeof__(test) *)resolve("test");
    return f(pd_temp, pdd, pf_temp, pfp, pqtot, pf_ip, pintener1, pconvchk, ptoldisp, ptolfor, ptolener);
}

double __wrap_dot(double *pa, double *pb, int n)
{
    static __typeof__(dot) *f = NULL;
    if (!f) f = (__typeof__(dot) *)resolve("dot");
    return f(pa, pb, n);
}
