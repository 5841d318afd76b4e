/* cubens_gb300 drop-in layer: the hot-path entry points of CU-BENs'
 * prototypes.h with the reference's own signatures, computed on the GPU.
 *
 * Library: cu-bens_gb300/lib/libcubens_dropin.so (depends on
 * libcubens_gb300.so). Sizes come from the globals that CU-BENs' main.c
 * defines (main.c:323-328: NJ, NE_TR, NE_FR, NE_SH, NEQ, NTSTPS, ANAFLAG,
 * ALGFLAG, SLVFLAG and dt); the library binds them weakly, so it also loads
 * in a process that defines them elsewhere, and its entry points report an
 * error when they are missing.
 *
 * Every call copies the arrays it reads to the GPU, runs the element,
 * factorisation or vector kernels there and copies what the reference
 * writes back into the caller's arrays, with the reference's meaning and
 * layout (element arrays concatenated by type: trusses, frames, shells).
 * Accumulating outputs (f_temp, ss, sm) are added to in the reference's
 * order. Scope: ANAFLAG 2, SLVFLAG 0, no member end offsets, releases or
 * distributed loads, no prescribed motion (NBC 0); other inputs get the
 * error return (int functions) or a message on stderr. skyfact keeps the
 * factor on the GPU keyed by the address of ss, and skysolve / solve with
 * fact = 1 reuse it while ss is the array last factored.
 *
 * This layer is for parity with the reference, one call at a time; the
 * resident API of cubens_gb300.h is the fast path.
 */
#ifndef CUBENS_GB300_DROPIN_H
#define CUBENS_GB300_DROPIN_H

#ifdef __cplusplus
extern "C" {
#endif

/* misc.c:71-185 (prototypes.h:356) */
void updatc(double *px_temp, double *px_ip, double *pxfr_temp, double *pdd, double *pdefllen_i,
            double *pdeffarea_i, double *pdefslen_i, double *poffset, int *posflag, double *pauxpt,
            double *pc1_i, double *pc2_i, double *pc3_i, long *pminc, long *pjcode);

/* truss.c:82-204 (prototypes.h:91) */
void stiff_tr(double *pss, double *pemod, double *pcarea, double *plength, double *pdefllen_ip,
              double *pyield, double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pef_ip,
              long *pmaxa, long *pmcode);

/* truss.c:231-378 (prototypes.h:100) */
void forces_tr(double *pf_temp, double *pef_i, double *pd, double *pemod, double *pcarea,
               double *pllength, double *pdefllen_i, double *pyield, double *pc1_i, double *pc2_i,
               double *pc3_i, long *pmcode);

/* frame.c:226-362 (prototypes.h:122) */
void stiff_fr(double *pss, double *pemod, double *pgmod, double *pcarea, double *poffset,
              int *posflag, double *pllength, double *pdefllen_ip, double *pistrong,
              double *piweak, double *pipolar, double *piwarp, int *pyldflag, double *pyield,
              double *pzstrong, double *pzweak, double *pc1_ip, double *pc2_ip, double *pc3_ip,
              double *pef_ip, double *pefFE_ip, int *pmendrel, long *pmaxa, long *pmcode);

/* frame.c:902-1312 (prototypes.h:149) */
int forces_fr(double *pf_temp, double *pef_ip, double *pef_i, double *pefFE_ref, double *pefFE_ip,
              double *pefFE_i, int *pyldflag, double *pdd, double *pemod, double *pgmod,
              double *pcarea, double *poffset, int *posflag, double *pllength,
              double *pdefllen_ip, double *pistrong, double *piweak, double *pipolar,
              double *piwarp, double *pyield, double *pzstrong, double *pzweak, double *pc1_ip,
              double *pc2_ip, double *pc3_ip, double *pc1_i, double *pc2_i, double *pc3_i,
              int *pmendrel, long *pmcode, double *pdlpf, int *pitecnt);

/* frame.c:1314-1391 (prototypes.h:159) */
void mass_fr(double *psm, double *pcarea, double *pllength, double *pistrong, double *piweak,
             double *pipolar, double *piwarp, double *pdens, int *posflag, double *poffset,
             double *px, double *pxfr, long *pminc, long *pmcode, double *pjac);

/* shell.c:110-344 (prototypes.h:187) */
void stiff_sh(double *pss, double *pemod, double *pnu, double *px_temp, double *pxlocal,
              double *pthick, double *pfarea, double *pdeffarea_ip, double *pslength,
              double *pdefslen_ip, double *pyield, double *pc1_ip, double *pc2_ip, double *pc3_ip,
              double *pef_ip, double *pd_temp, double *pchi_temp, double *pefN_temp,
              double *pefM_temp, long *pmaxa, long *pminc, long *pmcode);

/* shell.c:1593-2400 (prototypes.h:246) */
int forces_sh(double *pf_temp, double *pef_ip, double *pef_i, double *pefN_temp, double *pefM_temp,
              double *pdd, double *pd_temp, double *pchi_temp, double *px_temp, double *px_ip,
              double *pemod, double *pnu, double *pxlocal, double *pthick, double *pfarea,
              double *pdeffarea_ip, double *pslength, double *pdefslen_ip, double *pyield,
              double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pc1_i, double *pc2_i,
              double *pc3_i, long *pminc, long *pmcode, long *pjcode);

/* solve.c:51-533 (prototypes.h:312), the SLVFLAG 0 paths of ALGFLAG 3 and 5 */
int solve(long *pjcode_fsi, double *pss, double *pss_fsi, double *psm, double *psm_fsi,
          double *psd_fsi, double *pr, double *pdd, long *pmaxa, double *pssd, int *pdet,
          double *pum, double *pvm, double *pam, double *puc, double *pvc, double *pac,
          double *pqdyn, double *ptstps, double *pKeff, double *pReff, double *pMeff, int *pAp,
          int *pAi, double *pAx, double alpham, double alphaf, int *pipiv, int fact, double ddt,
          double *ppdisp, long *pkht, int *piter, int *pii, int *pij, int tstp);

/* solve.c:539-698 (prototypes.h:317, 320) */
int skyfact(long *pmaxa, double *pss_temp, double *pssd, double *pdd, int fact, int *pdet);
int skysolve(long *pmaxa, double *pss, double *pssd, double *pdd, int fact, int *pdet);

/* arc.c:70-157 (prototypes.h:338) */
int quad(double *pa, double *pb, double *pc, double *pdt, double *pdp, double *pddr, double *pddq,
         double *pdd, double *pdlpf, double *plpft);

/* misc.c:187-250 (prototypes.h:351) */
int test(double *pd_temp, double *pdd, double *pf_temp, double *pfp, double *pqtot, double *pf_ip,
         double *pintener1, int *pconvchk, double *ptoldisp, double *ptolfor, double *ptolener);

/* misc.c:252-262 (prototypes.h:362) */
double dot(double *pa, double *pb, int n);

#ifdef __cplusplus
}
#endif
#endif
