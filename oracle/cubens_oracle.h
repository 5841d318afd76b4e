/* CPU oracle for the CU-BENs nonlinear equilibrium-loop hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * FP64 algorithms (each function cites the reference file:line it follows).
 * The parity tests use it as the checker, and bench.py times it as the CPU
 * baseline. The product (cu-bens_gb300/) never links, loads or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks this restatement against
 * golden vectors produced by the reference's own compiled code
 * (tests/golden/make_golden.py; oracle/Makefile target "ref").
 */
#ifndef CUBENS_ORACLE_H
#define CUBENS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_model orc_model;

/* Parse a model_def.txt text (ANAFLAG 2, SLVFLAG 0, OPTFLAG 1): ALGFLAG 3
 * (MSAL) with truss, frame and DKT shell elements, or ALGFLAG 5 (nonlinear
 * Newmark) with frame elements only. Returns NULL and fills err on failure. */
orc_model *orc_load(const char *text, char *err, int errlen);
void orc_free(orc_model *m);

/* out[0..7] = NJ, NE_TR, NE_FR, NE_SH, NEQ, lss (skyline length), dkdof, itemax */
void orc_sizes(const orc_model *m, long *out);

/* ALGFLAG 5 models: number of time steps NTSTPS and dt */
void orc_dyn_sizes(const orc_model *m, long *nsteps, double *dt);

/* jcode (NJ*7, 1-based equation numbers, 0 = fixed), reference load q (NEQ) */
void orc_topology(const orc_model *m, long *jcode, double *q);

/* Modified spherical arc-length run (main.c:2158-3141). Stops after max_steps
 * converged steps or when the reference would stop. Per converged step k:
 * lam[k], its[k], d[k*NEQ ...], res[k] = |lam q - f| / |lam q|. Returns the
 * number of converged steps, or -(error code) with the reason in err. */
int orc_msal(orc_model *m, int max_steps, double *lam, int *its, double *d, double *res,
             char *err, int errlen);
/* As orc_msal, also recording the monotonic wall time (seconds) at which each
 * converged step was accepted in tstamp[k] (may be NULL); d may be NULL. */
int orc_msal_timed(orc_model *m, int max_steps, double *lam, int *its, double *d, double *res,
                   double *tstamp, char *err, int errlen);

/* Nonlinear Newmark time loop (main.c:3305-3960). Per recorded time step k:
 * time[k], its[k], d[k*NEQ ...] (d may be NULL), res[k] = |dyn - f| / |dyn|.
 * Returns the number of steps recorded, or -(error code) with err set. */
/* linear Newmark (ANAFLAG 1, ALGFLAG 4): per step the time and the displacements */
int orc_linear_newmark(orc_model *m, long max_steps, double *time, double *d, char *err, int errlen);
int orc_newmark(orc_model *m, long max_steps, double *time, int *its, double *d, double *res,
                char *err, int errlen);

/* ---- element-level entry points (state given explicitly) ---- */

/* Shell internal forces for every shell element (shell.c:1593-2400, ANAFLAG 2),
 * preceded by the geometry update of updatc (misc.c:71-185):
 *   x_temp (NJ*3) current joint coordinates; dd (NEQ) displacement increment;
 *   c_ip (NE_SH*9, rows c1,c2,c3 per element) previous-iteration triads;
 *   ef_ip (NE_SH*18) previous element forces.
 * Outputs: c_i (NE_SH*9), area_i (NE_SH), ef_i (NE_SH*18), f (NEQ, overwritten). */
void orc_shell_forces(const orc_model *m, const double *x_temp, const double *dd,
                      const double *c_ip, const double *ef_ip, double *c_i, double *area_i,
                      double *ef_i, double *f);

/* Truss internal forces (truss.c:231-378, ANAFLAG 2) with the truss part of
 * updatc: x_temp (NJ*3) -> length_i (NE_TR), dir_i (NE_TR*3), ef_i (NE_TR*2),
 * f (NEQ) accumulated (+=). */
void orc_truss_forces(const orc_model *m, const double *x_temp, double *length_i,
                      double *dir_i, double *ef_i, double *f);

/* Tangent stiffness of the whole model in the reference's 1-based skyline
 * layout (maxa, ss[lss]); stiff_tr (truss.c:82-204) + stiff_sh
 * (shell.c:110-344). State: x (NJ*3) converged coordinates, shell triads c
 * (NE_SH*9), shell areas (NE_SH), truss lengths (NE_TR), truss directions
 * (NE_TR*3), truss forces ef_tr (NE_TR*2). */
void orc_tangent(const orc_model *m, const double *x, const double *c_sh, const double *area_sh,
                 const double *len_tr, const double *dir_tr, const double *ef_tr, long *maxa,
                 double *ss);

/* Frame elements (14 DOF per member, warping included; frame.c).
 *   orc_frame_initial: initial triads c (NE_FR*9, rows x^, y^, z^) and
 *     lengths (NE_FR) from prop_fr (frame.c:130-160).
 *   orc_frame_forces: forces_fr, ANAFLAG 2 (frame.c:902-1312), preceded by the
 *     frame part of updatc (misc.c:108-147): x_temp (NJ*3) current joint
 *     coordinates, dd (NEQ), previous-iteration triads c_ip, element forces
 *     ef_ip (NE_FR*14) and deformed lengths len_ip; lref the reference
 *     lengths used by the elastic stiffness. Outputs c_i, len_i, ef_i and
 *     f (NEQ, overwritten).
 *   orc_tangent_fr: stiff_fr (frame.c:226-362) into the skyline layout.
 *   orc_frame_mass: mass_fr lumped diagonal mass (frame.c:1314-1391) at the
 *     joint coordinates x, into sm (NEQ, overwritten). */
void orc_frame_initial(const orc_model *m, double *c, double *len);
void orc_frame_forces(const orc_model *m, const double *x_temp, const double *dd, const double *c_ip,
                      const double *ef_ip, const double *len_ip, const double *lref, double *c_i,
                      double *len_i, double *ef_i, double *f);
void orc_tangent_fr(const orc_model *m, const double *c_fr, const double *ef_fr, const double *len_fr,
                    const double *lref_fr, long *maxa, double *ss);
void orc_frame_mass(const orc_model *m, const double *x, double *sm);

/* Frame member equation numbers (NE_FR*14, 1-based, 0 = fixed) */
void orc_frame_mcode(const orc_model *m, long *mc);

/* Skyline LDL^T (solve.c:539-698): factor ss in place (fact == 0), then solve
 * in place on rhs; pivots to ssd, det = 1 when any pivot <= 0. */
void orc_skyline_solve(const orc_model *m, double *ss, double *rhs, double *ssd, int *det,
                       int fact);

/* Initial shell geometry from prop_sh (shell.c:43-108): c (NE_SH*9), area (NE_SH) */
void orc_shell_initial(const orc_model *m, double *c, double *area);
/* ... and the local coordinates xlocal (NE_SH*3) and side lengths slength (NE_SH*3) */
void orc_shell_geometry0(const orc_model *m, double *xl, double *slen);

/* Quadratic root selection of the arc-length constraint (arc.c:70-157). */
int orc_quad(long neq, double a, double b, double c, double *dt, const double *dp,
             const double *ddr, const double *ddq, double *dd, double *dlpf, double *lpft);

/* Convergence test (misc.c:187-250). */
int orc_test(long neq, const double *d_temp, const double *dd, const double *f_temp,
             const double *fp, const double *qtot, const double *f_ip, double intener1,
             int *convchk, double toldisp, double tolforc, double tolener);

#ifdef __cplusplus
}
#endif
#endif
