/* cubens_gb300 — GB300 (sm_103a) implementation of the CU-BENs nonlinear
 * equilibrium-loop hot path, behind a plain C ABI.
 *
 * Two groups of entry points:
 *
 *  1. Resident API (cb_*): the model, its state and the factorisation live in
 *     GPU memory; the host drives the modified spherical arc-length (MSAL)
 *     loop of main.c:2158-3141 one converged increment at a time, or the
 *     nonlinear Newmark loop of main.c:3305-3960 one time step at a time.
 *     This is the fast path.
 *
 *  2. Drop-in API: the prototypes.h entry points of the hot path with the
 *     reference's exact signatures (host pointers, sizes through the globals
 *     NEQ, NJ, NE_TR, NE_FR, NE_SH, ANAFLAG, ALGFLAG that main.c defines),
 *     declared in cubens_gb300_dropin.h. Each call copies its arrays to the
 *     GPU and back, so main.c links against it unmodified.
 *
 * Every function returns a status code (CB_OK == 0); none calls exit().
 * Handles are not thread-safe; one handle drives one CUDA stream.
 */
#ifndef CUBENS_GB300_H
#define CUBENS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum cb_status {
    CB_OK = 0,
    CB_ERR_ARG = 1,          /* bad argument */
    CB_ERR_PARSE = 2,        /* model_def text could not be read */
    CB_ERR_CUDA = 3,         /* CUDA runtime error (no device, out of memory, launch failure) */
    CB_ERR_UNSUPPORTED = 4,  /* model feature outside the GPU path (e.g. ANAFLAG 3) */
    CB_ERR_NUMERIC = 5,      /* zero pivot, or a zero norm in the convergence test (misc.c:210-245) */
    CB_ERR_DIVERGED = 6,     /* first increment failed or subdivisions exhausted (main.c:2535, 3040) */
    CB_ERR_STATE = 7,        /* call out of order (e.g. cb_msal_step before cb_msal_begin) */
    CB_ERR_TIMEOUT = 8,      /* a bounded device-side wait gave up */
    CB_ERR_LIMIT = 9         /* a size beyond a stated maximum */
};

typedef struct cb_model cb_model;

/* Precision of the tangent, its factorisation and the per-iteration solves.
 * The internal forces, residual, arc-length algebra and state updates are
 * FP64 in both modes. */
enum cb_precision {
    CB_FP64 = 0,   /* plain path: FP64 tangent and FP64 LDL^T (parity with the reference) */
    CB_MIXED = 1,  /* FP32 tangent and FP32 LDL^T; the modified-Newton loop refines in FP64 */
    CB_FP32X2 = 2  /* FP64 tangent assembled into a band of float pairs (about 48 significant
                      bits); the LDL^T and its direct solves in double-word arithmetic on the
                      FP32 pipe. For bands whose conditioning an FP32 factor cannot carry
                      (arc-length and Newton-Raphson models; band solver) */
};

/* Linear solver of the equilibrium iterations. */
enum cb_solver {
    CB_SOLVER_BAND = 0,   /* band LDL^T in the reference's equation order (skyfact/skysolve's
                             result; pivots give det and ssd) */
    CB_SOLVER_FGMRES = 1  /* FGMRES(m) with a nodal block-Jacobi preconditioner over a CSR
                             product, for nonlinear Newmark and MSAL models (not for static
                             Newton-Raphson). MSAL takes det from the sign of q . K^-1 q and
                             psi from the pivots of the joints' diagonal blocks. In
                             CB_MIXED precision each FP64 Arnoldi step is preconditioned by
                             an FP32 FGMRES(30) solve to 1e-4 with FP32 matrix and blocks */
};

/* Preconditioner of the FGMRES solver. */
enum cb_precond {
    CB_PRECOND_BLOCK_JACOBI = 0,  /* inverse of each joint's diagonal block */
    CB_PRECOND_LEARNED = 1        /* mesh message-passing network, trained online on the
                                     solver's own (residual, correction) pairs; block-Jacobi
                                     FGMRES takes over whenever it stalls */
};

typedef struct {
    int precision;       /* enum cb_precision */
    int device;          /* CUDA device ordinal */
    int use_graphs;      /* 1: replay the factor, solve and Arnoldi launch sequences as CUDA graphs */
    int solver;          /* enum cb_solver */
    int krylov_restart;  /* FGMRES restart length m (0: 50; at most 64) */
    int krylov_maxit;    /* FGMRES steps per solve before it gives up (0: 2000) */
    int precond;         /* enum cb_precond (FGMRES) */
    int factor_kernel;   /* band LDL^T in FP32: 0 the cooperative grid factor; 1 the
                            thread-block-cluster factor where the band's window fits a cluster's
                            distributed shared memory (measured slower on GB300: the grid factor
                            stays the default). In CB_FP32X2: 0 the trailing update on the
                            tensor cores (six bfloat16 slices per value, exact FP32
                            accumulation); 1 on the FP32 pipe in double-word arithmetic */
    int band_solve;      /* band LDL^T solves: 0 (default) block-bidiagonal solve with the
                            factor's block inverses for arc-length and modified Newton-Raphson
                            models, direct substitution for the others; 1 direct substitution
                            with the band for every model (no block inverses are formed) */
} cb_options;

typedef struct {
    long nj, ne_tr, ne_fr, ne_sh;  /* joints and elements per type */
    long neq;                      /* equations (codes, model.c:937-961) */
    long lss;                      /* reference skyline length (skylin, model.c:1264-1277) */
    long bandwidth;                /* max column height of the skyline */
    long block;                    /* block size of the block-bidiagonal solve */
    long nblocks;
    long dkdof;                    /* 0-based DOF of the prescribed displacement */
    size_t device_bytes;           /* GPU memory held by the handle */
    size_t h2d_bytes;              /* bytes copied host -> device when the model was created */
    int algflag;                   /* 1, 2: static (modified) Newton-Raphson, 3: MSAL, 5: nonlinear Newmark */
    long nsteps;                   /* Newmark: time steps NTSTPS (main.c:3361) */
    double dt;                     /* Newmark: time step */
    int solver;                    /* enum cb_solver in use */
    long nnz;                      /* FGMRES: stored entries of the CSR matrix (both triangles) */
    long node_blocks;              /* FGMRES: block-Jacobi blocks */
    int factor_cluster;            /* band LDL^T: CTAs of the thread-block-cluster factor (0: the
                                      cooperative grid factor) */
} cb_info;

/* Result of one converged increment or time step (what output() records,
 * misc.c:402-417). For Newmark steps lam is the time k dt, attempts the
 * load-factor passes tried, residual |dyn - f| / |dyn| with dyn = qtot - M a,
 * and dk 0. */
typedef struct {
    double lam;            /* load proportionality factor (Newmark: time) */
    int iterations;        /* itecnt at acceptance */
    int attempts;          /* increments tried (1 + arc-length cuts) */
    double residual;       /* |lam q - f| / |lam q| of the accepted state (FP64) */
    double dk;             /* displacement at the control DOF */
    int done;              /* 1: |lam| > lpfmax or |d_k| > dkimax (main.c:2647), or the last
                              time step was taken; no step was taken by this call */
} cb_step;

/* Per-kernel-class GPU time (ms, CUDA events on the handle's stream) and
 * launch count since the last reset. */
typedef struct {
    double ms_tangent, ms_factor, ms_solve, ms_force, ms_vector;
    long launches;
    long solves, factorizations, force_evals;
    double ms_train;  /* learned preconditioner: training (forward, backward, Adam) */
} cb_timers;

/* ---- resident API -------------------------------------------------------- */

int cb_default_options(cb_options *opt);

/* Parse a model_def.txt text and upload the model: ANAFLAG 2, SLVFLAG 0,
 * OPTFLAG 1; ALGFLAG 3 (MSAL) with truss, frame and DKT shell elements, or
 * ALGFLAG 5 (nonlinear Newmark) with frame elements. Replaces the setup part
 * of main() (main.c:330-1648: struc, codes, skylin, prop_tr, prop_fr,
 * prop_sh, load, msal). */
int cb_model_create(const char *model_def, size_t len, const cb_options *opt, cb_model **out);
int cb_model_destroy(cb_model *m);
int cb_model_info(const cb_model *m, cb_info *info);
/* Last error message of this handle (static storage owned by the handle). */
const char *cb_last_error(const cb_model *m);

/* First increment: Bathe-Dvorkin displacement control at the prescribed DOF
 * (main.c:2296-2560). */
int cb_msal_begin(cb_model *m, cb_step *out);
/* One converged arc-length increment (main.c:2647-3134). */
int cb_msal_step(cb_model *m, cb_step *out);
/* Current converged displacements d (NEQ) and lambda. */
int cb_get_displacements(const cb_model *m, double *d, double *lam);

/* Batched analyses: runs cb_msal_begin and steps - 1 cb_msal_step on each
 * of n independent handles (each created on its own, e.g. the panels of an
 * imperfection sweep) from a pool of `threads` host threads; the handles'
 * streams overlap on the GPU. out holds n * steps records (handle i's step k
 * at out[i * steps + k]; records after a stop have done = 1); status (may be
 * NULL) gets each handle's return code. Returns CB_OK or the first failing
 * handle's code. The handles must be distinct and not used by others
 * meanwhile. */
int cb_batch_msal(cb_model **models, int n, int steps, int threads, cb_step *out, int *status);

/* Static Newton-Raphson (ALGFLAG 1) and modified Newton-Raphson (ALGFLAG 2)
 * under load control (main.c:1820-2157). cb_newton_begin sets the undeformed
 * state (main.c:1672-1711); each cb_newton_step runs the passes of
 * main.c:1822-2150 until one load increment converges (subdivisions
 * included) and returns CB_OK with its record (lam = lpf), or out->done = 1
 * once lpf has passed lpfmax. Errors: CB_ERR_DIVERGED for the reference's
 * "maximum allowable load proportionality factor attempted without
 * convergence", "minimum allowable increment of load proportionality factor
 * reached" and "maximum allowable number of subdivisions exceeded";
 * CB_ERR_NUMERIC for a zero pivot or a zero norm in the test. */
int cb_newton_begin(cb_model *m);
int cb_newton_step(cb_model *m, cb_step *out);

/* Nonlinear Newmark (ALGFLAG 5, frame models). cb_newmark_begin sets the
 * initial state of main.c:3398-3447 (zero motion); each cb_newmark_step runs
 * one time step k of main.c:3449-3953 (load-factor passes and time-increment
 * halving included) and returns CB_OK with out->done = 1 once all NTSTPS
 * steps are taken. cb_get_displacements then returns d; cb_newmark_state
 * the displacement, velocity and acceleration (NEQ each; any may be NULL).
 * Linear Newmark models (ANAFLAG 1 with ALGFLAG 4, frame-only or shell-only,
 * FP64 band) use the
 * same calls: cb_newmark_begin forms the stiffness of the initial state and
 * the lumped mass and factors the effective stiffness once (main.c:3143-3302,
 * solve.c:139-222); each cb_newmark_step solves one time step k of
 * solve.c:246-467 from the model's initial conditions on. */
int cb_newmark_begin(cb_model *m);
int cb_newmark_step(cb_model *m, cb_step *out);
int cb_newmark_state(const cb_model *m, double *u, double *v, double *a);
/* Reference load vector q (NEQ) and 1-based equation numbers jcode (NJ*7). */
int cb_get_topology(const cb_model *m, long *jcode, double *q);

/* FGMRES controls and counters. The tolerance is relative to |b| for each
 * solve (default 1e-12: the Newton iteration counts of the direct solve). */
typedef struct {
    long solves;          /* FGMRES solves since the handle was created */
    long iterations;      /* Arnoldi steps over those solves */
    long unconverged;     /* solves that hit krylov_maxit */
    int last_iterations;  /* Arnoldi steps of the latest solve */
    double last_residual; /* |b - A x| / |b| estimate of the latest solve */
    long learned_solves;  /* solves preconditioned by the network */
    long fallbacks;       /* network solves that stalled and were redone with block-Jacobi */
    long train_steps;     /* Adam steps taken by the network */
    double train_loss;    /* latest training loss (relative squared error) */
    long inner_iterations; /* mixed precision: Arnoldi steps of the FP32 inner solves */
} cb_krylov_stats;
int cb_set_krylov_tolerance(cb_model *m, double rtol);
int cb_get_krylov_stats(const cb_model *m, cb_krylov_stats *s);

/* Learned preconditioner (solver CB_SOLVER_FGMRES, precond CB_PRECOND_LEARNED).
 * Online schedule: the time steps (MSAL: arc-length increments) k <
 * train_steps solve with block-Jacobi and store each solve's (right-hand
 * side, FP64 solution) pair; after
 * each such solve the network takes adam_per_solve Adam steps (learning rate
 * lr) on the stored pairs. Later solves use the network; one that has not
 * converged after stall_factor times the block-Jacobi average of Arnoldi
 * steps (at least 10) is redone with block-Jacobi. train_steps < 0 keeps the
 * default (Newmark: a tenth of the time steps, at least one; MSAL: 5). */
int cb_set_learning(cb_model *m, int train_steps, int adam_per_solve, double lr, double stall_factor);
/* The network itself, for checks against a CPU definition. Parameters are
 * cb_mpnn_param_count() float32 values (layout in cu-bens_gb300/csrc/mpnn.cu).
 * cb_mpnn_eval runs the network on host vectors r and p (NEQ; p stands for
 * the block-Jacobi image of r) into z (may be NULL); with t (may be NULL) it
 * also forms the loss |z - t|^2 / |t|^2 and the parameter gradient, and with
 * train = 1 takes one Adam step with it. */
long cb_mpnn_param_count(void);
int cb_mpnn_set_params(cb_model *m, const float *theta);
int cb_mpnn_get_params(const cb_model *m, float *theta, float *grad);
int cb_mpnn_eval(cb_model *m, const double *r, const double *p, const double *t, int train, double *z,
                 double *loss);

/* results*.txt writers (output(), misc.c:345-451). cb_results_open creates
 * dir/results2.txt (displacements), results3.txt (truss forces),
 * results4.txt (frame forces) and results5.txt (shell forces) with the
 * reference's layout lines; cb_results_write appends the current converged
 * state as one record (lam: the load factor or time, iterations: itecnt),
 * element forces averaged over the element's nodes as output() does;
 * cb_results_close closes them (cb_model_destroy does too). It also writes
 * dir/results1.txt: the reference's echo of the model_def and then the
 * run's messages as they occur (errors, reduced Newmark time increments,
 * the closing "Solution successful" or "Solution failed"). */
int cb_results_open(cb_model *m, const char *dir);
int cb_results_write(cb_model *m, double lam, int iterations);
int cb_results_close(cb_model *m);
/* The input echo of results1.txt for a model_def text, without a GPU: the
 * text the reference writes while it reads the file. Writes at most cap - 1
 * bytes and a terminating zero into buf (may be NULL) and the full length
 * into *needed (may be NULL); returns the parser's status. */
int cb_input_echo(const char *text, size_t len, char *buf, size_t cap, size_t *needed);

/* Checkpoint and restart of the nonlinear Newmark driver (checkPoint and
 * restartStep, misc.c:494-716). cb_checkpoint_save writes the converged
 * state after the last completed time step to a binary file, bit for bit:
 * velocities, accelerations, mass, d, f, coordinates, triads, deformed
 * lengths and element forces, the next step and the time increment
 * multiplier. cb_checkpoint_load, on a handle of the same model after
 * cb_newmark_begin, restores it, and the following cb_newmark_step calls
 * continue exactly as the uninterrupted run. The learned preconditioner's
 * network is not part of the state. Errors: CB_ERR_UNSUPPORTED for other
 * drivers, CB_ERR_STATE before cb_newmark_begin, CB_ERR_ARG when the file
 * cannot be opened or written or belongs to a model of other sizes,
 * CB_ERR_PARSE for a file of another format or a truncated one (the handle
 * is unchanged then). */
int cb_checkpoint_save(cb_model *m, const char *path);
int cb_checkpoint_load(cb_model *m, const char *path);

int cb_get_timers(const cb_model *m, cb_timers *t);
int cb_reset_timers(cb_model *m);
/* Enable/disable per-phase CUDA-event timing (adds event records). */
int cb_set_timing(cb_model *m, int on);

/* Bound of every device-side wait of the handle's persistent kernels (the
 * grid barriers of the band LDL^T and of the solves): a CTA that has polled
 * `polls` times without seeing the other CTAs arrive records a timeout and
 * the kernel returns early; the call that launched it then returns
 * CB_ERR_TIMEOUT and the handle stays usable. polls = 0 restores the
 * default (2^24 polls, well over a second); polls < 0 makes a CTA that is
 * not the last to arrive give up at once (for tests of the timeout path). */
int cb_set_wait_limit(cb_model *m, long long polls);

/* Convergence history of the latest first increment or arc-length increment:
 * for each iteration (attempts of cut increments included, in order) three
 * doubles, the load factor, |dd| / |d| and the FP64 equilibrium residual
 * |lam q - f| / |lam q| after the iteration. Copies at most max_iters
 * iterations into out (may be NULL) and the number recorded into *n. */
int cb_get_iteration_log(const cb_model *m, double *out, int max_iters, int *n);

/* ---- measurement hooks ---- */

/* Record CUDA event `slot` (0..7) on the handle's stream. */
int cb_event_mark(cb_model *m, int slot);
/* Milliseconds between two recorded events (waits for event b). */
int cb_event_elapsed(cb_model *m, int a, int b, double *ms);

/* Kernels that cb_profile_kernel times in isolation. */
enum cb_kernel_id {
    CB_K_SOLVE = 0,        /* one solve: the persistent block-bidiagonal solve kernel */
    CB_K_SHELL_FORCE = 1,  /* the DKT internal-force kernel over all shell elements */
    CB_K_FACTOR = 2,       /* one whole band LDL^T + block inverses (graph replay) */
    CB_K_BAND_LDLT = 3,    /* the persistent band LDL^T kernel alone (refactors the band in place) */
    CB_K_SOLVE_BLOCKS = 4, /* Linv, Pn, Rn of the solve from the current factor */
    CB_K_FRAME_FORCE = 5,  /* the frame internal-force kernel over all members */
    CB_K_SPMV = 6          /* FGMRES: one CSR product y = A x of the current matrix */
};
/* Launch kernel `which` reps times back to back between two CUDA events and
 * report the mean milliseconds per launch and the algorithmic bytes and
 * flops of one launch. Timing a factor-modifying kernel leaves the handle's
 * factorisation invalid until the next step refactors. */
int cb_profile_kernel(cb_model *m, int which, int reps, double *ms_per_launch,
                      double *bytes_per_launch, double *flops_per_launch);

/* ---- element-level resident entry points (used by the parity tests) ---- */

/* Geometry update (updatc, misc.c:71-185) and internal forces of all
 * elements (forces_tr truss.c:231-378, forces_sh shell.c:1593-2400) for an
 * explicit state. Host arrays in the reference's layouts:
 *   x_temp   NJ*3  coordinates after the increment dd
 *   dd       NEQ   displacement increment
 *   c_ip     NE_SH*9 previous-iteration shell triads (rows c1, c2, c3)
 *   ef_ip    NE_SH*18 previous-iteration shell element forces
 * Outputs: c_i (NE_SH*9), area_i (NE_SH), ef_i (NE_SH*18), truss ef_tr
 * (NE_TR*2), f (NEQ). */
int cb_eval_forces(cb_model *m, const double *x_temp, const double *dd, const double *c_ip,
                   const double *ef_ip, double *c_i, double *area_i, double *ef_i,
                   double *ef_tr, double *f);

/* Tangent stiffness (stiff_tr truss.c:82-204, stiff_sh shell.c:110-344) at
 * an explicit converged state, assembled on the GPU and returned in the
 * reference's 1-based skyline layout (maxa, ss[lss]). State: x (NJ*3),
 * c_sh (NE_SH*9), area_sh (NE_SH), ef_tr (NE_TR*2). */
int cb_eval_tangent(cb_model *m, const double *x, const double *c_sh, const double *area_sh,
                    const double *ef_tr, long *maxa, double *ss);

/* Frame element entry points (frame-only models), arrays element-major:
 *   cb_eval_frame_forces: forces_fr (frame.c:902-1312) with the frame part of
 *     updatc (misc.c:108-147): x_temp (NJ*3), dd (NEQ), c_ip (NE_FR*9, rows
 *     x^, y^, z^), ef_ip (NE_FR*14), len_ip and lref (NE_FR: deformed length
 *     of the previous iteration, reference length) -> c_i, len_i, ef_i, and
 *     f (NEQ, overwritten). Outputs other than f may be NULL.
 *   cb_eval_frame_tangent: stiff_fr (frame.c:226-362) of the state (c, ef,
 *     len, lref) into the reference's skyline layout (maxa, ss[lss]).
 *   cb_eval_frame_mass: mass_fr (frame.c:1314-1391) lumped mass at the joint
 *     coordinates x into sm (NEQ, overwritten); len (NE_FR, may be NULL) gets
 *     the member lengths at x.
 * They overwrite the handle's iteration state; call them between analyses. */
int cb_eval_frame_forces(cb_model *m, const double *x_temp, const double *dd, const double *c_ip,
                         const double *ef_ip, const double *len_ip, const double *lref, double *c_i,
                         double *len_i, double *ef_i, double *f);
int cb_eval_frame_tangent(cb_model *m, const double *c, const double *ef, const double *len,
                          const double *lref, long *maxa, double *ss);
int cb_eval_frame_mass(cb_model *m, const double *x, double *sm, double *len);

/* Factor the tangent last assembled by cb_eval_tangent and solve K v = rhs
 * (skyfact/skysolve, solve.c:539-698). Outputs v (NEQ), the LDL^T pivots ssd
 * (NEQ) and det (1 when any pivot <= 0). */
int cb_factor_solve(cb_model *m, const double *rhs, double *v, double *ssd, int *det);

/* ---- allocation-free solve ---------------------------------------------- */

/* Solve K x = rhs with the factorisation the handle currently holds (from
 * the last arc-length increment, or from cb_factor_solve), allocating no GPU
 * memory. No counterpart in the reference: it serves callers that cannot
 * call cudaMalloc where they need the solve, such as a host application
 * whose allocator or fixed pool already owns the GPU's memory, or a loop
 * whose memory footprint must not change after start-up. rhs and x are
 * device pointers to NEQ doubles.
 *
 * The solve's three work vectors and its grid-barrier counters live in one
 * static device array of 3 x 524288 doubles plus 256 bytes (12 MiB), held by
 * every GPU that loads the library until the process exits; FP64 factors of
 * more than 524288 padded equations (FP32 factors of more than 1048576) get
 * CB_ERR_LIMIT. The first call on a device
 * looks up that array's device address (cudaGetSymbolAddress with the device
 * current) and keeps it; make that first call before any stream capture, and
 * do not use the entry point after a cudaDeviceReset. All calls share the
 * array, which keeps the last call's contents: each call clears the barrier
 * counters before its launch (every work element is written before it is
 * read), and calls that overlap on the GPU race with each other. The call is
 * ordered on the handle's stream and returns when the solve has finished;
 * CB_ERR_TIMEOUT when a grid-barrier wait of the solve gave up (x is then
 * incomplete). */
int cb_solve_noalloc(cb_model *m, const double *rhs, double *x);

#ifdef __cplusplus
}
#endif
#endif
