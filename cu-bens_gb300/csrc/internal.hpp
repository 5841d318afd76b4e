// Internal declarations shared by the host driver and the kernel files.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "cubens_gb300.h"

namespace cb {

// ---------------------------------------------------------------------------
// Host-side model: what main() builds during setup (main.c:330-1648)
// ---------------------------------------------------------------------------
// Input values the solver does not use but the reference echoes to
// results1.txt while it reads the model_def (struc model.c:381-390, prop_tr
// truss.c:48-70, prop_fr frame.c:171-181, prop_sh shell.c:51-100, load
// model.c:1316-1319, arc.c:52-53).
struct InputEcho {
    int ana = 2;
    std::vector<int> wrp;                      // NJ warping restraint flags ("j,7,r")
    std::vector<double> tr_dens, tr_yield;     // NE_TR
    std::vector<double> sh_dens, sh_yield;     // NE_SH
    std::vector<double> fr_yield;              // NE_FR*3: yield stress, plastic moduli (strong, weak)
    std::vector<long> load_jt;                 // static joint loads in input order (1-based joints)
    std::vector<int> load_dir;
    std::vector<double> load_mag;
    long dk_jt = 0;                            // MSAL initially prescribed displacement
    int dk_dir = 0;
};

struct HostModel {
    long nj = 0, ne_tr = 0, ne_fr = 0, ne_sh = 0, neq = 0, lss = 0, bw = 0;
    std::vector<long> jcode;   // NJ*7, 1-based equation numbers, 0 = fixed
    std::vector<long> maxa;    // NEQ+1, 1-based skyline diagonal addresses
    std::vector<double> x0;    // NJ*3
    std::vector<double> q;     // NEQ
    std::vector<int> tr_conn;  // NE_TR*2 (0-based joints)
    std::vector<double> tr_e, tr_a;
    std::vector<int> sh_conn;  // NE_SH*3
    std::vector<double> sh_e, sh_nu, sh_t;
    std::vector<int> fr_conn;  // NE_FR*2
    std::vector<double> fr_prop;  // NE_FR*8, per member: E, G, rho, A, I strong, I weak, J, I warping
    std::vector<double> fr_aux;   // NE_FR*3 auxiliary points
    std::vector<long> fr_mc;      // NE_FR*14 1-based equation numbers (0 = fixed), warping per member
    int alg = 3;                  // ALGFLAG: 1 NR, 2 modified NR, 3 MSAL, 4 linear Newmark, 5 nonlinear Newmark
    // nonlinear Newmark input (main.c:1600-1607, 3320-3326; load, model.c:1492-1609)
    long ntin = 0;                // input time points
    long nsteps = 0;              // NTSTPS = (long)(ttot/dt + 1)
    double dt = 0, ttot = 0, numopt = 0, spectrds = 1, lpf0 = 1, dlpf0 = 1, dlpfmax = 1, dlpfmin = 1;
    int solmin = 1;
    std::vector<double> pin;      // ntin*NEQ joint forces, time-major: pin[k*NEQ + i]
    std::vector<double> um0, vm0, am0;  // NEQ initial displacements, velocities, accelerations (ALGFLAG 4)
    // MSAL controls (arc.c:48, main.c:2240-2245)
    long dkdof = -1;
    double dk = 0, alpha = 1, psi_thresh = 0.1, lpfmax = 0, dkimax = 0;
    double toldisp = 1, tolforc = 1, tolener = 1;
    int iteopt = 6, itemax = 20, submax = 10, imagmax = 10, negmax = 10;
    InputEcho echo;
};

// The text the reference writes to results1.txt from the start of the run to
// the end of input processing (the input echo, main.c:386-433 through the
// MSAL parameters).
std::string input_echo(const HostModel &m);

// Parse a model_def text; returns an empty string on success, else the reason.
std::string parse_model_def(const char *text, size_t len, HostModel &m, int &status);

// Gather lists: out[i] = sum_{k in ptr[i]..ptr[i+1]} src[idx[k]] in list order.
struct GatherMap {
    std::vector<int> ptr;   // n+1
    std::vector<int> src;   // contributions, in the reference's accumulation order
    std::vector<int64_t> dst;  // destination slot per row (band map only)
};

// Force assembly: eq -> contributions into the per-element force buffer.
// Tangent assembly: band slot -> contributions into the per-element matrix buffer.
void build_force_map(const HostModel &m, GatherMap &g);
void build_tangent_map(const HostModel &m, long ld, GatherMap &g);

// Compressed sparse rows of the symmetric tangent, both triangles.
struct CsrPattern {
    std::vector<int> rowptr;  // n+1
    std::vector<int> col;     // nnz, ascending within a row
    std::vector<int> diag;    // n: slot of (i, i)
};
// Pattern of the assembled tangent and its gather map: g lists each lower
// pair's contributions (same order as the band map, so the sums are the
// band's values bit for bit) and writes them to g.dst (the pair) and dst2
// (its mirror, -1 on the diagonal).
void build_csr_tangent(const HostModel &m, CsrPattern &p, GatherMap &g, std::vector<int64_t> &dst2);
// Block-Jacobi blocks: start[b] .. start[b+1] are the equations of block b
// (one joint's equations, at most 8).
void build_node_blocks(const HostModel &m, std::vector<int> &start);

// ---------------------------------------------------------------------------
// Device buffers
// ---------------------------------------------------------------------------
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
};

// Shell element data, structure-of-arrays (index k*E + e).
struct DevShell {
    int *conn = nullptr;       // 3*E
    int *eq = nullptr;         // 18*E, 0-based equation or -1
    double *prop = nullptr;    // 3*E: E, nu, t
    double *xl = nullptr;      // 3*E initial local x2, x3, y3
    double *kem = nullptr;     // 36*E membrane stiffness
    double *keb = nullptr;     // 81*E bending stiffness
    double *c_c = nullptr, *c_ip = nullptr, *c_i = nullptr;     // 9*E triads
    double *a_c = nullptr, *a_i = nullptr;                      // E areas
    double *ef_c = nullptr, *ef_ip = nullptr, *ef_i = nullptr;  // 18*E element forces
};

// Frame member data, structure-of-arrays (index k*F + e).
struct DevFrame {
    int *conn = nullptr;       // 2*F
    int *eq = nullptr;         // 14*F, 0-based equation or -1
    double *prop = nullptr;    // 8*F: E, G, rho, A, I strong, I weak, J, I warping
    double *aux = nullptr;     // 3*F auxiliary points
    double *len0 = nullptr;    // F initial lengths
    double *c_c = nullptr, *c_ip = nullptr, *c_i = nullptr;        // 9*F triads (rows x^, y^, z^)
    double *ef_c = nullptr, *ef_ip = nullptr, *ef_i = nullptr;     // 14*F local element forces
    double *len_c = nullptr, *len_ip = nullptr, *len_i = nullptr;  // F deformed lengths
};

struct DevTruss {
    int *conn = nullptr;     // 2*T
    int *eq = nullptr;       // 6*T
    double *ea = nullptr;    // T: E*A
    double *len0 = nullptr;  // T
    double *len_c = nullptr, *len_i = nullptr;  // T
    double *dir_c = nullptr, *dir_i = nullptr;  // 3*T
    double *n_c = nullptr, *n_i = nullptr;      // T: axial force ef[0]
};

// Polls after which a device-side wait gives up (well over a second).
constexpr long long kDefaultWaitPolls = 1LL << 24;

// Counters of the bounded grid barrier of the persistent solve kernel.
struct GridBarrier {
    unsigned count;
    unsigned gen;
    int err;  // 1 when a wait gave up (CB_ERR_TIMEOUT)
    int pad;
};

// The band LDL^T factor in precision T and its block-bidiagonal inverse form.
struct BandFactor {
    long n = 0, bw = 0, ld = 0;  // lower band L[j*ld + (i-j)], 0 <= i-j <= bw
    long w = 0;                  // coupling width: bw rounded up to 32
    long s = 0, nblk = 0;        // block size (>= w, multiple of 32) and block count
    void *band = nullptr;        // ld * npad elements
    void *dinv = nullptr;        // npad: 1/d
    void *linv = nullptr;        // nblk * s*s: inverse of the unit-lower diagonal block (row-major)
    void *linvt = nullptr;       // nblk * s*s: its transpose (row-major)
    void *pmat = nullptr;        // nblk * s*w: Pn_i = Linv_i L_{i,i-1}[:, s-w:s] (row-major)
    void *rmat = nullptr;        // nblk * s*w: Rn_i = (L_{i+1,i}[0:w,:] Linv_i)^T (row-major)
    void *work = nullptr;        // max(3*npad, 64*bw + 32) work elements
    double *ssd = nullptr;       // n pivots (FP64 copy)
    int *flags = nullptr;        // [0] det (any pivot <= 0), [1] zero pivot seen
    GridBarrier *bar = nullptr;  // persistent-solve barrier
    GridBarrier *fbar = nullptr; // persistent-factor barrier
    void *stage = nullptr;       // 2 x 32x32: staged factored diagonal blocks (FP32 factor)
    void *look = nullptr;        // 2 x (32x32 + 32): the next panel's factored block (L, D) and 1/D
    bool fp32 = false;
    bool dw = false;             // double-word band (pairs of floats, band_dw.cu); always direct
    bool dw_simt = false;        // double-word factor: trailing update on the FP32 pipe instead of the
                                 // tensor cores (bfloat16 slices, exact FP32 accumulation)
    void *slices = nullptr;      // tensor-core factor: bfloat16 slices of the panel's W and L rows
    int *slice_exp = nullptr;    // ... and their row exponents
    bool direct = false;         // no solve blocks: substitution with the band (one solve per factor)
    int solve_grid = 1;          // CTAs of the cooperative solve launch
    int solve_grid_full = 1;     // ... when the handle has the GPU to itself
    int factor_grid = 1;         // most CTAs of the cooperative factor launch
    bool use_cluster = false;    // FP32: the cluster factor where the band's window fits
    int cluster = 0;             // CTAs of the cluster factor (0: the cooperative grid factor)
    int cluster_slots = 0, cluster_nwin = 0;
    size_t cluster_smem = 0;
    size_t bytes = 0;            // device memory held
    cudaGraphExec_t factor_graph = nullptr;
    long factor_launches = 0;
    long long max_polls = kDefaultWaitPolls;  // bound of every grid-barrier wait (< 0: give up at once)
};

// direct: the factor serves one solve (Newmark's full Newton): the solve
// substitutes with the band itself and no solve blocks are formed
// direct_block: the padding block of a direct band (0: one 32-row panel)
void band_alloc(BandFactor &f, long n, long bw, bool fp32, bool direct = false, bool use_cluster = false,
                long direct_block = 0);
void band_free(BandFactor &f);
// Double-word band (band_dw.cu): entries are pairs of floats (about 48
// significant bits), the factor and its solves run on the FP32 pipe.
// band_alloc_dw allocates the band and the block inverses of the solve; the
// tangent is gathered from FP64 element matrices by band_dw_gather.
void band_alloc_dw(BandFactor &f, long n, long bw, bool simt = false);
void band_dw_alloc(BandFactor &f);
size_t band_dw_extra_bytes(long n, long bw);
long band_dw_block();  // rows of the solve's blocks (the band is padded to a multiple)
void band_dw_gather(const int *ptr, const int *src, const int64_t *dst, const double *kel, BandFactor &f,
                    long nslots, cudaStream_t st);
void band_dw_factor(BandFactor &f, cudaStream_t st, long *launches);
void band_dw_solve(const BandFactor &f, const double *rhs, double *x, void *work, GridBarrier *bar,
                   cudaStream_t st);
// The band already holds an LDL^T factor (L below, D on the diagonal): form
// 1/d and the solve blocks so that band_solve can use it.
void band_use_factored(BandFactor &f, cudaStream_t st);
// Factor the band in place: pivots to f.ssd, det/zero flags to f.flags.
void band_factor(BandFactor &f, cudaStream_t st, bool use_graph, long *launches);
// One launch sequence for isolated timing: 3 = the persistent LDL^T of the
// band as it stands (overwrites it), 4 = the solve blocks from the factor.
void band_profile_launch(BandFactor &f, int which, cudaStream_t st);
// Handles that run concurrently (cb_batch_msal) give the block solve one warp
// per row of a block step (s/8 CTAs) instead of every SM, so that several
// handles' kernels fit at once; false restores the full grid.
void band_share_gpu(BandFactor &f, bool shared);
// FP64 effective stiffness kept beside an FP32 factor (same band layout):
// copy it into the factor's band as FP32, and r = b - K x with it (w: n
// scratch values).
void band_copy_to_f32(const double *band64, BandFactor &f, cudaStream_t st);
void band_residual64(const double *band64, long ld, long bw, long n, const double *b, const double *x, double *r,
                     double *w, cudaStream_t st);
// Bytes band_solve_with_work needs: 256 for the barrier + 3*npad work elements.
size_t band_work_bytes(const BandFactor &f);
// The solve with caller-provided work memory (band_work_bytes(f): the grid
// barrier counters, then 3*npad work elements); nothing allocated.
void band_solve_with_work(const BandFactor &f, const double *rhs, double *x, void *work,
                          cudaStream_t st);
// Solve K x = rhs with the factor (rhs, x: FP64 device vectors of length n).
void band_solve(BandFactor &f, const double *rhs, double *x, cudaStream_t st, bool use_graph,
                long *launches);

// ---------------------------------------------------------------------------
// Krylov solve (krylov.cu): restarted flexible GMRES, right-preconditioned,
// classical Gram-Schmidt applied twice, with a nodal block-Jacobi
// preconditioner over a CSR sparse matrix-vector product. The Arnoldi
// process, the Givens rotations and the restarts run on the device; the
// host replays a captured chunk of Arnoldi steps and reads a status word.
// ---------------------------------------------------------------------------
constexpr int kMaxRestart = 64;

struct KrylovCtl {
    int j;        // current Arnoldi column
    int done;     // the solve has ended (converged or gave up)
    int finish;   // the current cycle ends with this step
    int conv;     // the residual estimate met the tolerance
    int iters;    // Arnoldi steps of this solve
    int restarts;
    int status;   // 0 converged, 1 iteration limit, 2 breakdown to a non-finite value
    int ncols;    // columns of the finished cycle
    int m, maxit;
    unsigned arrive[4];  // blocks of the running pass that have finished (last-block reductions)
    double rtol, tol_abs, bnorm, beta, scale, resid;
    double hp[kMaxRestart + 1];    // coefficients of the current Gram-Schmidt pass
    double hcol[kMaxRestart + 1];  // Hessenberg column being formed
    double H[kMaxRestart * (kMaxRestart + 1)];  // rotated Hessenberg, column j at H[j*(m+1)]
    double cs[kMaxRestart], sn[kMaxRestart], g[kMaxRestart + 1], y[kMaxRestart];
};

// Preconditioner applied inside the Arnoldi step: z = P(w * scale), with
// v_j = w * scale stored as the basis vector.
enum class KrylovPrecond { block_jacobi, learned };

struct KrylovSolver {
    long n = 0, nnz = 0;
    int m = 50, maxit = 2000;
    double rtol = 1e-12;
    bool fp32_precond = false;   // block inverses in FP32 (mixed precision)
    int nred = 0;                // blocks of the Gram-Schmidt passes (fixed per model: reproducible sums)
    int rows_per_red = 0;        // rows per such block
    // matrix (FP64, both triangles)
    int *rowptr = nullptr, *col = nullptr, *diag = nullptr;
    double *val = nullptr;
    // assembly map (lower pairs -> CSR slots)
    int *amap_ptr = nullptr, *amap_src = nullptr;
    int64_t *amap_dst = nullptr, *amap_dst2 = nullptr;
    long amap_n = 0;
    // block-Jacobi
    long nblk = 0;
    int *blk_start = nullptr, *blk_off = nullptr, *row_blk = nullptr;
    void *binv = nullptr;        // per block its bs x bs inverse, row-major
    long binv_n = 0;
    // Krylov work
    double *V = nullptr, *Z = nullptr, *w = nullptr, *b = nullptr, *x = nullptr, *partial = nullptr;
    KrylovCtl *ctl = nullptr;
    KrylovCtl *ctl_h = nullptr;  // pinned host copy (the header up to hp is read per chunk)
    int chunk = 8;               // Arnoldi steps per graph replay
    cudaGraphExec_t step_graph[2] = {nullptr, nullptr};
    size_t bytes = 0;
    // nested precision (mixed): an FP32 FGMRES over FP32 copies of the matrix
    // and block inverses is the preconditioner of the FP64 FGMRES
    bool nested = false;
    int m32 = 30, maxit32 = 400;
    double rtol32 = 1e-4;
    float *valf = nullptr, *V32 = nullptr, *Z32 = nullptr, *w32 = nullptr, *b32 = nullptr, *x32 = nullptr;
    float *partial32 = nullptr;
    int nred32 = 0, rows_per_red32 = 0;
    KrylovCtl *ctl32 = nullptr, *ctl32_h = nullptr;
    cudaGraphExec_t graph32 = nullptr;
    long inner_iterations = 0;
    // learned preconditioner hook (filled by the MPNN module)
    void *mpnn = nullptr;
    // statistics
    long iterations_total = 0, solves = 0, unconverged = 0;
    int last_iters = 0;
    double last_resid = 0;
};

// fp32: mixed precision (FP32 block inverses, nested FP32 inner FGMRES)
void krylov_alloc(KrylovSolver &ks, const HostModel &h, int restart, int maxit, bool fp32, cudaStream_t st);
void krylov_free(KrylovSolver &ks);
// tangent values from the element matrices (FP64) into the CSR matrix
void krylov_assemble(KrylovSolver &ks, const double *kel, cudaStream_t st);
// Keff diagonal: val[diag[i]] += c0 sm[i] / den (the band's nm_keff arithmetic)
void krylov_shift_diag(KrylovSolver &ks, const double *sm, double c0, double den, cudaStream_t st);
// invert the nodal blocks of the current matrix (and, nested, form the FP32
// copy of the matrix)
void krylov_setup_block_jacobi(KrylovSolver &ks, cudaStream_t st);
// Solve A x = b to rtol (relative to |b|); returns the Arnoldi steps taken.
int krylov_solve(KrylovSolver &ks, const double *b, double *x, cudaStream_t st, bool use_graph,
                 KrylovPrecond pc, long *launches);
// piv = pivots of the LDL^T of every joint block's diagonal block (n values)
void krylov_block_pivots(const KrylovSolver &ks, double *piv, cudaStream_t st);
// y = A x (one CSR product; isolated timing)
void krylov_spmv(const KrylovSolver &ks, const double *x, double *y, cudaStream_t st);
// After a solve: t = z_k of the last cycle's preconditioned basis, b = A z_k
// (a (residual, correction) pair from inside the Krylov process)
void krylov_basis_pair(const KrylovSolver &ks, int k, double *b, double *t, cudaStream_t st);
// the learned preconditioner's step inside the Arnoldi sequence (mpnn.cu)
void krylov_apply_learned(KrylovSolver &ks, cudaStream_t st);

// ---------------------------------------------------------------------------
// Learned preconditioner (mpnn.cu): a message-passing network on the joint
// graph, trained online by its own forward, backward and Adam kernels.
// ---------------------------------------------------------------------------
struct Mpnn;
Mpnn *mpnn_create(const HostModel &h, unsigned seed, int capacity, cudaStream_t st);
void mpnn_destroy(Mpnn *mp);
long mpnn_param_count();
size_t mpnn_bytes(const Mpnn *mp);
long mpnn_adam_steps(const Mpnn *mp);
double mpnn_last_loss(const Mpnn *mp);
void mpnn_set_lr(Mpnn *mp, double lr);
void mpnn_set_params(Mpnn *mp, const float *theta, cudaStream_t st);
void mpnn_get_params(const Mpnn *mp, float *theta, float *grad, cudaStream_t st);
double mpnn_eval(Mpnn &mp, const KrylovSolver &ks, const double *r, const double *p, const double *t, double *z,
                 bool train, cudaStream_t st);
void mpnn_push_pair(Mpnn &mp, const double *b, const double *t, cudaStream_t st);
// the next ring slot's (b, t) buffers; mpnn_commit_pair then advances the ring
void mpnn_slot(Mpnn &mp, double **b, double **t);
void mpnn_commit_pair(Mpnn &mp);
double mpnn_train(Mpnn &mp, const KrylovSolver &ks, int steps, cudaStream_t st);

// ---------------------------------------------------------------------------
// Kernel entry points (host wrappers)
// ---------------------------------------------------------------------------
void launch_shell_setup(const DevShell &s, const double *x0, long ne, cudaStream_t st);
// lumped shell mass (mass_sh) into the element buffer layout me[k * E + e]
void launch_shell_mass(const DevShell &s, const double *x, const double *dens, double *me, long ne,
                       cudaStream_t st);
void launch_shell_forces(const DevShell &s, const double *x_t, const double *dd, double *fe,
                         long ne, cudaStream_t st);
void launch_truss_forces(const DevTruss &t, const double *x_t, double *fe, long nt,
                         cudaStream_t st);
template <typename T>
void launch_shell_tangent(const DevShell &s, const double *x_c, T *kel, long ne, cudaStream_t st);
template <typename T>
void launch_truss_tangent(const DevTruss &t, T *kel, long nt, cudaStream_t st);
void launch_frame_geometry(const DevFrame &fr, const double *x, double *c, double *len, long F,
                           cudaStream_t st);
// forces_fr with the frame part of updatc: c_i, len_i, ef_i and the element
// forces fe[k*F + e]; lref are the lengths the elastic stiffness uses
void launch_frame_forces(const DevFrame &fr, const double *x_t, const double *dd, const double *lref,
                         double *fe, long F, cudaStream_t st);
// the same with the current triads c_i[q*F + e] given instead of formed from x_t
void launch_frame_forces_given_triads(const DevFrame &fr, const double *c_i, const double *dd, const double *lref,
                                      double *fe, long F, cudaStream_t st);
template <typename T>
void launch_frame_tangent(const DevFrame &fr, const double *c, const double *ef, const double *len,
                          const double *lref, T *kel, long F, cudaStream_t st);
// lumped mass contributions me[k*F + e] at the coordinates x; lt <- member lengths
void launch_frame_mass(const DevFrame &fr, const double *x, double *lt, double *me, long F,
                       cudaStream_t st);
void launch_gather_f64(const int *ptr, const int *src, const double *in, double *out, long n,
                       cudaStream_t st);
template <typename T>
void launch_gather_band(const int *ptr, const int *src, const int64_t *dst, const T *in, T *band,
                        long nslots, cudaStream_t st);
void launch_update_coords(const int *eq_x, const double *dd, double *x_t, long neq,
                          cudaStream_t st);

// ---------------------------------------------------------------------------
// Arc-length vector algebra (vecops.cu)
// ---------------------------------------------------------------------------
// Scalars the device-side steps of one iteration exchange. The host reads
// the block back once per iteration.
struct MsalScalars {
    double dots[16];     // latest fused reductions (see the kernels for the slots)
    double lam_t;        // lpf_temp
    double lam_old;      // lpf_temp when the residual was formed (qtot = lam_old q)
    double root;         // dlpf chosen by quad
    double a, arc, lamp, qq;  // inputs of quad (set by the host)
    int psi_ge;          // psi >= psi_thresh
    int quad_status;     // 0 ok, 2 imaginary roots, 3 both gammas <= 0 (arc.c:70-157)
    int convchk;         // misc.c:187-250
    int test_err;        // a zero denominator: 1 displacements, 2 force increment, 3 energy increment
    double toldisp, tolforc, tolener, intener1;
    int intener_first;   // the test takes intener1 from this iteration's dd . (qtot - f_ip) (static NR)
};

constexpr int kRedBlocks = 148;  // fixed partial-sum grid: bit-reproducible reductions

// r = lam_t q - f; records lam_old = lam_t
void launch_residual(const double *q, const double *f, double *r, MsalScalars *sc, long n,
                     cudaStream_t st);
// dots for b, c and the quad gammas over (d_temp, dp, ddr, ddq) -> sc->dots[0..11]
void launch_quad_dots(const double *dt, const double *dp, const double *ddr, const double *ddq,
                      double *partial, MsalScalars *sc, long n, cudaStream_t st);
// quad (arc.c:70-157) on the device: root, status, lam_t += root
void launch_quad(const double *partial, MsalScalars *sc, cudaStream_t st);
// dd = ddr + root ddq; d_temp = (d_temp - dp + dd) + dp; x_t += dd (translations)
void launch_quad_update(const double *ddr, const double *ddq, const double *dp, double *dt,
                        double *dd, const int *eq_x, double *x_t, const MsalScalars *sc, long n,
                        cudaStream_t st);
// test dots (misc.c:187-250) -> sc->dots[0..6] and convchk
void launch_test(const double *dd, const double *dt, const double *dp, const double *q,
                 const double *f, const double *fp, const double *fip, double *partial,
                 MsalScalars *sc, long n, cudaStream_t st);
// generic: sc->dots[slot] = a . b (b == nullptr: a . a; diff: (a-b).(a-b))
void launch_dot(const double *a, const double *b, double *partial, MsalScalars *sc, int slot,
                long n, cudaStream_t st, bool diff = false);
// first increment corrector (main.c:2355-2370): dl = -ddr[k]/ddq[k]; lam_t += dl;
// dd = ddr + dl ddq; d += dd; x_t += dd
void launch_first_update(const double *ddr, const double *ddq, long kdof, double *d, double *dd,
                         const int *eq_x, double *x_t, MsalScalars *sc, long n, cudaStream_t st);
// psi = min(1, min_i |ssd_i / ssd_o_i|) -> sc->dots[slot]
void launch_psi(const double *ssd, const double *ssd_o, double *partial, MsalScalars *sc, int slot,
                long n, cudaStream_t st);
// y = alpha * x
void launch_scale(const double *x, double alpha, double *y, long n, cudaStream_t st);
// y += alpha * x
void launch_axpy(const double *x, double alpha, double *y, long n, cudaStream_t st);

// ---------------------------------------------------------------------------
// Nonlinear Newmark vector algebra (vecops.cu)
// ---------------------------------------------------------------------------
// qtot (predictor modes 0, 1) and Reff = residual + M-weighted inertia terms
void launch_nm_reff(int mode, double sub_dt, double lpf, double alpham, double alphaf, double a2, double a3,
                    const double *pin_km1, const double *pin_k, const double *f_temp, const double *sm,
                    const double *vc_i, const double *ac_i, double *qtot, double *reff, long n, cudaStream_t st);
// band diagonal += c0 sm / den
template <typename T>
void launch_nm_keff(T *band, long ld, const double *sm, double c0, double den, long n, cudaStream_t st);
// dd sign, d_temp, Newmark kinematics, x_temp
void launch_nm_update(double *dd, int neg, double *d_temp, const double *um, const double *vm, const double *am,
                      double *uc_i, double *vc_i, double *ac_i, double a0, double a2, double a3, double a6,
                      double a7, const int *eq_x, double *x_t, long n, cudaStream_t st);
// Linear Newmark (solve.c:246-467): the effective load of time step k,
// reff = p_k [+ c p_(k-1)] + M_eff(um, vm, am) [- c K um] with c = af / (1 - af)
// (nku = -K um, or null when af = 0), and after the solve u = uc the
// kinematics ac, vc, then (um, vm, am) <- (uc, vc, ac) and d = uc
void launch_lin_reff(int first, double alpham, double alphaf, double a0, double a2, double a3,
                     const double *pin_km1, const double *pin_k, const double *sm, const double *um,
                     const double *vm, const double *am, const double *nku, double *reff, long n, cudaStream_t st);
void launch_lin_update(const double *uc, double *um, double *vm, double *am, double *vc, double *ac, double *d,
                       double a0, double a2, double a3, double a6, double a7, long n, cudaStream_t st);
// dyn = qtot - sm ac_i, the test sums -> sc->dots[0..6], intener1 on the first
// iteration, convchk / test_err
void launch_nm_test(const double *dd, const double *dt, const double *f, const double *fp, const double *fip,
                    const double *qtot, const double *sm, const double *ac_i, double *dyn, double *partial,
                    MsalScalars *sc, int first, long n, cudaStream_t st);

}  // namespace cb
