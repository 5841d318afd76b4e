// GPU-resident nonlinear Newmark driver (ALGFLAG 5) for frame models, and
// the element-level C ABI of the frame kernels.
//
// The host keeps the scalar control flow of main.c:3305-3960: the time-step
// loop, the load-factor loop inside a time step (lpf, dlpf, solmin, subcnt)
// and the halving of the time increment (ddt, sub_dt, tsflag), including its
// oddities. Every iteration is a full Newton iteration as in the reference:
// the tangent is formed from the previous iteration's element state, the
// lumped mass at the converged coordinates, Keff = K + a0 (1 - am)/(1 - af) M
// is factored on the GPU and solved for the effective residual. The host
// reads one small scalar block back per iteration.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "cubens_gb300.h"
#include "internal.hpp"
#include "model.hpp"

namespace drv {

// K x = rhs with FGMRES on the handle's current matrix and block-Jacobi
// preconditioner. With the learned preconditioner: while `training`, solve
// with block-Jacobi and train the network on the solve's (rhs, x) pair and
// three pairs from inside its last Arnoldi cycle; afterwards solve with the
// network, capped at stall_factor times the block-Jacobi average of Arnoldi
// steps, and redo a stalled solve with block-Jacobi.
void krylov_solve_learned(cb_model *m, const double *rhs, double *x, bool training)
{
    cb::KrylovSolver &ks = *m->ks;
    const bool graphs = m->opt.use_graphs != 0;
    auto bj_solve = [&] {
        PhaseTimer t(m, &m->tm.ms_solve);
        const int it = cb::krylov_solve(ks, rhs, x, m->st, graphs, cb::KrylovPrecond::block_jacobi,
                                        &m->tm.launches);
        m->tm.solves++;
        return it;
    };
    if (!m->mp) {
        bj_solve();
        return;
    }
    if (training) {
        // the block-Jacobi work per solve: Arnoldi steps, inner ones included
        const long inner0 = ks.inner_iterations;
        m->bj_iters += bj_solve() + (ks.inner_iterations - inner0);
        m->bj_solves++;
        PhaseTimer t(m, &m->tm.ms_train);
        // the solve's own pair and three from inside its last Arnoldi cycle
        // (the vectors the preconditioner is applied to)
        cb::mpnn_push_pair(*m->mp, rhs, x, m->st);
        const int nc = ks.ctl_h->ncols;
        for (int k : {0, nc / 2, nc - 1}) {
            if (k < 0 || nc <= 0) continue;
            double *b = nullptr, *tt = nullptr;
            cb::mpnn_slot(*m->mp, &b, &tt);
            cb::krylov_basis_pair(ks, k, b, tt, m->st);
            cb::mpnn_commit_pair(*m->mp);
        }
        cb::mpnn_train(*m->mp, ks, m->learn_adam, m->st);
        return;
    }
    const double avg = m->bj_solves ? (double)m->bj_iters / (double)m->bj_solves : (double)ks.maxit;
    const int cap = std::max(10, (int)(m->learn_stall * avg));
    const int saved = ks.maxit;
    ks.maxit = std::min(cap, saved);
    {
        PhaseTimer t(m, &m->tm.ms_solve);
        cb::krylov_solve(ks, rhs, x, m->st, graphs, cb::KrylovPrecond::learned, &m->tm.launches);
        m->tm.solves++;
    }
    ks.maxit = saved;
    m->learned_solves++;
    if (ks.ctl_h->status == 1) {
        // stalled: the unconverged count is the fallback's business
        ks.unconverged--;
        m->fallbacks++;
        bj_solve();
    }
}

}  // namespace drv

namespace {

using namespace drv;

// Most refinement steps of a mixed-precision Newmark solve. Each FP32 solve
// of the frame building's effective stiffness gains one to two digits, so a
// solve needs several corrections to reach the FP64 solution that keeps the
// full Newton iteration counts of the FP64 path.
constexpr int kRefineSteps = 12;

struct NewmarkParams {
    double alpham = 0, alphaf = 0, alpha = 0.25, delta = 0.5;
};

// main.c:3329-3343
NewmarkParams newmark_params(const cb::HostModel &h)
{
    NewmarkParams p;
    if (h.numopt == 1) {
        p.alpham = (2 * h.spectrds - 1) / (h.spectrds + 1);
        p.alphaf = h.spectrds / (h.spectrds + 1);
    } else if (h.numopt == 2) {
        p.alphaf = (1 - h.spectrds) / (1 + h.spectrds);
    } else if (h.numopt == 3) {
        p.alpham = (h.spectrds - 1) / (h.spectrds + 1);
    }
    p.alpha = std::pow(1 - p.alpham + p.alphaf, 2) / 4;
    p.delta = 0.5 - p.alpham + p.alphaf;
    return p;
}

void push_test_controls(cb_model *m)
{
    cb::MsalScalars &s = *m->sc_h;
    std::memset(&s, 0, sizeof s);
    s.toldisp = m->h.toldisp;
    s.tolforc = m->h.tolforc;
    s.tolener = m->h.tolener;
    s.convchk = 1;
    h2d(m->sc, m->sc_h, 1, m->st);
}

// initial state (main.c:3398-3447): zero displacements, forces, motion;
// deformed lengths = undeformed; the frame lengths llength_temp = L0
void newmark_begin(cb_model *m)
{
    const cb::HostModel &h = m->h;
    const long N = h.neq, F = h.ne_fr, NJ = h.nj;
    cudaStream_t st = m->st;
    for (double *v : {m->d, m->f, m->uc, m->vc, m->ac, m->sm})
        CB_CUDA(cudaMemsetAsync(v, 0, N * sizeof(double), st));
    d2d(m->x_c, m->x0, NJ * 3, st);
    if (F) {
        cb::launch_frame_geometry(m->fr, m->x0, m->fr.c_c, m->fr.len_c, F, st);
        CB_CUDA(cudaMemsetAsync(m->fr.ef_c, 0, 14 * F * sizeof(double), st));
        d2d(m->fr_lref, m->fr.len0, F, st);
    }
    push_test_controls(m);
    CB_CUDA(cudaStreamSynchronize(st));
    m->nm_k = 0;
    m->nm_ddt = 1;
    m->nm_phase = 1;
}

// Keff dd = Reff with FGMRES: the preconditioner from the current matrix,
// then the solve (m->r -> m->dd). With the learned preconditioner the first
// time steps train the network (drv::krylov_solve_learned).
void krylov_newmark_solve(cb_model *m)
{
    cb::KrylovSolver &ks = *m->ks;
    {
        PhaseTimer t(m, &m->tm.ms_factor);
        cb::krylov_setup_block_jacobi(ks, m->st);
        m->tm.launches += 1;
        m->tm.factorizations++;
    }
    const long train = m->learn_steps >= 0 ? m->learn_steps : std::max(1L, m->h.nsteps / 10);
    krylov_solve_learned(m, m->r, m->dd, m->nm_k < train);
}

// one Newton iteration of main.c:3543-3745; returns the scalar block
cb::MsalScalars &newmark_iteration(cb_model *m, const NewmarkParams &p, long k, double sub_dt, double lpf,
                                   int itecnt, double a0, double a2, double a3, double a6, double a7)
{
    const cb::HostModel &h = m->h;
    const long N = h.neq, F = h.ne_fr;
    cudaStream_t st = m->st;
    // tangent of the previous iteration's state with llength_temp as it
    // stands, then the mass at the converged coordinates, which rewrites
    // llength_temp (mass_fr, frame.c:1339)
    cb::KrylovSolver *ks = m->ks;
    const bool refine = !ks && m->bf.fp32;
    if (ks) {
        // FGMRES: FP64 tangent into the CSR matrix
        PhaseTimer t(m, &m->tm.ms_tangent);
        const cb::DevFrame &fr = m->fr;
        cb::launch_frame_tangent<double>(fr, fr.c_ip, fr.ef_ip, fr.len_ip, m->fr_lref, (double *)m->kel, F, st);
        cb::krylov_assemble(*ks, (const double *)m->kel, st);
        m->tm.launches += 2;
    } else if (refine) {
        // mixed: the effective stiffness is assembled in FP64 and kept; its
        // FP32 copy is factored and the solve refined against it
        PhaseTimer t(m, &m->tm.ms_tangent);
        const cb::DevFrame &fr = m->fr;
        CB_CUDA(cudaMemsetAsync(m->band64, 0, sizeof(double) * (size_t)m->bf.ld * m->bf.nblk * m->bf.s, st));
        cb::launch_frame_tangent<double>(fr, fr.c_ip, fr.ef_ip, fr.len_ip, m->fr_lref, m->kel64, F, st);
        cb::launch_gather_band<double>(m->tmap_ptr, m->tmap_src, m->tmap_dst, m->kel64, m->band64, m->tmap_n, st);
        m->tm.launches += 3;
    } else {
        assemble_tangent(m, TangentState::previous_iteration);
    }
    {
        PhaseTimer t(m, &m->tm.ms_tangent);
        cb::launch_frame_mass(m->fr, m->x_c, m->fr_lref, m->me, F, st);
        cb::launch_gather_f64(m->fmap_ptr, m->fmap_src, m->me, m->sm, N, st);
        m->tm.launches += 2;
    }
    {
        PhaseTimer t(m, &m->tm.ms_vector);
        const int mode = itecnt > 0 ? 2 : (k == 0 ? 0 : 1);
        const double *pin_k = m->pin + (size_t)k * N;
        const double *pin_km1 = k > 0 ? m->pin + (size_t)(k - 1) * N : pin_k;
        cb::launch_nm_reff(mode, sub_dt, lpf, p.alpham, p.alphaf, a2, a3, pin_km1, pin_k, m->fcur, m->sm, m->vc_i,
                           m->ac_i, m->qtot, m->r, N, st);
        const double c0 = a0 * (1 - p.alpham), den = 1 - p.alphaf;
        if (ks) {
            cb::krylov_shift_diag(*ks, m->sm, c0, den, st);
        } else if (refine) {
            cb::launch_nm_keff<double>(m->band64, m->bf.ld, m->sm, c0, den, N, st);
            cb::band_copy_to_f32(m->band64, m->bf, st);
            m->tm.launches += 1;
        } else if (m->bf.fp32) {
            cb::launch_nm_keff<float>((float *)m->bf.band, m->bf.ld, m->sm, c0, den, N, st);
        } else {
            cb::launch_nm_keff<double>((double *)m->bf.band, m->bf.ld, m->sm, c0, den, N, st);
        }
        m->tm.launches += 2;
    }
    if (ks) {
        krylov_newmark_solve(m);
    } else {
        factor(m);
        solve(m, m->r, m->dd);
    }
    if (refine) {
        // iterative refinement: dd += K32^-1 (Reff - K64 dd) until the
        // correction is below 1e-12 of dd (at most kRefineSteps corrections)
        for (int it = 0; it < kRefineSteps; ++it) {
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::band_residual64(m->band64, m->bf.ld, m->bf.bw, N, m->r, m->dd, m->ref_r, m->ref_w, st);
                m->tm.launches += 2;
            }
            solve(m, m->ref_r, m->ref_x);
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::launch_axpy(m->ref_x, 1.0, m->dd, N, st);
                m->tm.launches += 1;
            }
            const double cx = device_dot(m, m->ref_x, nullptr), xx = device_dot(m, m->dd, nullptr);
            if (!(cx > 1e-24 * xx)) break;
        }
    }
    std::swap(m->fcur, m->fprev);  // f_ip = f_temp
    {
        PhaseTimer t(m, &m->tm.ms_vector);
        cb::launch_nm_update(m->dd, itecnt > 0, m->dt, m->um, m->vm, m->am, m->uc_i, m->vc_i, m->ac_i, a0, a2, a3,
                             a6, a7, m->eq_x, m->x_t, N, st);
        m->tm.launches += 1;
    }
    internal_force(m, m->dd, m->fcur);
    {
        PhaseTimer t(m, &m->tm.ms_vector);
        cb::launch_nm_test(m->dd, m->dt, m->fcur, m->fp, m->fprev, m->qtot, m->sm, m->ac_i, m->dyn, m->partial,
                           m->sc, itecnt == 0, N, st);
        m->tm.launches += 2;
    }
    return pull_scalars(m);
}

// one time step k of main.c:3449-3953
void newmark_step(cb_model *m, cb_step *out)
{
    const cb::HostModel &h = m->h;
    const long N = h.neq;
    cudaStream_t st = m->st;
    out->done = 0;
    if (m->nm_k >= h.nsteps) {
        ref_success(m, "\nSolution successful!!\n");  // main.c:3956-3958
        out->done = 1;
        out->lam = (double)(h.nsteps - 1) * h.dt;
        out->iterations = 0;
        out->attempts = 0;
        out->residual = 0;
        out->dk = 0;
        return;
    }
    const long k = m->nm_k;
    const NewmarkParams p = newmark_params(h);
    const double dt = h.dt, lpfmax = h.lpfmax;
    double ddt = m->nm_ddt;
    double dt_temp = ddt * dt, sub_dt = ddt, tsflag = 0;
    int convchk = 1, itecnt = 0, passes = 0;
    double res_num = 0, res_den = 0;
    do {
        const double a0 = 1 / (p.alpha * std::pow(dt_temp, 2));
        const double a2 = 1 / (p.alpha * dt_temp);
        const double a3 = 1 / (2 * p.alpha) - 1;
        const double a6 = (dt_temp) * (1 - p.delta);
        const double a7 = p.delta * (dt_temp);
        int solcnt = 0, subcnt = 0;
        double lpf = h.lpf0, dlpf = h.dlpf0, dlpfp = dlpf;
        do {
            if (lpf > lpfmax) lpf = lpfmax;
            d2d(m->fp, m->f, N, st);
            d2d(m->dt, m->d, N, st);
            d2d(m->fcur, m->f, N, st);
            dlpfp = dlpf;
            reset_to_converged(m);
            d2d(m->um, m->uc, N, st);
            d2d(m->uc_i, m->uc, N, st);
            d2d(m->vm, m->vc, N, st);
            d2d(m->vc_i, m->vc, N, st);
            d2d(m->am, m->ac, N, st);
            d2d(m->ac_i, m->ac, N, st);
            ++passes;
            itecnt = 0;
            do {
                cb::MsalScalars &s = newmark_iteration(m, p, k, sub_dt, lpf, itecnt, a0, a2, a3, a6, a7);
                if (s.test_err) fail_run(m, CB_ERR_NUMERIC, "zero norm in the convergence test", test_message(s.test_err));
                convchk = s.convchk;
                res_num = s.dots[2];
                res_den = s.dots[6];
                advance_iteration(m);
                itecnt++;
            } while (convchk != 0 && itecnt <= h.itemax);
            if (convchk != 0 && subcnt <= h.submax) {
                if (lpf == lpfmax) {  // main.c:3777-3782
                    ref_message(m, "\n***ERROR*** Maximum allowable load proportionality factor attempted without "
                                   "convergence at current time step\n");
                    break;
                } else if (dlpfp == h.dlpfmin) {  // main.c:3783-3787
                    ref_message(m, "\n***ERROR*** Minimum allowable increment of load proportionality factor "
                                   "reached at current time step\n");
                    break;
                }
                dlpf = dlpfp / 2;
                if (dlpf < h.dlpfmin) dlpf = h.dlpfmin;
                lpf = lpf - dlpfp + dlpf;
                subcnt++;
                solcnt = 0;
            } else if (subcnt > h.submax) {
                ref_message(m, "\n***ERROR*** Maximum allowable number of subdivisions exceeded at current time "
                               "step\n");  // main.c:3802-3805
                break;
            } else {
                solcnt++;
                subcnt = 0;
                if (solcnt >= h.solmin) {
                    dlpf *= 2;
                    solcnt = 0;
                }
                lpf += dlpf;
            }
        } while (lpf <= lpfmax);
        if (convchk != 0) {
            // halve the time increment (main.c:3823-3843)
            ref_message(m, "\nTime increment interval reduced\n");
            ddt = ddt / 2;
            dt_temp = ddt * dt;
            if (tsflag == 0) sub_dt = ddt;
            else if (tsflag == 1) sub_dt = sub_dt - ddt;
        } else {
            // accept (main.c:3845-3917); the newest element state is in ip
            d2d(m->d, m->dt, N, st);
            d2d(m->f, m->fcur, N, st);
            d2d(m->uc, m->uc_i, N, st);
            d2d(m->vc, m->vc_i, N, st);
            d2d(m->ac, m->ac_i, N, st);
            accept_state(m, true);
        }
        if (ddt < 1) {
            if (sub_dt <= 1) {
                sub_dt = sub_dt + ddt;
                tsflag = 1;
            }
            if (sub_dt > 1) {
                ddt = ddt * 2;
                tsflag = 2;
            }
        } else if (ddt == 1) {
            tsflag = 2;
        }
    } while (ddt >= 0.0001 && tsflag != 2);
    if (convchk != 0)
        fail_run(m, CB_ERR_DIVERGED, "minimum time increment interval reached without convergence",
                 "\n***ERROR*** Minimum time increment interval reached without convergence\n");  // main.c:3941
    CB_CUDA(cudaStreamSynchronize(st));
    m->nm_ddt = ddt;
    out->lam = (double)k * dt;
    out->iterations = itecnt;
    out->attempts = passes;
    out->residual = res_den > 0 ? std::sqrt(res_num / res_den) : 0.0;
    out->dk = 0;
    m->itecnt = itecnt;
    m->nm_k = k + 1;
    if (m->nm_k >= h.nsteps) m->nm_phase = 2;
}

// ---- linear Newmark (ANAFLAG 1, ALGFLAG 4): main.c:3143-3302 with the
// effective stiffness of solve.c:139-222 and the time loop of solve.c:246-467
// (SLVFLAG 0, no prescribed motion, no restart) ----

struct LinearCoeffs {
    double a0, a2, a3, a6, a7;
};

LinearCoeffs linear_coeffs(const NewmarkParams &p, double dt)
{
    const double dt_temp = 1 * dt;  // the solve's ddt is 1 (main.c:3268)
    return LinearCoeffs{1 / (p.alpha * std::pow(dt_temp, 2)), 1 / (p.alpha * dt_temp), 1 / (2 * p.alpha) - 1,
                        (dt_temp) * (1 - p.delta), p.delta * (dt_temp)};
}

// The stiffness of the initial state (the element forces are zero, so the
// frame and shell tangents are stiffe alone, as ANAFLAG 1 forms them), kept
// for K u_m; the lumped mass (mass_fr or mass_sh); K_eff = K + a0 (1 - am) /
// (1 - af) M factored once; the motion from the initial conditions.
void linear_begin(cb_model *m)
{
    newmark_begin(m);
    const cb::HostModel &h = m->h;
    const long N = h.neq, F = h.ne_fr;
    cudaStream_t st = m->st;
    const NewmarkParams p = newmark_params(h);
    const LinearCoeffs c = linear_coeffs(p, h.dt);
    assemble_tangent(m, TangentState::converged);
    d2d(m->band64, (const double *)m->bf.band, (size_t)m->bf.ld * m->bf.nblk * m->bf.s, st);
    {
        PhaseTimer t(m, &m->tm.ms_tangent);
        const long E = h.ne_sh, T = h.ne_tr;
        if (E) cb::launch_shell_mass(m->sh, m->x_c, m->sh_dens, m->me, E, st);
        if (F) cb::launch_frame_mass(m->fr, m->x_c, m->fr_lref, m->me + 18 * E + 6 * T, F, st);
        cb::launch_gather_f64(m->fmap_ptr, m->fmap_src, m->me, m->sm, N, st);
        cb::launch_nm_keff<double>((double *)m->bf.band, m->bf.ld, m->sm, c.a0 * (1 - p.alpham), 1 - p.alphaf, N,
                                   st);
        m->tm.launches += 3;
    }
    factor(m);
    h2d(m->um, h.um0.data(), N, st);
    h2d(m->vm, h.vm0.data(), N, st);
    h2d(m->am, h.am0.data(), N, st);
    (void)pull_scalars(m);  // a timed-out factorisation barrier is reported here
}

// time step k: K_eff uc = p_k [+ af/(1-af) p_(k-1)] + M_eff [- af/(1-af) K u_m],
// then the kinematics
void linear_step(cb_model *m, cb_step *out)
{
    const cb::HostModel &h = m->h;
    const long N = h.neq;
    cudaStream_t st = m->st;
    out->done = 0;
    if (m->nm_k >= h.nsteps) {
        ref_success(m, "\nSolution successful!!\n");  // main.c:3300-3302
        out->done = 1;
        out->lam = (double)(h.nsteps - 1) * h.dt;
        out->iterations = 0;
        out->attempts = 0;
        out->residual = 0;
        out->dk = 0;
        return;
    }
    const long k = m->nm_k;
    const NewmarkParams p = newmark_params(h);
    const LinearCoeffs c = linear_coeffs(p, h.dt);
    const double *pin_k = m->pin + (size_t)k * N;
    const double *pin_km1 = k > 0 ? m->pin + (size_t)(k - 1) * N : pin_k;
    {
        PhaseTimer t(m, &m->tm.ms_vector);
        const double *nku = nullptr;
        if (p.alphaf != 0) {
            // -K u_m from the kept stiffness (the band product r = b - K x with b = 0)
            CB_CUDA(cudaMemsetAsync(m->ref_x, 0, N * sizeof(double), st));
            cb::band_residual64(m->band64, m->bf.ld, m->bf.bw, N, m->ref_x, m->um, m->ref_r, m->ref_w, st);
            nku = m->ref_r;
            m->tm.launches += 2;
        }
        cb::launch_lin_reff(k == 0, p.alpham, p.alphaf, c.a0, c.a2, c.a3, pin_km1, pin_k, m->sm, m->um, m->vm, m->am,
                            nku, m->r, N, st);
        m->tm.launches += 1;
    }
    solve(m, m->r, m->uc);
    {
        PhaseTimer t(m, &m->tm.ms_vector);
        cb::launch_lin_update(m->uc, m->um, m->vm, m->am, m->vc, m->ac, m->d, c.a0, c.a2, c.a3, c.a6, c.a7, N, st);
        m->tm.launches += 1;
    }
    (void)pull_scalars(m);  // one synchronisation; a timed-out solve barrier is reported
    out->lam = (double)k * h.dt;
    out->iterations = 0;
    out->attempts = 1;
    out->residual = 0;
    out->dk = 0;
    m->itecnt = 0;
    m->nm_k = k + 1;
    if (m->nm_k >= h.nsteps) m->nm_phase = 2;
}

}  // namespace

extern "C" {

int cb_newmark_begin(cb_model *m)
{
    if (!m || !m->st) return CB_ERR_ARG;
    if (m->h.alg != 5 && m->h.alg != 4) {
        m->err = "cb_newmark_begin needs an ALGFLAG 5 (nonlinear Newmark) or ALGFLAG 4 (linear Newmark) model";
        return CB_ERR_STATE;
    }
    return guarded(m, [&] {
        if (m->h.alg == 4) linear_begin(m);
        else newmark_begin(m);
    });
}

int cb_newmark_step(cb_model *m, cb_step *out)
{
    if (!m || !out) return CB_ERR_ARG;
    if (m->nm_phase == 0) {
        m->err = "cb_newmark_begin has not completed";
        return CB_ERR_STATE;
    }
    return guarded(m, [&] {
        if (m->h.alg == 4) linear_step(m, out);
        else newmark_step(m, out);
    });
}

int cb_set_krylov_tolerance(cb_model *m, double rtol)
{
    if (!m || !(rtol > 0) || !(rtol < 1)) return CB_ERR_ARG;
    if (!m->ks) {
        m->err = "the handle does not use the FGMRES solver";
        return CB_ERR_STATE;
    }
    m->ks->rtol = rtol;
    return CB_OK;
}

int cb_get_krylov_stats(const cb_model *m, cb_krylov_stats *s)
{
    if (!m || !s) return CB_ERR_ARG;
    std::memset(s, 0, sizeof *s);
    if (!m->ks) return CB_OK;
    const cb::KrylovSolver &ks = *m->ks;
    s->solves = ks.solves;
    s->iterations = ks.iterations_total;
    s->unconverged = ks.unconverged;
    s->last_iterations = ks.last_iters;
    s->last_residual = ks.last_resid;
    s->learned_solves = m->learned_solves;
    s->fallbacks = m->fallbacks;
    s->train_steps = cb::mpnn_adam_steps(m->mp);
    s->train_loss = cb::mpnn_last_loss(m->mp);
    s->inner_iterations = ks.inner_iterations;
    return CB_OK;
}

int cb_set_learning(cb_model *m, int train_steps, int adam_per_solve, double lr, double stall_factor)
{
    if (!m || adam_per_solve < 0 || !(lr > 0) || !(stall_factor > 0)) return CB_ERR_ARG;
    if (!m->mp) {
        m->err = "the handle has no learned preconditioner";
        return CB_ERR_STATE;
    }
    m->learn_steps = train_steps;
    m->learn_adam = adam_per_solve;
    m->learn_stall = stall_factor;
    cb::mpnn_set_lr(m->mp, lr);
    return CB_OK;
}

long cb_mpnn_param_count(void) { return cb::mpnn_param_count(); }

int cb_mpnn_set_params(cb_model *m, const float *theta)
{
    if (!m || !theta) return CB_ERR_ARG;
    if (!m->mp) {
        m->err = "the handle has no learned preconditioner";
        return CB_ERR_STATE;
    }
    return guarded(m, [&] {
        cb::mpnn_set_params(m->mp, theta, m->st);
        CB_CUDA(cudaStreamSynchronize(m->st));
    });
}

int cb_mpnn_get_params(const cb_model *m, float *theta, float *grad)
{
    if (!m) return CB_ERR_ARG;
    cb_model *mm = const_cast<cb_model *>(m);
    if (!m->mp) {
        mm->err = "the handle has no learned preconditioner";
        return CB_ERR_STATE;
    }
    return guarded(mm, [&] { cb::mpnn_get_params(m->mp, theta, grad, m->st); });
}

int cb_mpnn_eval(cb_model *m, const double *r, const double *p, const double *t, int train, double *z,
                 double *loss)
{
    if (!m || !r || !p) return CB_ERR_ARG;
    if (!m->mp) {
        m->err = "the handle has no learned preconditioner";
        return CB_ERR_STATE;
    }
    return guarded(m, [&] {
        const long N = m->h.neq;
        cudaStream_t st = m->st;
        double *rd = m->r, *pd = m->ddr, *td = m->ddq, *zd = m->dt;
        h2d(rd, r, N, st);
        h2d(pd, p, N, st);
        if (t) h2d(td, t, N, st);
        const double L = cb::mpnn_eval(*m->mp, *m->ks, rd, pd, t ? td : nullptr, zd, train != 0, st);
        if (z) d2h(z, zd, N, st);
        CB_CUDA(cudaStreamSynchronize(st));
        if (loss) *loss = L;
    });
}

int cb_newmark_state(const cb_model *m, double *u, double *v, double *a)
{
    if (!m || (m->h.alg != 5 && m->h.alg != 4)) return CB_ERR_ARG;
    cb_model *mm = const_cast<cb_model *>(m);
    return guarded(mm, [&] {
        const long N = m->h.neq;
        if (u) d2h(u, m->uc, N, m->st);
        if (v) d2h(v, m->vc, N, m->st);
        if (a) d2h(a, m->ac, N, m->st);
        CB_CUDA(cudaStreamSynchronize(m->st));
    });
}

int cb_eval_frame_forces(cb_model *m, const double *x_temp, const double *dd, const double *c_ip,
                         const double *ef_ip, const double *len_ip, const double *lref, double *c_i,
                         double *len_i, double *ef_i, double *f)
{
    if (!m || !x_temp || !dd || !c_ip || !ef_ip || !len_ip || !lref || !f) return CB_ERR_ARG;
    const long F = m->h.ne_fr, N = m->h.neq;
    if (F == 0 || m->h.ne_tr || m->h.ne_sh) {
        m->err = "cb_eval_frame_forces needs a frame-only model";
        return CB_ERR_UNSUPPORTED;
    }
    return guarded(m, [&] {
        cudaStream_t st = m->st;
        cb::DevFrame &fr = m->fr;
        h2d(m->x_t, x_temp, m->h.nj * 3, st);
        h2d(m->dd, dd, N, st);
        std::vector<double> cs = to_soa(c_ip, F, 9), es = to_soa(ef_ip, F, 14);
        h2d(fr.c_ip, cs.data(), cs.size(), st);
        h2d(fr.ef_ip, es.data(), es.size(), st);
        h2d(fr.len_ip, len_ip, F, st);
        h2d(m->fr_lref, lref, F, st);
        internal_force(m, m->dd, m->fcur);
        d2h(f, m->fcur, N, st);
        std::vector<double> c(9 * F), e(14 * F), L(F);
        d2h(c.data(), fr.c_i, 9 * F, st);
        d2h(e.data(), fr.ef_i, 14 * F, st);
        d2h(L.data(), fr.len_i, F, st);
        CB_CUDA(cudaStreamSynchronize(st));
        if (c_i) from_soa(c, F, 9, c_i);
        if (ef_i) from_soa(e, F, 14, ef_i);
        if (len_i) std::memcpy(len_i, L.data(), sizeof(double) * F);
    });
}

int cb_eval_frame_tangent(cb_model *m, const double *c, const double *ef, const double *len, const double *lref,
                          long *maxa, double *ss)
{
    if (!m || !c || !ef || !len || !lref || !ss) return CB_ERR_ARG;
    if (!m->bf.band) {
        m->err = "this entry point works on the band LDL^T; the handle uses the FGMRES solver";
        return CB_ERR_UNSUPPORTED;
    }
    const long F = m->h.ne_fr, N = m->h.neq;
    if (F == 0 || m->h.ne_tr || m->h.ne_sh) {
        m->err = "cb_eval_frame_tangent needs a frame-only model";
        return CB_ERR_UNSUPPORTED;
    }
    return guarded(m, [&] {
        cudaStream_t st = m->st;
        cb::DevFrame &fr = m->fr;
        std::vector<double> cs = to_soa(c, F, 9), es = to_soa(ef, F, 14);
        h2d(fr.c_c, cs.data(), cs.size(), st);
        h2d(fr.ef_c, es.data(), es.size(), st);
        h2d(fr.len_c, len, F, st);
        h2d(m->fr_lref, lref, F, st);
        assemble_tangent(m, TangentState::converged);
        cb::BandFactor &bf = m->bf;
        const long npad = bf.nblk * bf.s;
        std::vector<double> band((size_t)bf.ld * npad);
        if (bf.fp32) {
            std::vector<float> bfl((size_t)bf.ld * npad);
            d2h(bfl.data(), (const float *)bf.band, bfl.size(), st);
            CB_CUDA(cudaStreamSynchronize(st));
            for (size_t i = 0; i < bfl.size(); ++i) band[i] = bfl[i];
        } else {
            d2h(band.data(), (const double *)bf.band, band.size(), st);
            CB_CUDA(cudaStreamSynchronize(st));
        }
        if (maxa) std::memcpy(maxa, m->h.maxa.data(), sizeof(long) * (N + 1));
        for (long j = 1; j <= N; ++j) {
            long hgt = m->h.maxa[j] - m->h.maxa[j - 1] - 1;
            for (long off = 0; off <= hgt; ++off) {
                long i = j - off;
                ss[m->h.maxa[j - 1] - 1 + off] = band[(size_t)(i - 1) * bf.ld + off];
            }
        }
    });
}

int cb_eval_frame_mass(cb_model *m, const double *x, double *sm, double *len)
{
    if (!m || !x || !sm) return CB_ERR_ARG;
    const long F = m->h.ne_fr, N = m->h.neq;
    if (F == 0 || m->h.ne_tr || m->h.ne_sh) {
        m->err = "cb_eval_frame_mass needs a frame-only model";
        return CB_ERR_UNSUPPORTED;
    }
    return guarded(m, [&] {
        cudaStream_t st = m->st;
        h2d(m->x_t, x, m->h.nj * 3, st);
        double *me = m->fe;  // frame-only: the contribution buffer holds 14 F entries
        cb::launch_frame_mass(m->fr, m->x_t, m->fr_lref, me, F, st);
        cb::launch_gather_f64(m->fmap_ptr, m->fmap_src, me, m->r, N, st);
        d2h(sm, m->r, N, st);
        if (len) d2h(len, m->fr_lref, F, st);
        CB_CUDA(cudaStreamSynchronize(st));
    });
}

}  // extern "C"
