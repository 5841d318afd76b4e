// Resident model setup, the driver steps shared with the Newmark driver, the
// GPU-resident modified spherical arc-length driver and the C ABI.
//
// The host keeps the scalar control flow of main.c:2158-3141 (step-size
// control, subdivision counters, acceptance); every vector and element
// operation runs on the GPU, and the host reads one small scalar block back
// per Newton iteration.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cubens_gb300.h"
#include "internal.hpp"
#include "model.hpp"

using cb::HostModel;

namespace drv {

void upload_model(cb_model *m)
{
    HostModel &h = m->h;
    cudaStream_t st = m->st;
    auto h2d = [m](auto *dst, const auto *src, size_t n, cudaStream_t s) {
        m->h2d_bytes += n * sizeof(*src);
        ::h2d(dst, src, n, s);
    };
    const long NJ = h.nj, N = h.neq, E = h.ne_sh, T = h.ne_tr, F = h.ne_fr;
    m->x0 = m->alloc<double>(NJ * 3);
    m->x_c = m->alloc<double>(NJ * 3);
    m->x_t = m->alloc<double>(NJ * 3);
    h2d(m->x0, h.x0.data(), NJ * 3, st);
    d2d(m->x_c, m->x0, NJ * 3, st);
    std::vector<int> eqx(N, -1);
    for (long i = 0; i < NJ; ++i)
        for (int j = 0; j < 3; ++j)
            if (h.jcode[i * 7 + j]) eqx[h.jcode[i * 7 + j] - 1] = (int)(i * 3 + j);
    m->eq_x = m->alloc<int>(N);
    h2d(m->eq_x, eqx.data(), N, st);
    for (double **v : {&m->q, &m->d, &m->dp, &m->dpp, &m->ddq, &m->ddr, &m->dd, &m->dt, &m->r, &m->f,
                       &m->zero, &m->ssd_o, &m->fcur, &m->fprev})
        *v = m->alloc<double>(N);
    h2d(m->q, h.q.data(), N, st);
    // shells
    if (E > 0) {
        cb::DevShell &s = m->sh;
        s.conn = m->alloc<int>(3 * E);
        s.eq = m->alloc<int>(18 * E);
        s.prop = m->alloc<double>(3 * E);
        s.xl = m->alloc<double>(3 * E);
        s.kem = m->alloc<double>(36 * E);
        s.keb = m->alloc<double>(81 * E);
        s.c_c = m->alloc<double>(9 * E);
        s.c_ip = m->alloc<double>(9 * E);
        s.c_i = m->alloc<double>(9 * E);
        s.a_c = m->alloc<double>(E);
        s.a_i = m->alloc<double>(E);
        s.ef_c = m->alloc<double>(18 * E);
        s.ef_ip = m->alloc<double>(18 * E);
        s.ef_i = m->alloc<double>(18 * E);
        std::vector<int> conn(3 * E), eq(18 * E);
        std::vector<double> prop(3 * E);
        for (long e = 0; e < E; ++e) {
            for (int a = 0; a < 3; ++a) {
                int n = h.sh_conn[e * 3 + a];
                conn[a * E + e] = n;
                for (int dof = 0; dof < 6; ++dof) eq[(a * 6 + dof) * E + e] = (int)h.jcode[n * 7 + dof] - 1;
            }
            prop[e] = h.sh_e[e];
            prop[E + e] = h.sh_nu[e];
            prop[2 * E + e] = h.sh_t[e];
        }
        h2d(s.conn, conn.data(), conn.size(), st);
        h2d(s.eq, eq.data(), eq.size(), st);
        h2d(s.prop, prop.data(), prop.size(), st);
        cb::launch_shell_setup(s, m->x0, E, st);
        CB_CUDA(cudaGetLastError());
    }
    if (T > 0) {
        cb::DevTruss &t = m->tr;
        t.conn = m->alloc<int>(2 * T);
        t.eq = m->alloc<int>(6 * T);
        t.ea = m->alloc<double>(T);
        t.len0 = m->alloc<double>(T);
        t.len_c = m->alloc<double>(T);
        t.len_i = m->alloc<double>(T);
        t.dir_c = m->alloc<double>(3 * T);
        t.dir_i = m->alloc<double>(3 * T);
        t.n_c = m->alloc<double>(T);
        t.n_i = m->alloc<double>(T);
        std::vector<int> conn(2 * T), eq(6 * T);
        std::vector<double> ea(T), len0(T), dir0(3 * T);
        for (long e = 0; e < T; ++e) {
            int na = h.tr_conn[e * 2], nb = h.tr_conn[e * 2 + 1];
            conn[e] = na;
            conn[T + e] = nb;
            for (int a = 0; a < 2; ++a)
                for (int dof = 0; dof < 3; ++dof)
                    eq[(a * 3 + dof) * T + e] = (int)h.jcode[h.tr_conn[e * 2 + a] * 7 + dof] - 1;
            double el[3];
            for (int k = 0; k < 3; ++k) el[k] = h.x0[nb * 3 + k] - h.x0[na * 3 + k];
            double L = std::sqrt(el[0] * el[0] + el[1] * el[1] + el[2] * el[2]);
            len0[e] = L;
            for (int k = 0; k < 3; ++k) dir0[k * T + e] = el[k] / L;
            ea[e] = h.tr_e[e] * h.tr_a[e];
        }
        h2d(t.conn, conn.data(), conn.size(), st);
        h2d(t.eq, eq.data(), eq.size(), st);
        h2d(t.ea, ea.data(), T, st);
        h2d(t.len0, len0.data(), T, st);
        d2d(t.len_c, t.len0, T, st);
        h2d(t.dir_c, dir0.data(), 3 * T, st);
    }
    if (F > 0) {
        cb::DevFrame &fr = m->fr;
        fr.conn = m->alloc<int>(2 * F);
        fr.eq = m->alloc<int>(14 * F);
        fr.prop = m->alloc<double>(8 * F);
        fr.aux = m->alloc<double>(3 * F);
        fr.len0 = m->alloc<double>(F);
        for (double **v : {&fr.c_c, &fr.c_ip, &fr.c_i}) *v = m->alloc<double>(9 * F);
        for (double **v : {&fr.ef_c, &fr.ef_ip, &fr.ef_i}) *v = m->alloc<double>(14 * F);
        for (double **v : {&fr.len_c, &fr.len_ip, &fr.len_i}) *v = m->alloc<double>(F);
        m->fr_lref = m->alloc<double>(F);
        std::vector<int> conn(2 * F), eq(14 * F);
        std::vector<double> prop(8 * F), aux(3 * F);
        for (long e = 0; e < F; ++e) {
            conn[e] = h.fr_conn[e * 2];
            conn[F + e] = h.fr_conn[e * 2 + 1];
            for (int k = 0; k < 14; ++k) eq[k * F + e] = (int)h.fr_mc[e * 14 + k] - 1;
            for (int k = 0; k < 8; ++k) prop[k * F + e] = h.fr_prop[e * 8 + k];
            for (int k = 0; k < 3; ++k) aux[k * F + e] = h.fr_aux[e * 3 + k];
        }
        h2d(fr.conn, conn.data(), conn.size(), st);
        h2d(fr.eq, eq.data(), eq.size(), st);
        h2d(fr.prop, prop.data(), prop.size(), st);
        h2d(fr.aux, aux.data(), aux.size(), st);
        // initial triads and lengths (prop_fr, frame.c:130-160)
        cb::launch_frame_geometry(fr, m->x0, fr.c_c, fr.len0, F, st);
        CB_CUDA(cudaGetLastError());
        d2d(fr.len_c, fr.len0, F, st);
        d2d(m->fr_lref, fr.len0, F, st);
    }
    if (h.alg >= 4) {
        for (double **v : {&m->uc, &m->vc, &m->ac, &m->uc_i, &m->vc_i, &m->ac_i, &m->um, &m->vm, &m->am, &m->sm,
                           &m->qtot, &m->dyn, &m->fp})
            *v = m->alloc<double>(N);
        m->me = m->alloc<double>(18 * E + 6 * T + 14 * F);  // element masses in the force buffer's layout
        if (E) {
            m->sh_dens = m->alloc<double>(E);
            h2d(m->sh_dens, h.echo.sh_dens.data(), E, st);
        }
        m->pin = m->alloc<double>(h.pin.size());
        h2d(m->pin, h.pin.data(), h.pin.size(), st);
    }
    m->fe = m->alloc<double>(18 * E + 6 * T + 14 * F);
    // gather maps
    cb::GatherMap fm, tm;
    cb::build_force_map(h, fm);
    m->fmap_ptr = m->alloc<int>(fm.ptr.size());
    m->fmap_src = m->alloc<int>(fm.src.size());
    h2d(m->fmap_ptr, fm.ptr.data(), fm.ptr.size(), st);
    h2d(m->fmap_src, fm.src.data(), fm.src.size(), st);
    const bool fp32 = m->opt.precision == CB_MIXED;
    const bool dwp = m->opt.precision == CB_FP32X2;
    if (m->opt.solver == CB_SOLVER_FGMRES) {
        // FP64 matrix and Krylov vectors; mixed precision stores the
        // preconditioner in FP32
        m->ks = new cb::KrylovSolver();
        cb::krylov_alloc(*m->ks, h, m->opt.krylov_restart, m->opt.krylov_maxit, fp32, st);
        m->bytes += m->ks->bytes;
        if (m->opt.precond == CB_PRECOND_LEARNED) {
            m->mp = cb::mpnn_create(h, 20240611u, 32, st);
            m->ks->mpnn = m->mp;
            m->bytes += cb::mpnn_bytes(m->mp);
        }
        m->kel = m->alloc<double>(171 * E + 21 * T + 105 * F);
        if (h.alg == 3) m->bpiv = m->alloc<double>(N);
        m->sc = m->alloc<cb::MsalScalars>(1);
        m->partial = m->alloc<double>(16 * cb::kRedBlocks);
        CB_CUDA(cudaMallocHost(&m->sc_h, sizeof(cb::MsalScalars)));
        std::memset(m->sc_h, 0, sizeof(cb::MsalScalars));
        CB_CUDA(cudaMallocHost(&m->hs, sizeof(cb_host_stage)));
        std::memset(m->hs, 0, sizeof(cb_host_stage));
        CB_CUDA(cudaStreamSynchronize(st));
        return;
    }
    // Newmark and full Newton-Raphson refactor every iteration and solve once
    // per factorisation: direct substitution, no solve blocks
    if (dwp)
        cb::band_alloc_dw(m->bf, N, h.bw, m->opt.factor_kernel == 1);
    else
        cb::band_alloc(m->bf, N, h.bw, fp32, h.alg >= 4 || h.alg == 1 || m->opt.band_solve == 1,
                       m->opt.factor_kernel == 1);
    m->bytes += m->bf.bytes;
    cb::build_tangent_map(h, m->bf.ld, tm);
    m->tmap_n = (long)tm.dst.size();
    m->tmap_ptr = m->alloc<int>(tm.ptr.size());
    m->tmap_src = m->alloc<int>(tm.src.size());
    m->tmap_dst = m->alloc<int64_t>(tm.dst.size());
    h2d(m->tmap_ptr, tm.ptr.data(), tm.ptr.size(), st);
    h2d(m->tmap_src, tm.src.data(), tm.src.size(), st);
    h2d(m->tmap_dst, tm.dst.data(), tm.dst.size(), st);
    if (fp32) m->kel = m->alloc<float>(171 * E + 21 * T + 105 * F);
    else m->kel = m->alloc<double>(171 * E + 21 * T + 105 * F);
    if (fp32 && h.alg == 5) {
        m->band64 = m->alloc<double>((size_t)m->bf.ld * m->bf.nblk * m->bf.s);
        m->kel64 = m->alloc<double>(105 * F);
        for (double **v : {&m->ref_r, &m->ref_x, &m->ref_w}) *v = m->alloc<double>(N);
    }
    if (h.alg == 4) {
        // linear Newmark: the stiffness kept beside the factored K_eff (K u_m
        // of the effective load), and work vectors of the band product
        m->band64 = m->alloc<double>((size_t)m->bf.ld * m->bf.nblk * m->bf.s);
        for (double **v : {&m->ref_r, &m->ref_x, &m->ref_w}) *v = m->alloc<double>(N);
    }
    m->sc = m->alloc<cb::MsalScalars>(1);
    m->partial = m->alloc<double>(16 * cb::kRedBlocks);
    CB_CUDA(cudaMallocHost(&m->sc_h, sizeof(cb::MsalScalars)));
    std::memset(m->sc_h, 0, sizeof(cb::MsalScalars));
    CB_CUDA(cudaMallocHost(&m->hs, sizeof(cb_host_stage)));
    std::memset(m->hs, 0, sizeof(cb_host_stage));
    CB_CUDA(cudaStreamSynchronize(st));
}

// ---- state transitions of main.c ----

// i, ip <- converged (main.c:2582-2623, 2667-2707)
void reset_to_converged(cb_model *m)
{
    const long NJ = m->h.nj, E = m->h.ne_sh, T = m->h.ne_tr;
    cudaStream_t st = m->st;
    d2d(m->x_t, m->x_c, NJ * 3, st);
    if (E) {
        d2d(m->sh.c_i, m->sh.c_c, 9 * E, st);
        d2d(m->sh.c_ip, m->sh.c_c, 9 * E, st);
        d2d(m->sh.a_i, m->sh.a_c, E, st);
        d2d(m->sh.ef_i, m->sh.ef_c, 18 * E, st);
        d2d(m->sh.ef_ip, m->sh.ef_c, 18 * E, st);
    }
    if (T) {
        d2d(m->tr.len_i, m->tr.len_c, T, st);
        d2d(m->tr.dir_i, m->tr.dir_c, 3 * T, st);
        d2d(m->tr.n_i, m->tr.n_c, T, st);
    }
    const long F = m->h.ne_fr;
    if (F) {
        cb::DevFrame &fr = m->fr;
        d2d(fr.c_i, fr.c_c, 9 * F, st);
        d2d(fr.c_ip, fr.c_c, 9 * F, st);
        d2d(fr.ef_i, fr.ef_c, 14 * F, st);
        d2d(fr.ef_ip, fr.ef_c, 14 * F, st);
        d2d(fr.len_i, fr.len_c, F, st);
        d2d(fr.len_ip, fr.len_c, F, st);
    }
}

// ip <- i after an iteration (main.c:2399-2428, 3712-3740)
void advance_iteration(cb_model *m)
{
    std::swap(m->sh.c_ip, m->sh.c_i);
    std::swap(m->sh.ef_ip, m->sh.ef_i);
    std::swap(m->fr.c_ip, m->fr.c_i);
    std::swap(m->fr.ef_ip, m->fr.ef_i);
    std::swap(m->fr.len_ip, m->fr.len_i);
}

// converged <- i on acceptance (main.c:3060-3105); ip is left as it is.
// latest_in_ip: the caller already advanced (ip <- i by pointer swap), so the
// newest triads and element forces are in the ip buffers.
void accept_state(cb_model *m, bool latest_in_ip)
{
    const long NJ = m->h.nj, E = m->h.ne_sh, T = m->h.ne_tr;
    cudaStream_t st = m->st;
    d2d(m->x_c, m->x_t, NJ * 3, st);
    if (E) {
        d2d(m->sh.c_c, latest_in_ip ? m->sh.c_ip : m->sh.c_i, 9 * E, st);
        d2d(m->sh.a_c, m->sh.a_i, E, st);
        d2d(m->sh.ef_c, latest_in_ip ? m->sh.ef_ip : m->sh.ef_i, 18 * E, st);
    }
    if (T) {
        d2d(m->tr.len_c, m->tr.len_i, T, st);
        d2d(m->tr.dir_c, m->tr.dir_i, 3 * T, st);
        d2d(m->tr.n_c, m->tr.n_i, T, st);
    }
    const long F = m->h.ne_fr;
    if (F) {
        cb::DevFrame &fr = m->fr;
        d2d(fr.c_c, latest_in_ip ? fr.c_ip : fr.c_i, 9 * F, st);
        d2d(fr.ef_c, latest_in_ip ? fr.ef_ip : fr.ef_i, 14 * F, st);
        d2d(fr.len_c, latest_in_ip ? fr.len_ip : fr.len_i, F, st);
    }
}

// updatc geometry + forces_tr + forces_fr + forces_sh + deterministic
// assembly into fout
void internal_force(cb_model *m, const double *dd_vec, double *fout)
{
    PhaseTimer t(m, &m->tm.ms_force);
    const long E = m->h.ne_sh, T = m->h.ne_tr, F = m->h.ne_fr;
    if (T) cb::launch_truss_forces(m->tr, m->x_t, m->fe + 18 * E, T, m->st);
    if (F) cb::launch_frame_forces(m->fr, m->x_t, dd_vec, m->fr_lref, m->fe + 18 * E + 6 * T, F, m->st);
    if (E) cb::launch_shell_forces(m->sh, m->x_t, dd_vec, m->fe, E, m->st);
    cb::launch_gather_f64(m->fmap_ptr, m->fmap_src, m->fe, fout, m->h.neq, m->st);
    m->tm.launches += (T ? 1 : 0) + (F ? 1 : 0) + (E ? 1 : 0) + 1;
    m->tm.force_evals++;
}

template <typename K>
void assemble_tangent_t(cb_model *m, TangentState which)
{
    const long E = m->h.ne_sh, T = m->h.ne_tr, F = m->h.ne_fr;
    cb::BandFactor &bf = m->bf;
    K *k = (K *)m->kel;
    if (which == TangentState::converged) {
        if (E) cb::launch_shell_tangent<K>(m->sh, m->x_c, k, E, m->st);
        if (T) cb::launch_truss_tangent<K>(m->tr, k + 171 * E, T, m->st);
    } else {
        // the latest iteration's state (stiff_sh with x_temp, c_ip, deffarea_ip;
        // stiff_tr with defllen_ip, c_ip, ef_ip: main.c:1897-1919)
        if (E) {
            cb::DevShell s = m->sh;
            s.c_c = m->sh.c_ip;
            s.a_c = m->sh.a_i;
            cb::launch_shell_tangent<K>(s, m->x_t, k, E, m->st);
        }
        if (T) {
            cb::DevTruss t = m->tr;
            t.len_c = m->tr.len_i;
            t.dir_c = m->tr.dir_i;
            t.n_c = m->tr.n_i;
            cb::launch_truss_tangent<K>(t, k + 171 * E, T, m->st);
        }
    }
    if (F) {
        const cb::DevFrame &fr = m->fr;
        const bool conv = which == TangentState::converged;
        cb::launch_frame_tangent<K>(fr, conv ? fr.c_c : fr.c_ip, conv ? fr.ef_c : fr.ef_ip,
                                    conv ? fr.len_c : fr.len_ip, m->fr_lref, k + 171 * E + 21 * T, F, m->st);
    }
    m->tm.launches += 1 + (E ? 1 : 0) + (T ? 1 : 0) + (F ? 1 : 0);
    if (m->ks) {
        // arc-length with FGMRES: the CSR gather, the nodal block-Jacobi
        // inverses and the nodal blocks' pivots (psi's substitute for ssd)
        cb::krylov_assemble(*m->ks, (const double *)k, m->st);
        cb::krylov_setup_block_jacobi(*m->ks, m->st);
        cb::krylov_block_pivots(*m->ks, m->bpiv, m->st);
        m->tm.launches += 2;
        return;
    }
    if (bf.dw) cb::band_dw_gather(m->tmap_ptr, m->tmap_src, m->tmap_dst, (const double *)k, bf, m->tmap_n, m->st);
    else cb::launch_gather_band<K>(m->tmap_ptr, m->tmap_src, m->tmap_dst, k, (K *)bf.band, m->tmap_n, m->st);
}

// tangent into the band (stiff_tr + stiff_fr + stiff_sh)
void assemble_tangent(cb_model *m, TangentState which)
{
    PhaseTimer t(m, &m->tm.ms_tangent);
    if (m->ks) {
        assemble_tangent_t<double>(m, which);
        return;
    }
    cb::BandFactor &bf = m->bf;
    const size_t es = bf.fp32 ? 4 : 8;
    CB_CUDA(cudaMemsetAsync(bf.band, 0, es * (size_t)bf.ld * bf.nblk * bf.s, m->st));
    if (bf.fp32) assemble_tangent_t<float>(m, which);
    else assemble_tangent_t<double>(m, which);
}

void factor(cb_model *m)
{
    if (m->ks) return;  // FGMRES: the block-Jacobi inverses were formed with the tangent
    PhaseTimer t(m, &m->tm.ms_factor);
    cb::band_factor(m->bf, m->st, m->opt.use_graphs != 0, &m->tm.launches);
    m->tm.factorizations++;
}

void solve(cb_model *m, const double *rhs, double *x)
{
    if (m->ks) {
        // arc-length with FGMRES: the first increments train a learned
        // preconditioner (when the handle has one), later ones use it
        const long train = m->learn_steps >= 0 ? m->learn_steps : 5;
        krylov_solve_learned(m, rhs, x, m->msal_incs < train);
        return;
    }
    PhaseTimer t(m, &m->tm.ms_solve);
    cb::band_solve(m->bf, rhs, x, m->st, m->opt.use_graphs != 0, &m->tm.launches);
    m->tm.solves++;
}

// Read the scalar block back (one synchronisation point).
cb::MsalScalars &pull_scalars(cb_model *m)
{
    d2h(m->sc_h, m->sc, 1, m->st);
    cb::GridBarrier *bar = m->hs->bar;
    bar[0].err = bar[1].err = 0;
    if (m->bf.bar) d2h(&bar[0], m->bf.bar, 1, m->st);
    if (m->bf.fbar) d2h(&bar[1], m->bf.fbar, 1, m->st);
    CB_CUDA(cudaStreamSynchronize(m->st));
    if (bar[0].err) throw cb_status_error(CB_ERR_TIMEOUT, "a grid barrier of the solve timed out");
    if (bar[1].err) throw cb_status_error(CB_ERR_TIMEOUT, "a grid barrier of the factorisation timed out");
    return *m->sc_h;
}

// One line of the convergence history from the test's reductions
// (dots 0, 1, 2, 6: |dd|^2, |d|^2, |lam q - f|^2, |lam q|^2).
void log_iteration(cb_model *m, const cb::MsalScalars &s)
{
    m->iter_log.push_back(s.lam_t);
    m->iter_log.push_back(s.dots[1] > 0 ? std::sqrt(s.dots[0] / s.dots[1]) : 0.0);
    m->iter_log.push_back(s.dots[6] > 0 ? std::sqrt(s.dots[2] / s.dots[6]) : 0.0);
}

double device_dot(cb_model *m, const double *a, const double *b, bool diff)
{
    PhaseTimer t(m, &m->tm.ms_vector);
    cb::launch_dot(a, b, m->partial, m->sc, 15, m->h.neq, m->st, diff);
    m->tm.launches += 2;
    d2h(&m->hs->val[0], &m->sc->dots[15], 1, m->st);
    CB_CUDA(cudaStreamSynchronize(m->st));
    return m->hs->val[0];
}

double device_elem(cb_model *m, const double *v, long i)
{
    double x = 0;
    d2h(&x, v + i, 1, m->st);
    CB_CUDA(cudaStreamSynchronize(m->st));
    return x;
}

}  // namespace drv

namespace {

using namespace drv;

// The pivots psi compares step to step: the band factor's (skyfact's ssd),
// or with FGMRES those of the joints' diagonal blocks.
const double *pivots(cb_model *m) { return m->ks ? m->bpiv : m->bf.ssd; }

// Push the host-side scalars the device kernels read.
void push_scalars(cb_model *m, double lam_t, double a, double intener1)
{
    cb::MsalScalars &s = *m->sc_h;
    s.lam_t = lam_t;
    s.lam_old = lam_t;
    s.a = a;
    s.arc = m->arc;
    s.lamp = m->lpfp;
    s.qq = m->qq;
    s.psi_ge = m->psi >= m->h.psi_thresh;
    s.toldisp = m->h.toldisp;
    s.tolforc = m->h.tolforc;
    s.tolener = m->h.tolener;
    s.intener1 = intener1;
    s.quad_status = 0;
    s.convchk = 1;
    s.test_err = 0;
    h2d(m->sc, m->sc_h, 1, m->st);
}

double true_residual(cb_model *m, double lam, const double *fvec)
{
    // |lam q - f| / |lam q|
    cb::launch_scale(m->q, lam, m->r, m->h.neq, m->st);
    double num = device_dot(m, m->r, fvec, true);
    double den = device_dot(m, m->r, nullptr);
    return den > 0 ? std::sqrt(num / den) : 0.0;
}

int fail(cb_model *m, int code, const std::string &msg)
{
    m->err = msg;
    return code;
}

// ---- the first increment (main.c:2296-2560) ----
void msal_begin(cb_model *m, cb_step *out)
{
    HostModel &h = m->h;
    const long N = h.neq;
    cudaStream_t st = m->st;
    m->iter_log.clear();
    reset_to_converged(m);
    CB_CUDA(cudaMemsetAsync(m->d, 0, N * sizeof(double), st));
    CB_CUDA(cudaMemsetAsync(m->dp, 0, N * sizeof(double), st));
    CB_CUDA(cudaMemsetAsync(m->f, 0, N * sizeof(double), st));
    m->lpfp = 0;
    m->qq = device_dot(m, m->q, nullptr);
    assemble_tangent(m);
    factor(m);
    solve(m, m->q, m->ddq);
    d2d(m->ssd_o, pivots(m), N, st);
    double ddq_k = device_elem(m, m->ddq, h.dkdof);
    double lpf = h.dk / ddq_k;
    // d = dd = lpf ddq; intener1 = dd . (lpf q)
    cb::launch_scale(m->ddq, lpf, m->dd, N, st);
    d2d(m->d, m->dd, N, st);
    double intener1 = lpf * device_dot(m, m->dd, m->q);
    cb::launch_update_coords(m->eq_x, m->dd, m->x_t, N, st);
    internal_force(m, m->dd, m->fcur);
    int itecnt = 1;
    advance_iteration(m);
    int convchk = 1;
    do {
        push_scalars(m, lpf, 0.0, intener1);
        {
            PhaseTimer t(m, &m->tm.ms_vector);
            cb::launch_residual(m->q, m->fcur, m->r, m->sc, N, st);
        }
        solve(m, m->r, m->ddr);
        {
            PhaseTimer t(m, &m->tm.ms_vector);
            cb::launch_first_update(m->ddr, m->ddq, h.dkdof, m->d, m->dd, m->eq_x, m->x_t, m->sc, N, st);
        }
        std::swap(m->fcur, m->fprev);  // fprev = f_ip
        internal_force(m, m->dd, m->fcur);
        {
            PhaseTimer t(m, &m->tm.ms_vector);
            cb::launch_test(m->dd, m->d, m->zero, m->q, m->fcur, m->zero, m->fprev, m->partial, m->sc, N, st);
        }
        m->tm.launches += 4;
        cb::MsalScalars &s = pull_scalars(m);
        if (s.test_err) fail_run(m, CB_ERR_NUMERIC, "zero norm in the convergence test", test_message(s.test_err));
        log_iteration(m, s);
        lpf = s.lam_t;
        convchk = s.convchk;
        itecnt++;
        advance_iteration(m);
    } while (convchk != 0 && itecnt <= h.itemax);
    if (convchk != 0)
        fail_run(m, CB_ERR_DIVERGED, "initially prescribed displacement too large",
                 "\n***ERROR*** Initially presecribed displacement too large\n");  // main.c:2520-2521
    // the first increment advances ip <- i after every iteration, converged or not
    // (main.c:2399-2428 run before the loop condition), so the newest state is in ip
    accept_state(m, true);
    d2d(m->f, m->fcur, N, st);
    m->lpf = lpf;
    out->lam = lpf;
    out->iterations = itecnt;
    out->attempts = 1;
    out->residual = true_residual(m, lpf, m->f);
    out->dk = device_elem(m, m->d, h.dkdof);
    out->done = 0;
    m->dkc = std::fabs(out->dk);
    m->lpfc = std::fabs(lpf);
    d2d(m->dpp, m->dp, N, st);
    d2d(m->dp, m->d, N, st);
    m->lpfpp = m->lpfp;
    m->lpfp = lpf;
    reset_to_converged(m);
    double nd = std::sqrt(device_dot(m, m->dp, nullptr));
    m->dnorm = nd;
    m->dnormallow = h.alpha * nd;
    m->beta = std::sqrt((double)h.iteopt / (double)itecnt) * (m->dnormallow / m->dnorm);
    m->psi = 1;
    cb::launch_psi(pivots(m), m->ssd_o, m->partial, m->sc, 14, N, st);
    d2h(&m->hs->val[0], &m->sc->dots[14], 1, st);
    CB_CUDA(cudaStreamSynchronize(st));
    m->psi = m->hs->val[0];
    m->errchk2 = m->subcnt = m->imagcnt = m->negcnt = 0;
    m->itecnt = itecnt;
    m->phase = 1;
    m->msal_incs = 1;
}

// ---- one arc-length increment (main.c:2647-3134) ----
void msal_step(cb_model *m, cb_step *out)
{
    HostModel &h = m->h;
    const long N = h.neq;
    cudaStream_t st = m->st;
    out->done = 0;
    if (!(m->lpfc <= h.lpfmax && m->dkc <= h.dkimax)) {
        ref_success(m, "\nSolution successful\n");  // main.c:3138-3140
        out->done = 1;
        out->lam = m->lpf;
        out->iterations = 0;
        out->attempts = 0;
        out->residual = 0;
        out->dk = 0;
        return;
    }
    int attempts = 0;
    m->iter_log.clear();
    for (;;) {
        ++attempts;
        d2d(m->dt, m->d, N, st);
        double lam_t = m->lpf;
        if (m->errchk2 == 0) {
            double dot = device_dot(m, m->dp, m->dpp, true);
            m->arc = m->psi >= h.psi_thresh
                         ? m->beta * std::sqrt(dot + (m->lpfp - m->lpfpp) * (m->lpfp - m->lpfpp))
                         : m->beta * std::sqrt(dot);
        } else {
            reset_to_converged(m);
            m->errchk2 = 0;
        }
        assemble_tangent(m);
        factor(m);
        solve(m, m->q, m->ddq);
        int det = 0;
        if (m->ks) {
            // FGMRES gives no pivots: K is taken as indefinite when q . K^-1 q <= 0
            // (the sign of the current stiffness parameter), the predictor
            // direction that skyfact's det gives when one eigenvalue has crossed
            det = device_dot(m, m->q, m->ddq) <= 0.0 ? 1 : 0;
        } else {
            int *flags = m->hs->flags;
            d2h(flags, m->bf.flags, 2, st);
            CB_CUDA(cudaStreamSynchronize(st));
            if (flags[1])
                fail_run(m, CB_ERR_NUMERIC, "singular stiffness matrix (zero pivot)",
                         "\n***ERROR*** Singular stiffness matrix\n");  // solve.c:566
            det = flags[0];
        }
        double a = m->psi >= h.psi_thresh ? m->qq + device_dot(m, m->ddq, nullptr) : device_dot(m, m->ddq, nullptr);
        double dlpf = det == 0 ? m->arc * std::sqrt(1 / a) : -m->arc * std::sqrt(1 / a);
        lam_t += dlpf;
        // predictor (main.c:2772-2782): dd = dlpf ddq; d_temp += dd;
        // intener1 = dd . (dlpf q); x_temp += dd
        cb::launch_scale(m->ddq, dlpf, m->dd, N, st);
        double intener1 = dlpf * device_dot(m, m->dd, m->q);
        cb::launch_axpy(m->dd, 1.0, m->dt, N, st);
        cb::launch_update_coords(m->eq_x, m->dd, m->x_t, N, st);
        m->tm.launches += 3;
        internal_force(m, m->dd, m->fcur);
        advance_iteration(m);
        int itecnt = 1;
        int convchk = 1;
        push_scalars(m, lam_t, a, intener1);
        do {
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::launch_residual(m->q, m->fcur, m->r, m->sc, N, st);
            }
            solve(m, m->r, m->ddr);
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::launch_quad_dots(m->dt, m->dp, m->ddr, m->ddq, m->partial, m->sc, N, st);
                cb::launch_quad(m->partial, m->sc, st);
                cb::launch_quad_update(m->ddr, m->ddq, m->dp, m->dt, m->dd, m->eq_x, m->x_t, m->sc, N, st);
            }
            std::swap(m->fcur, m->fprev);
            internal_force(m, m->dd, m->fcur);
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::launch_test(m->dd, m->dt, m->dp, m->q, m->fcur, m->f, m->fprev, m->partial, m->sc, N, st);
            }
            m->tm.launches += 6;
            cb::MsalScalars &s = pull_scalars(m);
            int status = s.quad_status;
            if (status == 0) {
                if (s.test_err) fail_run(m, CB_ERR_NUMERIC, "zero norm in the convergence test", test_message(s.test_err));
                log_iteration(m, s);
                convchk = s.convchk;
                if (convchk == 0) {
                    m->dnorm = std::sqrt(s.dots[5]);
                    if (m->dnorm > 100 * m->dnormallow) {
                        m->arc /= m->beta;
                        m->beta = m->dnormallow / m->dnorm;
                        m->arc *= m->beta;
                        m->errchk2 = 1;
                    }
                } else {
                    itecnt++;
                    if (itecnt > h.itemax) {
                        m->arc *= 0.5;
                        m->subcnt++;
                        m->errchk2 = 1;
                    }
                    advance_iteration(m);
                }
            } else {
                m->arc *= 0.5;
                if (status == 2) m->imagcnt++;
                else m->negcnt++;
                m->errchk2 = status;
                // the scalar block keeps lam_t; the increment is abandoned
            }
        } while (convchk != 0 && m->errchk2 == 0 && m->subcnt <= h.submax && m->imagcnt <= h.imagmax &&
                 m->negcnt <= h.negmax);
        if (m->subcnt > h.submax || m->imagcnt > h.imagmax || m->negcnt > h.negmax)
            fail_run(m, CB_ERR_DIVERGED, "maximum allowable number of subdivisions exceeded",
                     "\n***ERROR*** Maximum allowable number of subdivisions exceeded\n");  // main.c:3041-3042
        if (m->errchk2 != 0) continue;
        // accept (main.c:3045-3133)
        cb::MsalScalars &s = *m->sc_h;
        m->beta = std::sqrt((double)h.iteopt / (double)itecnt) * (m->dnormallow / m->dnorm);
        d2d(m->dpp, m->dp, N, st);
        d2d(m->dp, m->dt, N, st);
        d2d(m->d, m->dt, N, st);
        d2d(m->f, m->fcur, N, st);
        m->lpfpp = m->lpfp;
        m->lpf = m->lpfp = s.lam_t;
        accept_state(m);
        out->dk = device_elem(m, m->d, h.dkdof);
        m->dkc = std::fabs(out->dk);
        m->lpfc = std::fabs(m->lpf);
        cb::launch_psi(pivots(m), m->ssd_o, m->partial, m->sc, 14, N, st);
        d2h(&m->hs->val[0], &m->sc->dots[14], 1, st);
        CB_CUDA(cudaStreamSynchronize(st));
        m->psi = m->hs->val[0];
        m->subcnt = m->imagcnt = m->negcnt = 0;
        m->itecnt = itecnt;
        out->lam = m->lpf;
        out->iterations = itecnt;
        out->attempts = attempts;
        out->residual = true_residual(m, m->lpf, m->f);
        m->msal_incs++;
        return;
    }
}

}  // namespace

extern "C" {

int cb_default_options(cb_options *opt)
{
    if (!opt) return CB_ERR_ARG;
    std::memset(opt, 0, sizeof *opt);
    opt->precision = CB_FP64;
    opt->device = 0;
    opt->use_graphs = 1;
    return CB_OK;
}

int cb_model_create(const char *model_def, size_t len, const cb_options *opt, cb_model **out)
{
    if (!model_def || !out) return CB_ERR_ARG;
    *out = nullptr;
    cb_model *m = new cb_model();
    if (opt) m->opt = *opt;
    else cb_default_options(&m->opt);
    int status = CB_OK;
    std::string msg = cb::parse_model_def(model_def, len, m->h, status);
    if (status != CB_OK) {
        m->err = msg;
        *out = m;  // the handle carries the message; caller destroys it
        return status;
    }
    if (m->h.neq < 2) {
        m->err = "fewer than two equations";
        *out = m;
        return CB_ERR_UNSUPPORTED;
    }
    if (m->opt.solver != CB_SOLVER_BAND && m->opt.solver != CB_SOLVER_FGMRES) {
        m->err = "unknown solver";
        *out = m;
        return CB_ERR_ARG;
    }
    if (m->h.alg == 4 && (m->opt.solver != CB_SOLVER_BAND || m->opt.precision != CB_FP64)) {
        m->err = "the linear Newmark driver (ALGFLAG 4) factors its effective stiffness once with the FP64 band";
        *out = m;
        return CB_ERR_UNSUPPORTED;
    }
    if (m->opt.solver == CB_SOLVER_FGMRES && m->h.alg != 5 && m->h.alg != 3) {
        m->err = "the FGMRES solver serves the nonlinear Newmark and arc-length drivers; static "
                 "Newton-Raphson keeps the direct solve";
        *out = m;
        return CB_ERR_UNSUPPORTED;
    }
    if (m->opt.precision != CB_FP64 && m->opt.precision != CB_MIXED && m->opt.precision != CB_FP32X2) {
        m->err = "unknown precision";
        *out = m;
        return CB_ERR_ARG;
    }
    if (m->opt.precision == CB_FP32X2 && (m->opt.solver != CB_SOLVER_BAND || m->h.alg == 5)) {
        m->err = "the double-word band factor serves the band solver of arc-length and Newton-Raphson "
                 "models (it has no FGMRES form and no Newmark driver)";
        *out = m;
        return CB_ERR_UNSUPPORTED;
    }
    if (m->opt.precond != CB_PRECOND_BLOCK_JACOBI && m->opt.precond != CB_PRECOND_LEARNED) {
        m->err = "unknown preconditioner";
        *out = m;
        return CB_ERR_ARG;
    }
    int rc = guarded(m, [&] {
        int ndev = 0;
        CB_CUDA(cudaGetDeviceCount(&ndev));
        if (ndev <= 0) throw cb_status_error(CB_ERR_CUDA, "no CUDA device");
        CB_CUDA(cudaSetDevice(m->opt.device));
        CB_CUDA(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
        CB_CUDA(cudaEventCreate(&m->ev[0]));
        CB_CUDA(cudaEventCreate(&m->ev[1]));
        upload_model(m);
    });
    *out = m;
    return rc;
}

int cb_model_destroy(cb_model *m)
{
    if (!m) return CB_ERR_ARG;
    if (m->st) cudaStreamSynchronize(m->st);
    cb_results_close(m);
    cb::band_free(m->bf);
    if (m->ks) {
        cb::krylov_free(*m->ks);
        delete m->ks;
    }
    cb::mpnn_destroy(m->mp);
    for (void *p : m->allocs) cudaFree(p);
    if (m->sc_h) cudaFreeHost(m->sc_h);
    if (m->hs) cudaFreeHost(m->hs);
    for (auto &e : m->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : m->marks)
        if (e) cudaEventDestroy(e);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
    return CB_OK;
}

int cb_model_info(const cb_model *m, cb_info *info)
{
    if (!m || !info) return CB_ERR_ARG;
    info->nj = m->h.nj;
    info->ne_tr = m->h.ne_tr;
    info->ne_fr = m->h.ne_fr;
    info->ne_sh = m->h.ne_sh;
    info->neq = m->h.neq;
    info->lss = m->h.lss;
    info->bandwidth = m->h.bw;
    info->block = m->bf.s;
    info->nblocks = m->bf.nblk;
    info->dkdof = m->h.dkdof;
    info->device_bytes = m->bytes;
    info->h2d_bytes = m->h2d_bytes;
    info->algflag = m->h.alg;
    info->nsteps = m->h.nsteps;
    info->dt = m->h.dt;
    info->solver = m->ks ? CB_SOLVER_FGMRES : CB_SOLVER_BAND;
    info->nnz = m->ks ? m->ks->nnz : 0;
    info->node_blocks = m->ks ? m->ks->nblk : 0;
    info->factor_cluster = m->bf.cluster;
    return CB_OK;
}

const char *cb_last_error(const cb_model *m) { return m ? m->err.c_str() : "null handle"; }

int cb_msal_begin(cb_model *m, cb_step *out)
{
    if (!m || !out || !m->st) return CB_ERR_ARG;
    if (m->h.alg != 3) return fail(m, CB_ERR_STATE, "cb_msal_begin needs an ALGFLAG 3 (MSAL) model");
    return guarded(m, [&] { msal_begin(m, out); });
}

int cb_msal_step(cb_model *m, cb_step *out)
{
    if (!m || !out) return CB_ERR_ARG;
    if (m->phase != 1) return fail(m, CB_ERR_STATE, "cb_msal_begin has not completed");
    return guarded(m, [&] { msal_step(m, out); });
}

int cb_get_displacements(const cb_model *m, double *d, double *lam)
{
    if (!m || !d) return CB_ERR_ARG;
    cb_model *mm = const_cast<cb_model *>(m);
    return guarded(mm, [&] {
        d2h(d, m->d, m->h.neq, m->st);
        CB_CUDA(cudaStreamSynchronize(m->st));
        if (lam) *lam = m->lpf;
    });
}

int cb_get_topology(const cb_model *m, long *jcode, double *q)
{
    if (!m) return CB_ERR_ARG;
    if (jcode) std::memcpy(jcode, m->h.jcode.data(), sizeof(long) * m->h.jcode.size());
    if (q) std::memcpy(q, m->h.q.data(), sizeof(double) * m->h.q.size());
    return CB_OK;
}

int cb_get_timers(const cb_model *m, cb_timers *t)
{
    if (!m || !t) return CB_ERR_ARG;
    *t = m->tm;
    return CB_OK;
}

int cb_reset_timers(cb_model *m)
{
    if (!m) return CB_ERR_ARG;
    m->tm = cb_timers{};
    return CB_OK;
}

int cb_set_timing(cb_model *m, int on)
{
    if (!m) return CB_ERR_ARG;
    m->timing = on != 0;
    return CB_OK;
}

int cb_get_iteration_log(const cb_model *m, double *out, int max_iters, int *n)
{
    if (!m || !n) return CB_ERR_ARG;
    const int k = (int)(m->iter_log.size() / 3);
    *n = k;
    if (out && max_iters > 0)
        std::memcpy(out, m->iter_log.data(), sizeof(double) * 3 * (size_t)std::min(k, max_iters));
    return CB_OK;
}

int cb_set_wait_limit(cb_model *m, long long polls)
{
    if (!m) return CB_ERR_ARG;
    m->bf.max_polls = polls == 0 ? cb::kDefaultWaitPolls : (polls < 0 ? -1 : polls);
    return CB_OK;
}

// Access to a handle's factorisation for solve_noalloc.cu.
cb::BandFactor *cb_internal_factor(cb_model *m, cudaStream_t *st, int *device)
{
    if (!m) return nullptr;
    *st = m->st;
    *device = m->opt.device;
    return &m->bf;
}

void cb_internal_share_gpu(cb_model *m, int shared)
{
    if (m) cb::band_share_gpu(m->bf, shared != 0);
}

void cb_internal_set_error(cb_model *m, const char *msg)
{
    if (m) m->err = msg;
}

int cb_event_mark(cb_model *m, int slot)
{
    if (!m || slot < 0 || slot >= 8) return CB_ERR_ARG;
    return guarded(m, [&] {
        if (!m->marks[slot]) CB_CUDA(cudaEventCreate(&m->marks[slot]));
        CB_CUDA(cudaEventRecord(m->marks[slot], m->st));
    });
}

int cb_event_elapsed(cb_model *m, int a, int b, double *ms)
{
    if (!m || !ms || a < 0 || a >= 8 || b < 0 || b >= 8 || !m->marks[a] || !m->marks[b]) return CB_ERR_ARG;
    return guarded(m, [&] {
        CB_CUDA(cudaEventSynchronize(m->marks[b]));
        float v = 0;
        CB_CUDA(cudaEventElapsedTime(&v, m->marks[a], m->marks[b]));
        *ms = v;
    });
}

int cb_profile_kernel(cb_model *m, int which, int reps, double *ms_per_launch, double *bytes_per_launch,
                      double *flops_per_launch)
{
    if (!m || reps <= 0 || !ms_per_launch) return CB_ERR_ARG;
    const bool band_kernel = which == CB_K_SOLVE || which == CB_K_FACTOR || which == CB_K_BAND_LDLT ||
                             which == CB_K_SOLVE_BLOCKS;
    if ((band_kernel && !m->bf.band) || (which == CB_K_SPMV && !m->ks)) {
        m->err = "the kernel belongs to the other solver";
        return CB_ERR_UNSUPPORTED;
    }
    return guarded(m, [&] {
        cudaStream_t st = m->st;
        const cb::BandFactor &bf = m->bf;
        const double es = bf.fp32 ? 4.0 : 8.0;
        const double s = (double)bf.s, nb = (double)bf.nblk;
        const long E = m->h.ne_sh;
        double bytes = 0, flops = 0;
        auto once = [&] {
            switch (which) {
            case CB_K_SOLVE: cb::band_solve(m->bf, m->q, m->ddr, st, false, nullptr); break;
            case CB_K_SHELL_FORCE: cb::launch_shell_forces(m->sh, m->x_t, m->dd, m->fe, E, st); break;
            case CB_K_FACTOR: cb::band_factor(m->bf, st, m->opt.use_graphs != 0, nullptr); break;
            case CB_K_BAND_LDLT: cb::band_profile_launch(m->bf, 3, st); break;
            case CB_K_SOLVE_BLOCKS: cb::band_profile_launch(m->bf, 4, st); break;
            case CB_K_FRAME_FORCE:
                cb::launch_frame_forces(m->fr, m->x_t, m->dd, m->fr_lref,
                                        m->fe + 18 * E + 6 * m->h.ne_tr, m->h.ne_fr, st);
                break;
            case CB_K_SPMV: cb::krylov_spmv(*m->ks, m->q, m->ddr, st); break;
            default: throw cb_status_error(CB_ERR_ARG, "unknown kernel id");
            }
        };
        const double w = (double)bf.w, n = (double)m->h.neq, b = (double)bf.bw;
        switch (which) {
        case CB_K_SOLVE:  // Linv lower halves twice, Pn and Rn once, vectors
            bytes = es * nb * (s * s + 2 * s * w) + 8.0 * 2 * n + es * 4 * nb * s;
            flops = 2 * nb * (s * s + 2 * s * w);
            break;
        case CB_K_SHELL_FORCE:
            // per element: reads conn 12 B, eq 72, xl 24, c_ip 72, ef_ip 144, ke_m columns 144,
            // ke_b 648, 3 vertex coordinates 72, 18 gathered increments 144; writes c_i 72,
            // area 8, ef_i 144, element force 144 (FP64)
            bytes = (double)E * (12 + 72 + 24 + 72 + 144 + 144 + 648 + 72 + 144 + 72 + 8 + 144 + 144);
            flops = (double)E * 2 * 430;
            break;
        case CB_K_FACTOR:
            flops = 2 * (n * b * b / 2) + nb * 2 * (s * s * s / 6 + s * s * w);
            bytes = es * ((double)bf.ld * nb * s * 2 + nb * s * (s + 2 * w));
            break;
        case CB_K_BAND_LDLT:  // n bw^2 / 2 FMA; the band read and written once from L2/HBM
            flops = n * b * b;
            bytes = es * (double)bf.ld * nb * s * 2;
            break;
        case CB_K_SOLVE_BLOCKS:
            flops = nb * 2 * (s * s * s / 6 + s * s * w);
            bytes = es * nb * s * (2 * s + 2 * w);
            break;
        case CB_K_FRAME_FORCE:  // per member ~500 B read, ~300 B written, ~1.2 kFLOP
            bytes = (double)m->h.ne_fr * 800;
            flops = (double)m->h.ne_fr * 1200;
            break;
        case CB_K_SPMV:  // values 8 B + column 4 B per entry, row pointers, x once, y written
            bytes = 12.0 * (double)m->ks->nnz + 4.0 * (n + 1) + 16.0 * n;
            flops = 2.0 * (double)m->ks->nnz;
            break;
        default: throw cb_status_error(CB_ERR_ARG, "unknown kernel id");
        }
        once();  // warm-up (also builds a graph where one is used)
        CB_CUDA(cudaStreamSynchronize(st));
        if (!m->marks[6]) CB_CUDA(cudaEventCreate(&m->marks[6]));
        if (!m->marks[7]) CB_CUDA(cudaEventCreate(&m->marks[7]));
        CB_CUDA(cudaEventRecord(m->marks[6], st));
        for (int k = 0; k < reps; ++k) once();
        CB_CUDA(cudaEventRecord(m->marks[7], st));
        CB_CUDA(cudaEventSynchronize(m->marks[7]));
        float ms = 0;
        CB_CUDA(cudaEventElapsedTime(&ms, m->marks[6], m->marks[7]));
        *ms_per_launch = ms / reps;
        if (bytes_per_launch) *bytes_per_launch = bytes;
        if (flops_per_launch) *flops_per_launch = flops;
    });
}

int cb_eval_forces(cb_model *m, const double *x_temp, const double *dd, const double *c_ip,
                   const double *ef_ip, double *c_i, double *area_i, double *ef_i, double *ef_tr,
                   double *f)
{
    if (!m || !x_temp || !dd || !f) return CB_ERR_ARG;
    const long E = m->h.ne_sh, T = m->h.ne_tr, N = m->h.neq;
    if (E && (!c_ip || !ef_ip)) return CB_ERR_ARG;
    return guarded(m, [&] {
        cudaStream_t st = m->st;
        h2d(m->x_t, x_temp, m->h.nj * 3, st);
        h2d(m->dd, dd, N, st);
        std::vector<double> cs, es;
        if (E) {
            cs = to_soa(c_ip, E, 9);
            es = to_soa(ef_ip, E, 18);
            h2d(m->sh.c_ip, cs.data(), cs.size(), st);
            h2d(m->sh.ef_ip, es.data(), es.size(), st);
        }
        internal_force(m, m->dd, m->fcur);
        d2h(f, m->fcur, N, st);
        std::vector<double> c(9 * E), a(E), e(18 * E), n(T);
        if (E) {
            d2h(c.data(), m->sh.c_i, 9 * E, st);
            d2h(a.data(), m->sh.a_i, E, st);
            d2h(e.data(), m->sh.ef_i, 18 * E, st);
        }
        if (T) d2h(n.data(), m->tr.n_i, T, st);
        CB_CUDA(cudaStreamSynchronize(st));
        if (E) {
            if (c_i) from_soa(c, E, 9, c_i);
            if (area_i) std::memcpy(area_i, a.data(), sizeof(double) * E);
            if (ef_i) from_soa(e, E, 18, ef_i);
        }
        if (T && ef_tr)
            for (long k = 0; k < T; ++k) {
                ef_tr[2 * k] = n[k];
                ef_tr[2 * k + 1] = -n[k];
            }
    });
}

int cb_eval_tangent(cb_model *m, const double *x, const double *c_sh, const double *area_sh,
                    const double *ef_tr, long *maxa, double *ss)
{
    if (!m || !x || !ss) return CB_ERR_ARG;
    const long E = m->h.ne_sh, T = m->h.ne_tr, N = m->h.neq;
    if ((E && (!c_sh || !area_sh)) || (T && !ef_tr)) return CB_ERR_ARG;
    if (!m->bf.band) {
        m->err = "this entry point works on the band LDL^T; the handle uses the FGMRES solver";
        return CB_ERR_UNSUPPORTED;
    }
    return guarded(m, [&] {
        cudaStream_t st = m->st;
        h2d(m->x_c, x, m->h.nj * 3, st);
        std::vector<double> cs;
        if (E) {
            cs = to_soa(c_sh, E, 9);
            h2d(m->sh.c_c, cs.data(), cs.size(), st);
            h2d(m->sh.a_c, area_sh, E, st);
        }
        std::vector<double> len(T), dir(3 * T), nc(T);
        for (long e = 0; e < T; ++e) {
            int na = m->h.tr_conn[e * 2], nb = m->h.tr_conn[e * 2 + 1];
            double el[3];
            for (int k = 0; k < 3; ++k) el[k] = x[nb * 3 + k] - x[na * 3 + k];
            double L = std::sqrt(el[0] * el[0] + el[1] * el[1] + el[2] * el[2]);
            len[e] = L;
            for (int k = 0; k < 3; ++k) dir[k * T + e] = el[k] / L;
            nc[e] = ef_tr[2 * e];
        }
        if (T) {
            h2d(m->tr.len_c, len.data(), T, st);
            h2d(m->tr.dir_c, dir.data(), 3 * T, st);
            h2d(m->tr.n_c, nc.data(), T, st);
        }
        assemble_tangent(m);
        cb::BandFactor &bf = m->bf;
        const long npad = bf.nblk * bf.s;
        std::vector<double> band((size_t)bf.ld * npad);
        if (bf.fp32) {
            std::vector<float> bfl((size_t)bf.ld * npad);
            d2h(bfl.data(), (const float *)bf.band, bfl.size(), st);
            CB_CUDA(cudaStreamSynchronize(st));
            for (size_t i = 0; i < bfl.size(); ++i) band[i] = bfl[i];
        } else if (bf.dw) {
            std::vector<float> pairs(2 * (size_t)bf.ld * npad);
            d2h(pairs.data(), (const float *)bf.band, pairs.size(), st);
            CB_CUDA(cudaStreamSynchronize(st));
            for (size_t i = 0; i < band.size(); ++i) band[i] = (double)pairs[2 * i] + (double)pairs[2 * i + 1];
        } else {
            d2h(band.data(), (const double *)bf.band, band.size(), st);
            CB_CUDA(cudaStreamSynchronize(st));
        }
        if (maxa) std::memcpy(maxa, m->h.maxa.data(), sizeof(long) * (N + 1));
        for (long j = 1; j <= N; ++j) {
            long hgt = m->h.maxa[j] - m->h.maxa[j - 1] - 1;
            for (long off = 0; off <= hgt; ++off) {
                long i = j - off;  // 1-based row above the diagonal of column j
                ss[m->h.maxa[j - 1] - 1 + off] = band[(size_t)(i - 1) * bf.ld + off];
            }
        }
    });
}

int cb_factor_solve(cb_model *m, const double *rhs, double *v, double *ssd, int *det)
{
    if (!m || !rhs || !v) return CB_ERR_ARG;
    const long N = m->h.neq;
    if (!m->bf.band) {
        m->err = "this entry point works on the band LDL^T; the handle uses the FGMRES solver";
        return CB_ERR_UNSUPPORTED;
    }
    return guarded(m, [&] {
        cudaStream_t st = m->st;
        factor(m);
        h2d(m->r, rhs, N, st);
        solve(m, m->r, m->ddr);
        d2h(v, m->ddr, N, st);
        if (ssd) d2h(ssd, m->bf.ssd, N, st);
        int fl[2] = {0, 0};
        d2h(fl, m->bf.flags, 2, st);
        cb::GridBarrier bar[2]{};
        d2h(&bar[0], m->bf.bar, 1, st);
        d2h(&bar[1], m->bf.fbar, 1, st);
        CB_CUDA(cudaStreamSynchronize(st));
        if (bar[0].err || bar[1].err) throw cb_status_error(CB_ERR_TIMEOUT, "a grid barrier timed out");
        if (det) *det = fl[0];
        if (fl[1]) throw cb_status_error(CB_ERR_NUMERIC, "zero pivot in the LDL^T factorisation");
    });
}

}  // extern "C"
