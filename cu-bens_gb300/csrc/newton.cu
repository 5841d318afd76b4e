// Static Newton-Raphson (ALGFLAG 1) and modified Newton-Raphson (ALGFLAG 2)
// under load control: main.c:1820-2157.
//
// The host keeps the reference's scalar control flow: the load increments
// (lpf, dlpf, lpfmax), the subdivisions (dlpf halved down to dlpfmin, at most
// submax in a row) and the doubling of dlpf after solmin converged increments
// in a row. Every vector and element operation runs on the GPU with the
// kernels of the other drivers. Full Newton-Raphson forms the tangent of the
// latest iteration's state and refactors every iteration (one solve per
// factor: direct substitution); modified Newton-Raphson factors once per
// increment and reuses the block solve.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "cubens_gb300.h"
#include "internal.hpp"
#include "model.hpp"

namespace {

using namespace drv;

// |lam q - f| / |lam q|
double residual_norm(cb_model *m, double lam, const double *fvec)
{
    cb::launch_scale(m->q, lam, m->r, m->h.neq, m->st);
    const double num = device_dot(m, m->r, fvec, true);
    const double den = device_dot(m, m->r, nullptr);
    return den > 0 ? std::sqrt(num / den) : 0.0;
}

void push_increment(cb_model *m, double lpf)
{
    cb::MsalScalars &s = *m->sc_h;
    std::memset(&s, 0, sizeof s);
    s.lam_t = lpf;
    s.lam_old = lpf;
    s.toldisp = m->h.toldisp;
    s.tolforc = m->h.tolforc;
    s.tolener = m->h.tolener;
    s.intener_first = 1;
    s.convchk = 1;
    h2d(m->sc, m->sc_h, 1, m->st);
}

// main.c:1672-1711: zero displacements and forces, undeformed element state
void newton_begin(cb_model *m)
{
    const long N = m->h.neq;
    cudaStream_t st = m->st;
    for (double *v : {m->d, m->f, m->zero}) CB_CUDA(cudaMemsetAsync(v, 0, N * sizeof(double), st));
    CB_CUDA(cudaStreamSynchronize(st));
    m->nr_lpf = m->h.lpf0;
    m->nr_dlpf = m->h.dlpf0;
    m->nr_solcnt = m->nr_subcnt = 0;
    m->nr_incs = 0;
    m->nr_phase = 1;
}

// one converged load increment of main.c:1822-2150 (with its subdivisions)
void newton_step(cb_model *m, cb_step *out)
{
    const cb::HostModel &h = m->h;
    const long N = h.neq;
    cudaStream_t st = m->st;
    const bool full = h.alg == 1;
    out->done = 0;
    // the do { } while (lpf <= lpfmax) loop: its first pass always runs
    if (m->nr_incs > 0 && !(m->nr_lpf <= h.lpfmax)) {
        ref_success(m, "\nSolution successful\n");  // main.c:2154-2156
        out->done = 1;
        out->lam = m->nr_lpf;
        out->iterations = out->attempts = 0;
        out->residual = out->dk = 0;
        return;
    }
    int passes = 0;
    for (;;) {
        double &lpf = m->nr_lpf, &dlpf = m->nr_dlpf;
        if (passes > 0 && !(lpf <= h.lpfmax)) {
            // a subdivision left the loop (the reference ends without an error line)
            out->done = 1;
            out->lam = lpf;
            out->iterations = 0;
            out->attempts = passes;
            out->residual = out->dk = 0;
            return;
        }
        if (lpf > h.lpfmax) lpf = h.lpfmax;
        ++passes;
        const double dlpfp = dlpf;
        d2d(m->dt, m->d, N, st);
        d2d(m->fcur, m->f, N, st);
        reset_to_converged(m);
        push_increment(m, lpf);
        int itecnt = 0, convchk = 1;
        do {
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::launch_residual(m->q, m->fcur, m->r, m->sc, N, st);
                m->tm.launches += 1;
            }
            if (full || itecnt == 0) {
                assemble_tangent(m, TangentState::previous_iteration);
                factor(m);
                int fl[2] = {0, 0};
                d2h(fl, m->bf.flags, 2, st);
                CB_CUDA(cudaStreamSynchronize(st));
                if (fl[1])
                    fail_run(m, CB_ERR_NUMERIC, "singular stiffness matrix (zero pivot)",
                             "\n***ERROR*** Singular stiffness matrix\n");  // solve.c:566
            }
            solve(m, m->r, m->dd);
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::launch_axpy(m->dd, 1.0, m->dt, N, st);
                cb::launch_update_coords(m->eq_x, m->dd, m->x_t, N, st);
                m->tm.launches += 2;
            }
            std::swap(m->fcur, m->fprev);  // f_ip = f_temp
            internal_force(m, m->dd, m->fcur);
            {
                PhaseTimer t(m, &m->tm.ms_vector);
                cb::launch_test(m->dd, m->dt, m->zero, m->q, m->fcur, m->f, m->fprev, m->partial, m->sc, N, st);
                m->tm.launches += 2;
            }
            cb::MsalScalars &s = pull_scalars(m);
            if (s.test_err) fail_run(m, CB_ERR_NUMERIC, "zero norm in the convergence test", test_message(s.test_err));
            convchk = s.convchk;
            advance_iteration(m);
            ++itecnt;
        } while (convchk != 0 && itecnt <= h.itemax);
        if (convchk != 0 && m->nr_subcnt <= h.submax) {
            if (lpf == h.lpfmax)
                fail_run(m, CB_ERR_DIVERGED, "maximum allowable load proportionality factor attempted without convergence",
                         "\n***ERROR*** Maximum allowable load proportionality factor attempted without convergence\n");
            if (dlpfp == h.dlpfmin)
                fail_run(m, CB_ERR_DIVERGED, "minimum allowable increment of load proportionality factor reached",
                         "\n***ERROR*** Minimum allowable increment of load proportionality factor reached\n");
            dlpf = dlpfp / 2;
            if (dlpf < h.dlpfmin) dlpf = h.dlpfmin;
            lpf = lpf - dlpfp + dlpf;
            m->nr_subcnt++;
            m->nr_solcnt = 0;
            continue;
        }
        if (m->nr_subcnt > h.submax)
            fail_run(m, CB_ERR_DIVERGED, "maximum allowable number of subdivisions exceeded",
                     "\n***ERROR*** Maximum allowable number of subdivisions exceeded\n");  // main.c:2065-2066
        // accept (main.c:2082-2147); the newest element state is in ip
        d2d(m->d, m->dt, N, st);
        d2d(m->f, m->fcur, N, st);
        accept_state(m, true);
        out->lam = lpf;
        out->iterations = itecnt;
        out->attempts = passes;
        out->residual = residual_norm(m, lpf, m->f);
        out->dk = 0;
        m->itecnt = itecnt;
        m->nr_incs++;
        m->nr_solcnt++;
        m->nr_subcnt = 0;
        if (m->nr_solcnt >= h.solmin) {
            dlpf *= 2;
            if (dlpf > h.dlpfmax) dlpf = h.dlpfmax;
            m->nr_solcnt = 0;
        }
        lpf += dlpf;
        return;
    }
}

}  // namespace

extern "C" {

int cb_newton_begin(cb_model *m)
{
    if (!m || !m->st) return CB_ERR_ARG;
    if (m->h.alg != 1 && m->h.alg != 2) {
        m->err = "cb_newton_begin needs an ALGFLAG 1 or 2 (static Newton-Raphson) model";
        return CB_ERR_STATE;
    }
    return guarded(m, [&] { newton_begin(m); });
}

int cb_newton_step(cb_model *m, cb_step *out)
{
    if (!m || !out) return CB_ERR_ARG;
    if (m->nr_phase == 0) {
        m->err = "cb_newton_begin has not completed";
        return CB_ERR_STATE;
    }
    return guarded(m, [&] { newton_step(m, out); });
}

}  // extern "C"
