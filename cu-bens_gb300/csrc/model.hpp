// The resident model handle (cb_model) and the driver steps that the
// arc-length (msal.cu) and Newmark (newmark.cu) drivers share.
//
// State that the reference keeps as "converged" (x, c, ef, deffarea,
// defllen) and "current/previous iteration" (x_temp, c_i, c_ip, ef_i, ef_ip,
// defllen_i, defllen_ip) arrays is kept in the same three roles on the
// device.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cubens_gb300.h"
#include "internal.hpp"

#define CB_CUDA(x)                                                                         \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + \
                                     " at " __FILE__ ":" + std::to_string(__LINE__));      \
    } while (0)

struct cb_status_error : std::runtime_error {
    int code;
    cb_status_error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

struct cb_results_state;

// Pinned host copies of the small values the drivers read back every
// iteration or step, so that each read is an asynchronous copy and one
// stream synchronisation serves them all.
struct cb_host_stage {
    cb::GridBarrier bar[2];  // the solve's and the factor's grid barriers (err flags)
    int flags[2];            // the factor's det and zero-pivot flags
    double val[2];           // one reduced scalar
};

struct cb_model {
    cb::HostModel h;
    cb_options opt{};
    std::string err;
    cudaStream_t st = nullptr;
    size_t bytes = 0;
    size_t h2d_bytes = 0;
    std::vector<void *> allocs;

    // nodes and equations
    double *x0 = nullptr, *x_c = nullptr, *x_t = nullptr;
    int *eq_x = nullptr;
    // global vectors (NEQ)
    double *q = nullptr, *d = nullptr, *dp = nullptr, *dpp = nullptr, *ddq = nullptr, *ddr = nullptr,
           *dd = nullptr, *dt = nullptr, *r = nullptr, *f = nullptr, *zero = nullptr, *ssd_o = nullptr;
    double *fcur = nullptr, *fprev = nullptr;  // f_temp and f_ip
    // elements
    cb::DevShell sh;
    cb::DevTruss tr;
    cb::DevFrame fr;
    double *fr_lref = nullptr;  // lengths the frame elastic stiffness uses (llength / llength_temp)
    double *fe = nullptr;       // element force contributions
    void *kel = nullptr;        // element tangents
    int *fmap_ptr = nullptr, *fmap_src = nullptr;
    int *tmap_ptr = nullptr, *tmap_src = nullptr;
    int64_t *tmap_dst = nullptr;
    long tmap_n = 0;
    cb::BandFactor bf;           // band LDL^T (CB_SOLVER_BAND)
    cb::KrylovSolver *ks = nullptr;  // FGMRES (CB_SOLVER_FGMRES)
    cb::Mpnn *mp = nullptr;          // learned preconditioner (CB_PRECOND_LEARNED)
    int learn_steps = -1, learn_adam = 4;
    double learn_stall = 2.0;
    long bj_solves = 0, bj_iters = 0, learned_solves = 0, fallbacks = 0;
    cb::MsalScalars *sc = nullptr, *sc_h = nullptr;
    cb_host_stage *hs = nullptr;  // pinned
    double *partial = nullptr;

    // MSAL host control state (main.c:2205-2230)
    int phase = 0;  // 0 created, 1 first increment done
    double lpf = 0, lpfp = 0, lpfpp = 0, beta = 0, psi = 1, dnormallow = 0, dnorm = 0, arc = 0, qq = 0;
    double dkc = 0, lpfc = 0;
    int errchk2 = 0, subcnt = 0, imagcnt = 0, negcnt = 0, itecnt = 0;

    // Newmark (ALGFLAG 5): kinematics and per-step vectors (NEQ), frame
    // mass contributions (14 F) and the per-step joint forces (ntin NEQ)
    double *uc = nullptr, *vc = nullptr, *ac = nullptr, *uc_i = nullptr, *vc_i = nullptr, *ac_i = nullptr,
           *um = nullptr, *vm = nullptr, *am = nullptr, *sm = nullptr, *qtot = nullptr, *dyn = nullptr,
           *fp = nullptr;
    double *me = nullptr;
    double *pin = nullptr;
    // mixed Newmark: the effective stiffness in FP64 beside the FP32 factor,
    // FP64 element tangents and the refinement vectors (r, correction, scratch)
    double *band64 = nullptr, *kel64 = nullptr, *ref_r = nullptr, *ref_x = nullptr, *ref_w = nullptr;
    int nm_phase = 0;       // 0 not started, 1 running, 2 finished
    // static Newton-Raphson load control (main.c:1820-2157)
    int nr_phase = 0;       // 0 not started, 1 running
    long nr_incs = 0;       // converged increments
    double nr_lpf = 0, nr_dlpf = 0;
    int nr_solcnt = 0, nr_subcnt = 0;
    long nm_k = 0;          // next time step
    double nm_ddt = 1;      // time increment multiplier carried between steps (main.c:3452)

    cb_results_state *results = nullptr;  // open results*.txt files (results.cpp)
    // the reference's results1.txt messages of the run (its lines after the
    // input echo), in order; the results writer appends them
    std::vector<std::string> ofp0;
    bool ofp0_closed = false;  // the run's closing line has been logged
    // convergence history of the latest increment: lam, |dd|/|d|, |lam q - f|/|lam q| per iteration
    std::vector<double> iter_log;
    // arc-length with FGMRES: pivots of the LDL^T of each joint's diagonal
    // block (psi), and the converged increments so far (learning schedule)
    double *bpiv = nullptr;
    double *sh_dens = nullptr;  // linear Newmark with shells: densities (mass_sh)
    long msal_incs = 0;

    // timing
    bool timing = false;
    cb_timers tm{};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaEvent_t marks[8] = {};

    template <typename T>
    T *alloc(size_t n)
    {
        void *p = nullptr;
        size_t b = std::max<size_t>(1, n) * sizeof(T);
        CB_CUDA(cudaMalloc(&p, b));
        CB_CUDA(cudaMemsetAsync(p, 0, b, st));
        allocs.push_back(p);
        bytes += b;
        return (T *)p;
    }
};

template <typename T>
inline void h2d(T *dst, const T *src, size_t n, cudaStream_t st)
{
    if (n) CB_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, st));
}
template <typename T>
inline void d2h(T *dst, const T *src, size_t n, cudaStream_t st)
{
    if (n) CB_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, st));
}
template <typename T>
inline void d2d(T *dst, const T *src, size_t n, cudaStream_t st)
{
    if (n && dst != src) CB_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
}

// AoS (element-major, k fastest) <-> SoA (k-major) for per-element arrays
inline std::vector<double> to_soa(const double *aos, long ne, int k)
{
    std::vector<double> s((size_t)ne * k);
    for (long e = 0; e < ne; ++e)
        for (int j = 0; j < k; ++j) s[(size_t)j * ne + e] = aos[(size_t)e * k + j];
    return s;
}
inline void from_soa(const std::vector<double> &s, long ne, int k, double *aos)
{
    for (long e = 0; e < ne; ++e)
        for (int j = 0; j < k; ++j) aos[(size_t)e * k + j] = s[(size_t)j * ne + e];
}

// Adds the GPU time of a driver phase to a timer when timing is on.
struct PhaseTimer {
    cb_model *m;
    double *acc;
    PhaseTimer(cb_model *m_, double *acc_) : m(m_), acc(acc_)
    {
        if (m->timing) CB_CUDA(cudaEventRecord(m->ev[0], m->st));
    }
    ~PhaseTimer()
    {
        if (!m->timing) return;
        cudaEventRecord(m->ev[1], m->st);
        cudaEventSynchronize(m->ev[1]);
        float ms = 0;
        cudaEventElapsedTime(&ms, m->ev[0], m->ev[1]);
        *acc += ms;
    }
};

// Runs fn, turning exceptions into the handle's status code and message.
template <typename F>
int guarded(cb_model *m, F &&fn)
{
    try {
        fn();
        return CB_OK;
    } catch (const cb_status_error &e) {
        m->err = e.what();
        return e.code;
    } catch (const std::exception &e) {
        m->err = e.what();
        return CB_ERR_CUDA;
    }
}

// A line of the reference's results1.txt messages.
inline void ref_message(cb_model *m, const char *text) { m->ofp0.push_back(text); }

// The run's successful end (main.c:2155, 3139, 3957), logged once.
inline void ref_success(cb_model *m, const char *text)
{
    if (m->ofp0_closed) return;
    m->ofp0_closed = true;
    m->ofp0.push_back(text);
}

// A failure that ends the reference's run: its message, then closeio's
// "Solution failed" (misc.c:474), and the status error for the caller.
[[noreturn]] inline void fail_run(cb_model *m, int code, const std::string &msg, const char *ref)
{
    if (!m->ofp0_closed) {
        m->ofp0_closed = true;
        m->ofp0.push_back(ref);
        m->ofp0.push_back("\nSolution failed\n");
    }
    throw cb_status_error(code, msg);
}

// test()'s message for a zero denominator (misc.c:200-247): 1 the
// displacements, 2 the force increment, 3 the energy increment.
inline const char *test_message(int err)
{
    return err == 1 ? "\n***ERROR*** Displacements are zero\n"
                    : err == 2 ? "\n***ERROR*** Force increment is zero\n" : "\n***ERROR*** Energy increment is zero\n";
}

namespace drv {

// Which element state the tangent is formed from: the converged one (MSAL,
// main.c:2719-2727) or the previous iteration's (Newmark, main.c:3596-3620).
enum class TangentState { converged, previous_iteration };

void upload_model(cb_model *m);
void reset_to_converged(cb_model *m);
void advance_iteration(cb_model *m);
void accept_state(cb_model *m, bool latest_in_ip = false);
void internal_force(cb_model *m, const double *dd_vec, double *fout);
void assemble_tangent(cb_model *m, TangentState which = TangentState::converged);
void factor(cb_model *m);
void solve(cb_model *m, const double *rhs, double *x);
cb::MsalScalars &pull_scalars(cb_model *m);
double device_dot(cb_model *m, const double *a, const double *b, bool diff = false);
double device_elem(cb_model *m, const double *v, long i);
// FGMRES solve with the block-Jacobi or learned preconditioner (newmark.cu)
void krylov_solve_learned(cb_model *m, const double *rhs, double *x, bool training);

}  // namespace drv
