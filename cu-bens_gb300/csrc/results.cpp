// results*.txt writers: the layout and records of the reference's output()
// (misc.c:345-451) for the resident API, so that a run through cb_* leaves
// the same results2.txt (displacements), results3.txt (truss forces),
// results4.txt (frame forces) and results5.txt (shell forces) as main.c,
// and the same results1.txt: the input echo (echo.cpp) followed by the
// run's messages (errors, subdivisions of a Newmark time step, the closing
// "Solution successful" or "Solution failed"), appended as they occur.
//
// A record is the converged state on the device: d and the element forces
// of the converged configuration, averaged over the element's nodes as
// output() does. The %e formatting of large models is spread over host
// threads (chunks formatted in parallel, written in order).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "cubens_gb300.h"
#include "internal.hpp"
#include "model.hpp"

namespace {

struct ResultFiles {
    FILE *f[4] = {nullptr, nullptr, nullptr, nullptr};  // results2..results5
    FILE *r1 = nullptr;                                  // results1.txt
    size_t r1_lines = 0;                                 // messages written so far
};

// Append the run's messages logged since the last call.
void flush_messages(cb_model *m, ResultFiles &r)
{
    if (!r.r1) return;
    for (; r.r1_lines < m->ofp0.size(); ++r.r1_lines) std::fputs(m->ofp0[r.r1_lines].c_str(), r.r1);
    std::fflush(r.r1);
}

// "\t%e" for every value, formatted in chunks by up to `threads` threads
void write_values(FILE *out, const std::vector<double> &v)
{
    const size_t n = v.size();
    if (n == 0) return;
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t chunks = std::min<size_t>(hw, (n + 4095) / 4096);
    std::vector<std::string> parts(chunks);
    auto work = [&](size_t c) {
        const size_t a = n * c / chunks, b = n * (c + 1) / chunks;
        std::string &s = parts[c];
        s.reserve((b - a) * 15);
        char buf[40];
        for (size_t i = a; i < b; ++i) {
            const int k = std::snprintf(buf, sizeof buf, "\t%e", v[i]);
            s.append(buf, (size_t)k);
        }
    };
    if (chunks == 1) {
        work(0);
    } else {
        std::vector<std::thread> ts;
        for (size_t c = 0; c < chunks; ++c) ts.emplace_back(work, c);
        for (auto &t : ts) t.join();
    }
    for (const std::string &s : parts) std::fwrite(s.data(), 1, s.size(), out);
}

std::vector<double> pull(const double *dev, size_t n, cudaStream_t st)
{
    std::vector<double> h(n);
    if (n) CB_CUDA(cudaMemcpyAsync(h.data(), dev, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    return h;
}

}  // namespace

struct cb_results_state : ResultFiles {};

extern "C" {

int cb_results_open(cb_model *m, const char *dir)
{
    if (!m || !dir) return CB_ERR_ARG;
    return guarded(m, [&] {
        if (m->results) throw cb_status_error(CB_ERR_STATE, "results files are already open");
        auto *r = new cb_results_state();
        for (int k = 0; k < 4; ++k) {
            const std::string path = std::string(dir) + "/results" + std::to_string(k + 2) + ".txt";
            r->f[k] = std::fopen(path.c_str(), "w");
            if (!r->f[k]) {
                for (int q = 0; q < k; ++q) std::fclose(r->f[q]);
                delete r;
                throw cb_status_error(CB_ERR_ARG, "cannot open " + path);
            }
        }
        const std::string p1 = std::string(dir) + "/results1.txt";
        r->r1 = std::fopen(p1.c_str(), "w");
        if (!r->r1) {
            for (FILE *f : r->f) std::fclose(f);
            delete r;
            throw cb_status_error(CB_ERR_ARG, "cannot open " + p1);
        }
        const std::string echo = cb::input_echo(m->h);
        std::fwrite(echo.data(), 1, echo.size(), r->r1);
        flush_messages(m, *r);
        const cb::HostModel &h = m->h;
        FILE *o1 = r->f[0], *o2 = r->f[1], *o3 = r->f[2], *o4 = r->f[3];
        // layout lines (output flag 0)
        std::fprintf(o1, "Model Displacements:\n\tLambda\t\tIterations");
        for (long i = 0; i < h.neq; ++i) {
            if (i + 1 <= 1000) std::fprintf(o1, "\tDOF %ld\t", i + 1);
            else std::fprintf(o1, "DOF %ld\t", i + 1);
        }
        if (h.ne_tr > 0) {
            std::fprintf(o2, "Truss Element Forces (averaged):\n\tLambda\t\tIterations");
            std::fprintf(o2, "\t");
            for (long i = 0; i < h.ne_tr; ++i) std::fprintf(o2, "Element %ld\t", i + 1);
        }
        if (h.ne_fr > 0) {
            std::fprintf(o3, "Frame Element Forces (averaged):\n\tLambda\t\tIterations");
            std::fprintf(o2, "\t");  // the reference writes this tab into the truss file
            for (long i = 0; i < h.ne_fr; ++i) std::fprintf(o3, "Element %ld\t\t\t\t\t\t\t\t\t\t\t\t\t", i + 1);
            std::fprintf(o3, "\n\t\t\t\t\t");
            for (long i = 0; i < h.ne_fr; ++i) {
                std::fprintf(o3, "X-Force\t\tY-Force\t\tZ-Force\t\tX-Moment\tY-Moment\t");
                std::fprintf(o3, "Z-Moment\tBi-Moment\t");
            }
        }
        if (h.ne_sh > 0) {
            std::fprintf(o4, "Shell Element Forces (averaged):\n\tLambda\t\tIterations");
            std::fprintf(o2, "\t");  // likewise
            for (long i = 0; i < h.ne_sh; ++i) std::fprintf(o4, "Element %ld\t\t\t\t\t\t\t\t\t\t\t", i + 1);
            std::fprintf(o4, "\n\t\t\t\t\t");
            for (long i = 0; i < h.ne_sh; ++i) {
                std::fprintf(o4, "X-Force\t\tY-Force\t\tZ-Force\t\tX-Moment\tY-Moment\t");
                std::fprintf(o4, "Z-Moment\t");
            }
        }
        m->results = r;
    });
}

int cb_results_write(cb_model *m, double lam, int iterations)
{
    if (!m) return CB_ERR_ARG;
    if (!m->results) {
        m->err = "cb_results_open has not been called";
        return CB_ERR_STATE;
    }
    return guarded(m, [&] {
        const cb::HostModel &h = m->h;
        const long T = h.ne_tr, F = h.ne_fr, E = h.ne_sh;
        cudaStream_t st = m->st;
        std::vector<double> d = pull(m->d, h.neq, st);
        std::vector<double> nt = pull(T ? m->tr.n_c : nullptr, T, st);
        std::vector<double> ef = pull(F ? m->fr.ef_c : nullptr, 14 * F, st);
        std::vector<double> es = pull(E ? m->sh.ef_c : nullptr, 18 * E, st);
        CB_CUDA(cudaStreamSynchronize(st));
        flush_messages(m, *m->results);
        FILE **o = m->results->f;
        std::fprintf(o[0], "\n\t%e\t%d\t", lam, iterations);
        write_values(o[0], d);
        if (T > 0) {
            // the element forces are (N, -N)
            std::vector<double> v(T);
            for (long i = 0; i < T; ++i) v[i] = (std::fabs(nt[i]) + std::fabs(-nt[i])) / 2;
            std::fprintf(o[1], "\n\t%e\t%d\t", lam, iterations);
            write_values(o[1], v);
        }
        if (F > 0) {
            std::vector<double> v(7 * F);
            for (long i = 0; i < F; ++i)
                for (int j = 0; j < 7; ++j)
                    v[i * 7 + j] = (std::fabs(ef[j * F + i]) + std::fabs(ef[(7 + j) * F + i])) / 2;
            std::fprintf(o[2], "\n\t%e\t%d\t", lam, iterations);
            write_values(o[2], v);
        }
        if (E > 0) {
            std::vector<double> v(6 * E);
            for (long i = 0; i < E; ++i)
                for (int j = 0; j < 6; ++j)
                    v[i * 6 + j] = (std::fabs(es[j * E + i]) + std::fabs(es[(6 + j) * E + i]) +
                                    std::fabs(es[(12 + j) * E + i])) /
                                   3;
            std::fprintf(o[3], "\n\t%e\t%d\t", lam, iterations);
            write_values(o[3], v);
        }
    });
}

int cb_results_close(cb_model *m)
{
    if (!m) return CB_ERR_ARG;
    if (!m->results) return CB_OK;
    int rc = CB_OK;
    flush_messages(m, *m->results);
    for (FILE *f : m->results->f)
        if (f && std::fclose(f) != 0) rc = CB_ERR_ARG;
    if (m->results->r1 && std::fclose(m->results->r1) != 0) rc = CB_ERR_ARG;
    delete m->results;
    m->results = nullptr;
    return rc;
}

}  // extern "C"
