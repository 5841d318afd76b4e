// Checkpoint and restart of the nonlinear Newmark driver, the counterpart of
// checkPoint / restartStep (misc.c:494-716).
//
// The reference writes the converged state after a time step to
// results8.txt as %e text (kinematics, stiffness and mass, d and f, element
// forces, coordinates, triads, deformed lengths, frame and shell element
// state) and reads it back to restart. This file keeps the same converged
// state in a binary file, bit for bit, so that a run restarted from it
// continues exactly as the uninterrupted run would: the same time steps,
// iterations and displacements. The stiffness is not stored (the next step
// forms it again from the element state); the mass is.
//
// Layout (native byte order): a fixed header (magic, version, the model's
// sizes, the next step and the time increment multiplier), then each state
// array as its length followed by its values, in a fixed order.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cubens_gb300.h"
#include "internal.hpp"
#include "model.hpp"

namespace {

constexpr char kMagic[8] = {'C', 'B', 'C', 'K', 'P', 'T', '0', '1'};

struct CkptHeader {
    char magic[8];
    int32_t version;
    int32_t algflag;
    int64_t neq, nj, ne_tr, ne_fr, ne_sh;
    int64_t next_step;  // nm_k: the next time step to run
    double ddt;         // nm_ddt: the time increment multiplier carried between steps
    int32_t phase;      // nm_phase
    int32_t narrays;
};

// The converged state, in file order: (device pointer, element count).
std::vector<std::pair<double *, size_t>> state_arrays(cb_model *m)
{
    const cb::HostModel &h = m->h;
    const size_t N = (size_t)h.neq, NJ = (size_t)h.nj, T = (size_t)h.ne_tr, F = (size_t)h.ne_fr,
                 E = (size_t)h.ne_sh;
    std::vector<std::pair<double *, size_t>> a = {
        {m->uc, N}, {m->vc, N}, {m->ac, N}, {m->sm, N}, {m->d, N}, {m->f, N}, {m->x_c, 3 * NJ},
    };
    if (T) {
        a.push_back({m->tr.len_c, T});
        a.push_back({m->tr.dir_c, 3 * T});
        a.push_back({m->tr.n_c, T});
    }
    if (F) {
        a.push_back({m->fr.c_c, 9 * F});
        a.push_back({m->fr.ef_c, 14 * F});
        a.push_back({m->fr.len_c, F});
        a.push_back({m->fr_lref, F});
    }
    if (E) {
        a.push_back({m->sh.c_c, 9 * E});
        a.push_back({m->sh.a_c, E});
        a.push_back({m->sh.ef_c, 18 * E});
    }
    return a;
}

void require_newmark(cb_model *m)
{
    if (m->h.alg != 5)
        throw cb_status_error(CB_ERR_UNSUPPORTED, "checkpoints hold the nonlinear Newmark state (ALGFLAG 5), "
                                                  "as the reference's checkPoint does");
    if (m->nm_phase == 0) throw cb_status_error(CB_ERR_STATE, "cb_newmark_begin has not completed");
}

struct File {
    FILE *f = nullptr;
    File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
};

}  // namespace

extern "C" {

int cb_checkpoint_save(cb_model *m, const char *path)
{
    if (!m || !path) return CB_ERR_ARG;
    return guarded(m, [&] {
        require_newmark(m);
        const auto arrays = state_arrays(m);
        std::vector<std::vector<double>> host(arrays.size());
        for (size_t k = 0; k < arrays.size(); ++k) {
            host[k].resize(arrays[k].second);
            d2h(host[k].data(), arrays[k].first, arrays[k].second, m->st);
        }
        CB_CUDA(cudaStreamSynchronize(m->st));
        CkptHeader hd{};
        std::memcpy(hd.magic, kMagic, sizeof kMagic);
        hd.version = 1;
        hd.algflag = m->h.alg;
        hd.neq = m->h.neq;
        hd.nj = m->h.nj;
        hd.ne_tr = m->h.ne_tr;
        hd.ne_fr = m->h.ne_fr;
        hd.ne_sh = m->h.ne_sh;
        hd.next_step = m->nm_k;
        hd.ddt = m->nm_ddt;
        hd.phase = m->nm_phase;
        hd.narrays = (int32_t)arrays.size();
        File out(path, "wb");
        if (!out.f) throw cb_status_error(CB_ERR_ARG, "cannot open the checkpoint file for writing");
        bool ok = std::fwrite(&hd, sizeof hd, 1, out.f) == 1;
        for (const auto &v : host) {
            const int64_t n = (int64_t)v.size();
            ok = ok && std::fwrite(&n, sizeof n, 1, out.f) == 1;
            ok = ok && (n == 0 || std::fwrite(v.data(), sizeof(double), v.size(), out.f) == v.size());
        }
        if (!ok) throw cb_status_error(CB_ERR_ARG, "short write to the checkpoint file");
    });
}

int cb_checkpoint_load(cb_model *m, const char *path)
{
    if (!m || !path) return CB_ERR_ARG;
    return guarded(m, [&] {
        require_newmark(m);
        File in(path, "rb");
        if (!in.f) throw cb_status_error(CB_ERR_ARG, "cannot open the checkpoint file");
        CkptHeader hd{};
        if (std::fread(&hd, sizeof hd, 1, in.f) != 1 || std::memcmp(hd.magic, kMagic, sizeof kMagic) != 0 ||
            hd.version != 1)
            throw cb_status_error(CB_ERR_PARSE, "not a checkpoint file of this format");
        const auto arrays = state_arrays(m);
        if (hd.algflag != m->h.alg || hd.neq != m->h.neq || hd.nj != m->h.nj || hd.ne_tr != m->h.ne_tr ||
            hd.ne_fr != m->h.ne_fr || hd.ne_sh != m->h.ne_sh || hd.narrays != (int32_t)arrays.size())
            throw cb_status_error(CB_ERR_ARG, "the checkpoint belongs to a model of other sizes");
        if (hd.next_step < 0 || hd.next_step > m->h.nsteps || !(hd.ddt > 0) || hd.phase < 1 || hd.phase > 2)
            throw cb_status_error(CB_ERR_PARSE, "inconsistent checkpoint header");
        std::vector<std::vector<double>> host(arrays.size());
        for (size_t k = 0; k < arrays.size(); ++k) {
            int64_t n = -1;
            if (std::fread(&n, sizeof n, 1, in.f) != 1 || n != (int64_t)arrays[k].second)
                throw cb_status_error(CB_ERR_PARSE, "checkpoint array of the wrong length");
            host[k].resize((size_t)n);
            if (n && std::fread(host[k].data(), sizeof(double), (size_t)n, in.f) != (size_t)n)
                throw cb_status_error(CB_ERR_PARSE, "truncated checkpoint file");
        }
        // everything read: only now does the handle's state change
        for (size_t k = 0; k < arrays.size(); ++k) h2d(arrays[k].first, host[k].data(), host[k].size(), m->st);
        CB_CUDA(cudaStreamSynchronize(m->st));
        m->nm_k = hd.next_step;
        m->nm_ddt = hd.ddt;
        m->nm_phase = hd.phase;
    });
}

}  // extern "C"
