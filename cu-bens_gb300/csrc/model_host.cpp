// model_def reader, equation numbering, skyline profile and the gather maps
// that drive the deterministic (atomics-free) assembly on the GPU.
//
// Reading order follows main.c:340-433 (header), struc model.c:95-264
// (incidences, constraints), skylin model.c:1156-1201 (prescribed-motion
// list of dynamic analyses), main.c:1395 (coordinates), prop_tr truss.c:66,
// prop_fr frame.c:43-224, prop_sh shell.c:61 (properties), load
// model.c:1313-1335 / 1492-1609 (joint loads, static or per time step) and
// msal arc.c:48 / main.c:2240-2245 (MSAL controls) or main.c:3320-3326
// (Newmark controls).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <thread>

#include "internal.hpp"

namespace cb {

namespace {

struct Tokens {
    const char *p, *end;
    bool ok = true;
    double next()
    {
        while (p < end && (*p == ',' || *p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
        if (p >= end) {
            ok = false;
            return 0;
        }
        char *e = nullptr;
        double v = std::strtod(p, &e);
        if (e == p) {
            ok = false;
            return 0;
        }
        p = e;
        return v;
    }
};

}  // namespace

std::string parse_model_def(const char *text, size_t len, HostModel &m, int &status)
{
    status = CB_ERR_PARSE;
    Tokens t{text, text + len};
    int ana = (int)t.next();
    if (ana == 4) {
        status = CB_ERR_UNSUPPORTED;
        return "ANAFLAG 4 (fluid-structure interaction) is outside the GPU path";
    }
    int alg = (int)t.next();
    if (!t.ok) return "empty model_def";
    if (!(ana == 2 || (ana == 1 && alg == 4))) {
        status = CB_ERR_UNSUPPORTED;
        return "the GPU path takes ANAFLAG 2 (second-order elastic), and ANAFLAG 1 (first-order elastic) with "
               "ALGFLAG 4 (linear Newmark)";
    }
    if (alg == 4 && ana != 1) {
        status = CB_ERR_UNSUPPORTED;
        return "ALGFLAG 4 (linear Newmark) is a first-order elastic analysis: ANAFLAG 1 (main.c:393)";
    }
    if (alg != 1 && alg != 2 && alg != 3 && alg != 4 && alg != 5) {
        status = CB_ERR_UNSUPPORTED;
        return "only ALGFLAG 1 and 2 (static Newton-Raphson, modified Newton-Raphson), 3 (modified spherical "
               "arc length), 4 (linear Newmark) and 5 (nonlinear Newmark) are on the GPU path";
    }
    m.alg = alg;
    m.echo.ana = ana;
    if (alg >= 4) {
        (void)t.next();  // CHKPT
        int rflag = (int)t.next();
        if (rflag != 0) {
            status = CB_ERR_UNSUPPORTED;
            return "restart from a checkpoint (RFLAG 1) is not supported";
        }
    }
    int slv = (int)t.next();
    int opt = (int)t.next();
    if (slv != 0) {
        status = CB_ERR_UNSUPPORTED;
        return "SLVFLAG must be 0 (the skyline path; the others are broken for MSAL in the reference)";
    }
    if (opt != 1) {
        status = CB_ERR_UNSUPPORTED;
        return "OPTFLAG 2 (Collins renumbering) is not supported; renumber before";
    }
    m.nj = (long)t.next();
    m.ne_tr = (long)t.next();
    m.ne_fr = (long)t.next();
    m.ne_sh = (long)t.next();
    long nsbr = (long)t.next(), nfbr = (long)t.next();
    if (!t.ok || m.nj <= 0) return "bad control block";
    if (nsbr || nfbr) {
        status = CB_ERR_UNSUPPORTED;
        return "brick elements are not on the GPU path";
    }
    if ((alg == 5 && (m.ne_tr || m.ne_sh)) || (alg == 4 && (m.ne_tr || (m.ne_sh && m.ne_fr)))) {
        status = CB_ERR_UNSUPPORTED;
        return "the GPU Newmark path takes frame-only models, and the linear one also shell-only models "
               "(the mass routines index the shared density array without the element-type offsets, "
               "frame.c:1357-1363, shell.c:1558)";
    }
    const long NJ = m.nj, F = m.ne_fr;
    std::vector<char> has_tr(NJ, 0), has_sh(NJ, 0);
    std::vector<int> nfr(NJ, 0), wrp(NJ, 0);
    m.tr_conn.resize(2 * m.ne_tr);
    for (long i = 0; i < 2 * m.ne_tr; ++i) {
        long j = (long)t.next() - 1;
        if (j < 0 || j >= NJ) return "truss incidence out of range";
        m.tr_conn[i] = (int)j;
        has_tr[j] = 1;
    }
    m.fr_conn.resize(2 * F);
    for (long i = 0; i < 2 * F; ++i) {
        long j = (long)t.next() - 1;
        if (j < 0 || j >= NJ) return "frame incidence out of range";
        m.fr_conn[i] = (int)j;
        nfr[j]++;
    }
    m.sh_conn.resize(3 * m.ne_sh);
    for (long i = 0; i < 3 * m.ne_sh; ++i) {
        long j = (long)t.next() - 1;
        if (j < 0 || j >= NJ) return "shell incidence out of range";
        m.sh_conn[i] = (int)j;
        has_sh[j] = 1;
    }
    // constraints (struc, model.c:216-264); "j,7,r" also sets the warping
    // restraint flag r: 1 gives every member end at the joint its own
    // warping DOF
    m.jcode.assign(NJ * 7, -1);
    for (;;) {
        long j = (long)t.next(), k = (long)t.next();
        if (!t.ok) return "constraint list not terminated";
        if (j == 0) break;
        if (j < 0 || j > NJ || k < 1 || k > 7) return "joint constraint input not recognized";
        if (k == 7) wrp[j - 1] = (int)t.next();
        m.jcode[(j - 1) * 7 + k - 1] = 0;
    }
    m.echo.wrp = wrp;
    // DOFs no element type uses (model.c:267-285): truss joints keep 1-3,
    // shell joints 1-6, frame joints all 7
    for (long i = 0; i < NJ; ++i) {
        if (nfr[i] == 0) {
            if (!has_sh[i]) {
                int from = has_tr[i] ? 3 : 0;
                for (int j = from; j < 7; ++j) m.jcode[i * 7 + j] = 0;
            } else {
                m.jcode[i * 7 + 6] = 0;
            }
        }
    }
    // equation numbers (codes, model.c:941-961)
    long neq = 0;
    for (long i = 0; i < NJ; ++i) {
        for (int j = 0; j < 6; ++j)
            if (m.jcode[i * 7 + j] != 0) m.jcode[i * 7 + j] = ++neq;
        if (m.jcode[i * 7 + 6] != 0) {
            m.jcode[i * 7 + 6] = ++neq;
        } else if (wrp[i] == 1) {
            m.jcode[i * 7 + 6] = ++neq;
            neq += nfr[i] - 1;
        }
    }
    m.neq = neq;
    if (neq == 0) return "no free degrees of freedom";
    // frame member codes; a joint with one warping DOF per member counts
    // them up over its members in element order (model.c:1007-1032)
    m.fr_mc.assign(14 * F, 0);
    {
        std::vector<int> cnt(nfr);
        for (long e = 0; e < F; ++e)
            for (int a = 0; a < 2; ++a) {
                long j = m.fr_conn[e * 2 + a];
                for (int d = 0; d < 6; ++d) m.fr_mc[e * 14 + a * 7 + d] = m.jcode[j * 7 + d];
                if (wrp[j] == 1) {
                    m.fr_mc[e * 14 + a * 7 + 6] = m.jcode[j * 7 + 6] + nfr[j] - cnt[j];
                    cnt[j]--;
                } else {
                    m.fr_mc[e * 14 + a * 7 + 6] = m.jcode[j * 7 + 6];
                }
            }
    }
    if (alg >= 4) {
        // prescribed support motion list (skylin, model.c:1156-1201)
        long j = (long)t.next();
        (void)t.next();
        if (!t.ok) return "model_def ended before the prescribed-motion list";
        if (j != 0) {
            status = CB_ERR_UNSUPPORTED;
            return "prescribed support motion (NBC > 0) is not supported";
        }
    }
    // skyline column heights (skylin, model.c:1204-1277)
    std::vector<long> kht(neq, 0);
    auto profile = [&](const long *mc, int nd) {
        long mn = neq;
        for (int k = 0; k < nd; ++k)
            if (mc[k] > 0 && mc[k] < mn) mn = mc[k];
        for (int k = 0; k < nd; ++k)
            if (mc[k] != 0 && mc[k] - mn > kht[mc[k] - 1]) kht[mc[k] - 1] = mc[k] - mn;
    };
    for (long e = 0; e < m.ne_tr; ++e) {
        long mc[6];
        for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 3; ++d) mc[a * 3 + d] = m.jcode[m.tr_conn[e * 2 + a] * 7 + d];
        profile(mc, 6);
    }
    for (long e = 0; e < F; ++e) profile(&m.fr_mc[e * 14], 14);
    for (long e = 0; e < m.ne_sh; ++e) {
        long mc[18];
        for (int a = 0; a < 3; ++a)
            for (int d = 0; d < 6; ++d) mc[a * 6 + d] = m.jcode[m.sh_conn[e * 3 + a] * 7 + d];
        profile(mc, 18);
    }
    m.maxa.resize(neq + 1);
    m.maxa[0] = 1;
    m.bw = 0;
    for (long i = 0; i < neq; ++i) {
        m.maxa[i + 1] = m.maxa[i] + kht[i] + 1;
        m.bw = std::max(m.bw, kht[i]);
    }
    m.lss = m.maxa[neq] - 1;
    m.x0.resize(NJ * 3);
    for (long i = 0; i < NJ * 3; ++i) m.x0[i] = t.next();
    m.tr_e.resize(m.ne_tr);
    m.tr_a.resize(m.ne_tr);
    m.echo.tr_dens.resize(m.ne_tr);
    m.echo.tr_yield.resize(m.ne_tr);
    for (long i = 0; i < m.ne_tr; ++i) {
        m.tr_e[i] = t.next();
        m.tr_a[i] = t.next();
        m.echo.tr_dens[i] = t.next();   // density
        m.echo.tr_yield[i] = t.next();  // yield stress (ANAFLAG 3 only)
    }
    // frame properties (prop_fr, frame.c:43-224)
    m.fr_prop.resize(8 * F);
    m.fr_aux.resize(3 * F);
    if (F > 0) {
        for (long i = 0; i < F * 8; ++i) m.fr_prop[i] = t.next();
        long j = (long)t.next();
        for (int k = 0; k < 6; ++k) (void)t.next();
        if (!t.ok) return "model_def ended inside the frame properties";
        if (j != 0) {
            status = CB_ERR_UNSUPPORTED;
            return "frame member end offsets are not supported";
        }
        for (long i = 0; i < F * 3; ++i) m.fr_aux[i] = t.next();
        m.echo.fr_yield.resize(3 * F);
        for (long i = 0; i < F * 3; ++i) m.echo.fr_yield[i] = t.next();  // yield stress, plastic moduli
        j = (long)t.next();
        for (int k = 0; k < 4; ++k) (void)t.next();
        if (!t.ok) return "model_def ended inside the frame properties";
        if (j != 0) {
            status = CB_ERR_UNSUPPORTED;
            return "frame member end releases are not supported";
        }
    }
    m.sh_e.resize(m.ne_sh);
    m.sh_nu.resize(m.ne_sh);
    m.sh_t.resize(m.ne_sh);
    m.echo.sh_dens.resize(m.ne_sh);
    m.echo.sh_yield.resize(m.ne_sh);
    for (long i = 0; i < m.ne_sh; ++i) {
        m.sh_e[i] = t.next();
        m.sh_nu[i] = t.next();
        m.sh_t[i] = t.next();
        m.echo.sh_dens[i] = t.next();
        m.echo.sh_yield[i] = t.next();
    }
    if (!t.ok) return "model_def ended inside the properties";
    m.q.assign(neq, 0.0);
    if (alg >= 4) {
        // time points (main.c:1600-1607) and per-step joint forces (load,
        // model.c:1516-1549): the lines of one DOF are consecutive time
        // points; in a nonlinear Newmark model a zero force is stored as 1e-30
        long ntsteps = (long)t.next();
        m.ttot = t.next();
        if (!t.ok || ntsteps <= 0) return "bad time-step line";
        m.dt = m.ttot / (double)ntsteps;
        m.ntin = ntsteps + 1;
        m.nsteps = (long)(m.ttot / m.dt + 1);
        if (m.nsteps != m.ntin) {
            status = CB_ERR_UNSUPPORTED;
            return "ttot/dt + 1 differs from the number of input time points";
        }
        m.pin.assign((size_t)m.ntin * neq, 0.0);
        long kps = 0, i = 0;
        for (;;) {
            long jt = (long)t.next();
            long dir = (long)t.next();
            double mag = t.next();
            if (!t.ok) return "joint load list not terminated";
            if (jt == 0) break;
            if (jt < 0 || jt > NJ || dir < 1 || dir > 7) return "joint load out of range";
            if (alg == 5 && mag == 0) mag = 1e-30;
            long ks = m.jcode[(jt - 1) * 7 + dir - 1];
            if (ks != kps) i = 0;
            if (ks != 0) {
                if (i >= m.ntin) return "more load lines for one DOF than input time points";
                m.pin[(size_t)i * neq + (ks - 1)] = mag;
            }
            kps = ks;
            ++i;
        }
        long jt = (long)t.next();
        (void)t.next();
        (void)t.next();
        if (!t.ok) return "prescribed displacement list not terminated";
        if (jt != 0) {
            status = CB_ERR_UNSUPPORTED;
            return "prescribed displacements are not supported";
        }
        // initial conditions (load, model.c:1583-1604): the linear driver
        // starts from them; the nonlinear one zeroes its motion before the
        // first step (main.c:3440-3443)
        m.um0.assign(neq, 0.0);
        m.vm0.assign(neq, 0.0);
        m.am0.assign(neq, 0.0);
        for (;;) {
            jt = (long)t.next();
            const long dir = (long)t.next();
            const double d0 = t.next(), v0 = t.next(), a0 = t.next();
            if (!t.ok) return "initial condition list not terminated";
            if (jt == 0) break;
            if (jt < 0 || jt > NJ || dir < 1 || dir > 7) return "initial condition out of range";
            const long k = m.jcode[(jt - 1) * 7 + dir - 1];
            if (k != 0) {
                if (d0 != 0) m.um0[k - 1] = d0;
                if (v0 != 0) m.vm0[k - 1] = v0;
                if (a0 != 0) m.am0[k - 1] = a0;
            }
        }
        if (alg == 4) {
            // linear Newmark controls (main.c:3184, 3192)
            m.numopt = t.next();
            m.spectrds = t.next();
            m.lpfmax = t.next();
            if (!t.ok) return "model_def ended inside the linear Newmark controls";
            if (m.numopt == 0 && m.spectrds != 1) return "invalid spectral radius for Newmark without dissipation";
            status = CB_OK;
            return "";
        }
        m.numopt = t.next();
        m.spectrds = t.next();
        m.lpfmax = t.next();
        m.lpf0 = t.next();
        m.dlpf0 = t.next();
        m.dlpfmax = t.next();
        m.dlpfmin = t.next();
        m.itemax = (int)t.next();
        m.submax = (int)t.next();
        m.solmin = (int)t.next();
        m.toldisp = t.next();
        m.tolforc = t.next();
        m.tolener = t.next();
        if (!t.ok) return "model_def ended inside the Newmark controls";
        if (m.numopt == 0 && m.spectrds != 1) return "invalid spectral radius for Newmark without dissipation";
        status = CB_OK;
        return "";
    }
    bool any_load = false;
    for (;;) {
        long jt = (long)t.next();
        long dir = (long)t.next();
        double mag = t.next();
        if (!t.ok) return "joint load list not terminated";
        if (jt == 0) break;
        if (jt < 0 || jt > NJ || dir < 1 || dir > 7) return "joint load out of range";
        long k = m.jcode[(jt - 1) * 7 + dir - 1];
        if (k != 0) m.q[k - 1] = mag;
        any_load = true;
        m.echo.load_jt.push_back(jt);
        m.echo.load_dir.push_back((int)dir);
        m.echo.load_mag.push_back(mag);
    }
    if (F > 0) {
        long fr = (long)t.next();
        (void)t.next();
        (void)t.next();
        if (!t.ok) return "distributed load list not terminated";
        if (fr != 0) {
            status = CB_ERR_UNSUPPORTED;
            return "frame distributed loads are not supported";
        }
    }
    if (!any_load) return "no forces present in input file";
    if (alg == 1 || alg == 2) {
        // load-control parameters (main.c:1809-1812)
        m.lpfmax = t.next();
        m.lpf0 = t.next();
        m.dlpf0 = t.next();
        m.dlpfmax = t.next();
        m.dlpfmin = t.next();
        m.itemax = (int)t.next();
        m.submax = (int)t.next();
        m.solmin = (int)t.next();
        m.toldisp = t.next();
        m.tolforc = t.next();
        m.tolener = t.next();
        if (!t.ok) return "model_def ended inside the Newton-Raphson controls";
        status = CB_OK;
        return "";
    }
    long jt = (long)t.next();
    long dir = (long)t.next();
    m.dk = t.next();
    m.alpha = t.next();
    m.psi_thresh = t.next();
    m.iteopt = (int)t.next();
    m.lpfmax = t.next();
    m.dkimax = t.next();
    m.itemax = (int)t.next();
    m.submax = (int)t.next();
    m.imagmax = (int)t.next();
    m.negmax = (int)t.next();
    m.toldisp = t.next();
    m.tolforc = t.next();
    m.tolener = t.next();
    if (!t.ok) return "model_def ended inside the MSAL controls";
    if (jt < 1 || jt > NJ || dir < 1 || dir > 7) return "prescribed displacement joint out of range";
    m.echo.dk_jt = jt;
    m.echo.dk_dir = (int)dir;
    m.dkdof = m.jcode[(jt - 1) * 7 + dir - 1] - 1;
    if (m.dkdof < 0) return "initially prescribed displacement at fixed degree of freedom";
    status = CB_OK;
    return "";
}

// Force map. The reference accumulates forces_tr, forces_fr, forces_sh in
// that order, elements in order, so every equation's list is sorted by
// (type, element). The contribution buffer holds the shell element forces at
// [k*E + e] (k < 18), the truss forces at 18E + [k*T + e] (k < 6) and the
// frame forces at 18E + 6T + [k*F + e] (k < 14).
void build_force_map(const HostModel &m, GatherMap &g)
{
    const long E = m.ne_sh, T = m.ne_tr, F = m.ne_fr;
    std::vector<std::vector<int>> lists(m.neq);
    for (long e = 0; e < T; ++e)
        for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 3; ++d) {
                long q = m.jcode[m.tr_conn[e * 2 + a] * 7 + d];
                if (q) lists[q - 1].push_back((int)(18 * E + (a * 3 + d) * T + e));
            }
    for (long e = 0; e < F; ++e)
        for (int k = 0; k < 14; ++k) {
            long q = m.fr_mc[e * 14 + k];
            if (q) lists[q - 1].push_back((int)(18 * E + 6 * T + k * F + e));
        }
    for (long e = 0; e < E; ++e)
        for (int a = 0; a < 3; ++a)
            for (int d = 0; d < 6; ++d) {
                long q = m.jcode[m.sh_conn[e * 3 + a] * 7 + d];
                if (q) lists[q - 1].push_back((int)((a * 6 + d) * E + e));
            }
    g.ptr.assign(m.neq + 1, 0);
    g.src.clear();
    for (long i = 0; i < m.neq; ++i) {
        g.src.insert(g.src.end(), lists[i].begin(), lists[i].end());
        g.ptr[i + 1] = (int)g.src.size();
    }
    g.dst.clear();
}

// Index of the local pair (ie <= je) of an nd x nd element matrix in its
// packed upper triangle (row-major).
static inline int packed(int ie, int je, int nd) { return ie * nd - ie * (ie - 1) / 2 + (je - ie); }

// Tangent contributions. Element matrices are packed upper triangles,
// shells at [p*E + e] (p < 171), trusses at 171E + [p*T + e] (p < 21),
// frames at 171E + 21T + [p*F + e] (p < 105). A local pair (ie <= je) adds
// K[ie][je] to the global pair (max(i,j), min(i,j)) of the lower triangle,
// as the reference adds K[ie][je] for ie <= je into its skyline
// (truss.c:170-193, frame.c:328-344, shell.c:307-329). Pairs come out in the
// order stiff_tr, stiff_fr, stiff_sh add them (truss, frame, shell; element).
namespace {
struct TangentPair {
    long r, c;  // 0-based, r >= c
    int src;
};

void collect_tangent_pairs(const HostModel &m, std::vector<TangentPair> &all)
{
    const long E = m.ne_sh, T = m.ne_tr, F = m.ne_fr;
    all.clear();
    all.reserve((size_t)(171 * E + 21 * T + 105 * F));
    auto add = [&](const long *mc, int ie, int je, int src) {
        if (!mc[ie] || !mc[je]) return;
        all.push_back({std::max(mc[ie], mc[je]) - 1, std::min(mc[ie], mc[je]) - 1, src});
    };
    for (long e = 0; e < T; ++e) {
        long mc[6];
        for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 3; ++d) mc[a * 3 + d] = m.jcode[m.tr_conn[e * 2 + a] * 7 + d];
        for (int je = 0; je < 6; ++je)
            for (int ie = 0; ie <= je; ++ie) add(mc, ie, je, (int)(171 * E + packed(ie, je, 6) * T + e));
    }
    for (long e = 0; e < F; ++e) {
        const long *mc = &m.fr_mc[e * 14];
        for (int je = 0; je < 14; ++je)
            for (int ie = 0; ie <= je; ++ie)
                add(mc, ie, je, (int)(171 * E + 21 * T + packed(ie, je, 14) * F + e));
    }
    // shells, the bulk: contiguous element ranges on host threads, each into
    // its own list, appended in range order (the same order as one loop)
    auto shells = [&](long e0, long e1, std::vector<TangentPair> &out) {
        for (long e = e0; e < e1; ++e) {
            long mc[18];
            for (int a = 0; a < 3; ++a)
                for (int d = 0; d < 6; ++d) mc[a * 6 + d] = m.jcode[m.sh_conn[e * 3 + a] * 7 + d];
            for (int je = 0; je < 18; ++je)
                for (int ie = 0; ie <= je; ++ie) {
                    if (!mc[ie] || !mc[je]) continue;
                    out.push_back({std::max(mc[ie], mc[je]) - 1, std::min(mc[ie], mc[je]) - 1,
                                   (int)(packed(ie, je, 18) * E + e)});
                }
        }
    };
    const unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (E < 4096 || nthreads == 1) {
        shells(0, E, all);
        return;
    }
    std::vector<std::vector<TangentPair>> parts(nthreads);
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t] {
            const long e0 = E * (long)t / nthreads, e1 = E * (long)(t + 1) / nthreads;
            parts[t].reserve((size_t)(171 * (e1 - e0)));
            shells(e0, e1, parts[t]);
        });
    for (std::thread &th : pool) th.join();
    for (const auto &part : parts) all.insert(all.end(), part.begin(), part.end());
}

// Groups contributions by key (stable, so each list keeps the order above).
// Large maps are split by key range into one bucket per host thread (a
// stable scatter, so equal keys keep their order), and the buckets are
// sorted in parallel; their concatenation is the sequential stable sort.
template <typename Key>
void group_pairs(std::vector<TangentPair> &all, Key key, GatherMap &g, std::vector<int64_t> &keys)
{
    auto less = [&](const TangentPair &a, const TangentPair &b) { return key(a) < key(b); };
    const size_t n = all.size();
    const unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < (size_t)1 << 16 || nthreads == 1) {
        std::stable_sort(all.begin(), all.end(), less);
    } else {
        int64_t kmax = 0;
        for (const TangentPair &p : all) kmax = std::max(kmax, key(p));
        const unsigned nb = nthreads;
        auto bucket = [&](const TangentPair &p) {  // non-decreasing in the key
            const unsigned b = (unsigned)((double)key(p) / ((double)kmax + 1.0) * nb);
            return std::min(b, nb - 1);
        };
        std::vector<size_t> start(nb + 1, 0);
        for (const TangentPair &p : all) ++start[bucket(p) + 1];
        for (unsigned b = 0; b < nb; ++b) start[b + 1] += start[b];
        std::vector<TangentPair> out(n);
        std::vector<size_t> pos(start.begin(), start.end() - 1);
        for (const TangentPair &p : all) out[pos[bucket(p)]++] = p;
        std::vector<std::thread> pool;
        for (unsigned b = 0; b < nb; ++b)
            pool.emplace_back([&, b] { std::stable_sort(out.begin() + start[b], out.begin() + start[b + 1], less); });
        for (std::thread &t : pool) t.join();
        all.swap(out);
    }
    g.ptr.clear();
    g.src.clear();
    keys.clear();
    g.ptr.push_back(0);
    for (size_t k = 0; k < all.size(); ++k) {
        if (k == 0 || key(all[k]) != key(all[k - 1])) {
            if (k) g.ptr.push_back((int)g.src.size());
            keys.push_back(key(all[k]));
        }
        g.src.push_back(all[k].src);
    }
    g.ptr.push_back((int)g.src.size());
}
}  // namespace

// Band map: one list per lower-band slot L[col*ld + (row-col)].
void build_tangent_map(const HostModel &m, long ld, GatherMap &g)
{
    std::vector<TangentPair> all;
    collect_tangent_pairs(m, all);
    group_pairs(all, [ld](const TangentPair &p) { return (int64_t)p.c * ld + (p.r - p.c); }, g, g.dst);
}

// CSR map: one list per lower pair (r >= c), written to the CSR slot of
// (r, c) (dst) and of its mirror (c, r) (dst2, -1 on the diagonal). The
// pattern holds both triangles, columns ascending in each row.
void build_csr_tangent(const HostModel &m, CsrPattern &p, GatherMap &g, std::vector<int64_t> &dst2)
{
    const long n = m.neq;
    std::vector<TangentPair> all;
    collect_tangent_pairs(m, all);
    std::vector<int64_t> keys;
    group_pairs(all, [n](const TangentPair &q) { return (int64_t)q.r * n + q.c; }, g, keys);
    // row lists: lower columns from the pairs, upper columns from the mirrors
    std::vector<std::vector<int>> cols(n);
    for (int64_t k : keys) {
        long r = (long)(k / n), c = (long)(k % n);
        cols[r].push_back((int)c);
        if (r != c) cols[c].push_back((int)r);
    }
    p.rowptr.assign(n + 1, 0);
    p.col.clear();
    p.diag.assign(n, -1);
    for (long i = 0; i < n; ++i) {
        std::sort(cols[i].begin(), cols[i].end());
        for (int c : cols[i]) {
            if (c == i) p.diag[i] = (int)p.col.size();
            p.col.push_back(c);
        }
        p.rowptr[i + 1] = (int)p.col.size();
    }
    auto slot = [&](long r, long c) -> int64_t {
        auto b = p.col.begin() + p.rowptr[r], e = p.col.begin() + p.rowptr[r + 1];
        return (int64_t)(std::lower_bound(b, e, (int)c) - p.col.begin());
    };
    g.dst.resize(keys.size());
    dst2.resize(keys.size());
    for (size_t k = 0; k < keys.size(); ++k) {
        long r = (long)(keys[k] / n), c = (long)(keys[k] % n);
        g.dst[k] = slot(r, c);
        dst2[k] = r == c ? -1 : slot(c, r);
    }
}

// Nodal blocks of consecutive equations for block-Jacobi: the equations of
// one joint (jcode, at most 7) form a block; an equation no joint owns (a
// member-end warping DOF) is a block of its own.
void build_node_blocks(const HostModel &m, std::vector<int> &start)
{
    std::vector<long> owner(m.neq, -1);
    for (long i = 0; i < m.nj; ++i)
        for (int d = 0; d < 7; ++d)
            if (m.jcode[i * 7 + d] > 0) owner[m.jcode[i * 7 + d] - 1] = i;
    start.clear();
    for (long q = 0; q < m.neq; ++q) {
        bool fresh = q == 0 || owner[q] < 0 || owner[q] != owner[q - 1] || q - start.back() >= 8;
        if (fresh) start.push_back((int)q);
    }
    start.push_back((int)m.neq);
}

}  // namespace cb
