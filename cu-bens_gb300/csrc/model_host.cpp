// model_def reader, equation numbering, skyline profile and the gather maps
// that drive the deterministic (atomics-free) assembly on the GPU.
//
// Reading order follows main.c:340-433 (header), struc model.c:95-264
// (incidences, constraints), main.c:1395 (coordinates), prop_tr truss.c:66,
// prop_sh shell.c:61 (properties), load model.c:1313-1335 (joint loads) and
// msal arc.c:48 / main.c:2240-2245 (MSAL controls).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>

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
    if (ana != 2) {
        status = CB_ERR_UNSUPPORTED;
        return "only ANAFLAG 2 (second-order elastic) is on the GPU path";
    }
    if (alg != 3) {
        status = CB_ERR_UNSUPPORTED;
        return "only ALGFLAG 3 (modified spherical arc length) is on the GPU path";
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
    if (m.ne_fr || nsbr || nfbr) {
        status = CB_ERR_UNSUPPORTED;
        return "frame and brick elements are not on the GPU MSAL path";
    }
    const long NJ = m.nj;
    std::vector<char> has_tr(NJ, 0), has_sh(NJ, 0);
    m.tr_conn.resize(2 * m.ne_tr);
    for (long i = 0; i < 2 * m.ne_tr; ++i) {
        long j = (long)t.next() - 1;
        if (j < 0 || j >= NJ) return "truss incidence out of range";
        m.tr_conn[i] = (int)j;
        has_tr[j] = 1;
    }
    m.sh_conn.resize(3 * m.ne_sh);
    for (long i = 0; i < 3 * m.ne_sh; ++i) {
        long j = (long)t.next() - 1;
        if (j < 0 || j >= NJ) return "shell incidence out of range";
        m.sh_conn[i] = (int)j;
        has_sh[j] = 1;
    }
    m.jcode.assign(NJ * 7, -1);
    for (;;) {
        long j = (long)t.next(), k = (long)t.next();
        if (!t.ok) return "constraint list not terminated";
        if (j == 0) break;
        if (j < 0 || j > NJ || k < 1 || k > 7) return "joint constraint input not recognized";
        if (k == 7) (void)t.next();
        m.jcode[(j - 1) * 7 + k - 1] = 0;
    }
    // DOFs no element type uses (model.c:267-285): truss joints keep 1-3,
    // shell joints keep 1-6, warping is fixed without frames.
    for (long i = 0; i < NJ; ++i) {
        if (!has_sh[i]) {
            int from = has_tr[i] ? 3 : 0;
            for (int j = from; j < 7; ++j) m.jcode[i * 7 + j] = 0;
        } else {
            m.jcode[i * 7 + 6] = 0;
        }
    }
    long neq = 0;
    for (long i = 0; i < NJ * 7; ++i)
        if (m.jcode[i] != 0) m.jcode[i] = ++neq;
    m.neq = neq;
    if (neq == 0) return "no free degrees of freedom";
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
    for (long i = 0; i < m.ne_tr; ++i) {
        m.tr_e[i] = t.next();
        m.tr_a[i] = t.next();
        (void)t.next();  // density
        (void)t.next();  // yield stress (ANAFLAG 3 only)
    }
    m.sh_e.resize(m.ne_sh);
    m.sh_nu.resize(m.ne_sh);
    m.sh_t.resize(m.ne_sh);
    for (long i = 0; i < m.ne_sh; ++i) {
        m.sh_e[i] = t.next();
        m.sh_nu[i] = t.next();
        m.sh_t[i] = t.next();
        (void)t.next();
        (void)t.next();
    }
    if (!t.ok) return "model_def ended inside the properties";
    m.q.assign(neq, 0.0);
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
    }
    if (!any_load) return "no forces present in input file";
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
    m.dkdof = m.jcode[(jt - 1) * 7 + dir - 1] - 1;
    if (m.dkdof < 0) return "initially prescribed displacement at fixed degree of freedom";
    status = CB_OK;
    return "";
}

// Force map. The reference accumulates forces_tr before forces_sh, elements
// in order, so every equation's list is sorted by (type, element). The
// contribution buffer holds the shell element forces at [k*E + e] (k < 18),
// followed by the truss forces at 18E + [k*T + e] (k < 6).
void build_force_map(const HostModel &m, GatherMap &g)
{
    const long E = m.ne_sh, T = m.ne_tr;
    std::vector<std::vector<int>> lists(m.neq);
    for (long e = 0; e < T; ++e)
        for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 3; ++d) {
                long q = m.jcode[m.tr_conn[e * 2 + a] * 7 + d];
                if (q) lists[q - 1].push_back((int)(18 * E + (a * 3 + d) * T + e));
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

// Tangent map. Element matrices are packed upper triangles, shells at
// [p*E + e] (p < 171), trusses at 171E + [p*T + e] (p < 21). For a local pair
// (ie <= je) the global slot is (max(i,j), min(i,j)) of the lower band,
// L[col*ld + (row-col)], and the value used is K[ie][je], as the reference
// adds K[ie][je] for ie <= je into its skyline (truss.c:170-193,
// shell.c:307-329). Lists are sorted by (slot, truss before shell, element).
void build_tangent_map(const HostModel &m, long ld, GatherMap &g)
{
    const long E = m.ne_sh, T = m.ne_tr;
    struct C {
        int64_t slot;
        int src;
    };
    std::vector<C> all;
    all.reserve((size_t)(171 * E + 21 * T));
    for (long e = 0; e < T; ++e) {
        long mc[6];
        for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 3; ++d) mc[a * 3 + d] = m.jcode[m.tr_conn[e * 2 + a] * 7 + d];
        for (int je = 0; je < 6; ++je)
            for (int ie = 0; ie <= je; ++ie) {
                if (!mc[ie] || !mc[je]) continue;
                long r = std::max(mc[ie], mc[je]) - 1, c = std::min(mc[ie], mc[je]) - 1;
                all.push_back({(int64_t)c * ld + (r - c), (int)(171 * E + packed(ie, je, 6) * T + e)});
            }
    }
    for (long e = 0; e < E; ++e) {
        long mc[18];
        for (int a = 0; a < 3; ++a)
            for (int d = 0; d < 6; ++d) mc[a * 6 + d] = m.jcode[m.sh_conn[e * 3 + a] * 7 + d];
        for (int je = 0; je < 18; ++je)
            for (int ie = 0; ie <= je; ++ie) {
                if (!mc[ie] || !mc[je]) continue;
                long r = std::max(mc[ie], mc[je]) - 1, c = std::min(mc[ie], mc[je]) - 1;
                all.push_back({(int64_t)c * ld + (r - c), (int)(packed(ie, je, 18) * E + e)});
            }
    }
    // stable sort keeps (truss, then shell; element order) within a slot
    std::stable_sort(all.begin(), all.end(), [](const C &a, const C &b) { return a.slot < b.slot; });
    g.ptr.clear();
    g.src.clear();
    g.dst.clear();
    g.ptr.push_back(0);
    for (size_t k = 0; k < all.size(); ++k) {
        if (k == 0 || all[k].slot != all[k - 1].slot) {
            if (k) g.ptr.push_back((int)g.src.size());
            g.dst.push_back(all[k].slot);
        }
        g.src.push_back(all[k].src);
    }
    g.ptr.push_back((int)g.src.size());
}

}  // namespace cb
