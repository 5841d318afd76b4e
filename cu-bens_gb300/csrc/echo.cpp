// results1.txt: the input echo the reference writes while it reads the
// model_def, and its C entry point.
//
// The sections come in the reference's order: analysis and algorithm type
// and the control variables (main.c:383-433), member incidences and joint
// constraints (struc, model.c:314-391), the number of equations (main.c:1035)
// and the skyline length (main.c:1357), joint coordinates and degrees of
// freedom (main.c:1392-1414), element properties (prop_tr truss.c:48-70,
// prop_fr frame.c:54-181, prop_sh shell.c:51-100), the static joint loads
// (load, model.c:1316-1319) and the arc-length's initially prescribed
// displacement (arc.c:52-53). The formats are the reference's printf
// formats; the derived values (element lengths, shell areas) are formed the
// way its prop_* routines form them.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "cubens_gb300.h"
#include "internal.hpp"

namespace cb {

namespace {

void put(std::string &s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    const int k = std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (k < 0) return;
    if ((size_t)k < sizeof buf) {
        s.append(buf, (size_t)k);
        return;
    }
    std::string big((size_t)k + 1, '\0');
    va_start(ap, fmt);
    std::vsnprintf(&big[0], big.size(), fmt, ap);
    va_end(ap);
    s.append(big.data(), (size_t)k);
}

double norm3(const double *a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

}  // namespace

std::string input_echo(const HostModel &m)
{
    std::string s;
    s.reserve(256 + 64 * (size_t)(m.nj * 3 + m.ne_tr + m.ne_fr + m.ne_sh));
    const int ana = m.echo.ana, alg = m.alg;
    if (alg < 4) {
        if (ana == 2) put(s, "Analysis Type:\n\t2nd Order Elastic\n");
        else if (ana == 3) put(s, "Analysis Type:\n\t2nd Order Inelastic\n");
    } else if (ana == 1 && alg == 4) {
        put(s, "Analysis Type:\n\t1st Order Elastic Dynamic\n");
    } else if (ana == 2 && alg == 5) {
        put(s, "Analysis Type:\n\t2nd Order Elastic Dynamic\n");
    } else if (ana == 3 && alg == 5) {
        put(s, "Analysis Type:\n\t2nd Order Inelastic Dynamic\n");
    }
    static const char *const algs[] = {"Direct Stiffness", "Newton Raphson", "Modified Newton Raphson",
                                       "Modified Spherical Arc Length", "Dynamic (Newmark)",
                                       "Dynamic (Newmark)"};
    if (alg >= 0 && alg <= 5) put(s, "\nAlgorithm Type:\n\t%s\n", algs[alg]);
    put(s, "\nControl Variables:\n\tNumber of Joints: %ld\n", m.nj);
    put(s, "\tNumber of Truss Elements: %ld\n", m.ne_tr);
    put(s, "\tNumber of Frame Elements: %ld\n", m.ne_fr);
    put(s, "\tNumber of Shell Elements: %ld\n", m.ne_sh);
    put(s, "\tNumber of Solid Brick Elements: %ld\n", 0L);
    put(s, "\tNumber of Fluid Brick Elements: %ld\n", 0L);

    // incidences (1-based joints)
    if (m.ne_tr > 0) {
        put(s, "\nTruss Member Incidences:\n\tMember\t\tEnd-1\t\tEnd-2\n");
        for (long i = 0; i < m.ne_tr; ++i)
            put(s, "\t%ld\t\t%ld\t\t%ld\n", i + 1, (long)m.tr_conn[2 * i] + 1, (long)m.tr_conn[2 * i + 1] + 1);
    }
    if (m.ne_fr > 0) {
        put(s, "\nFrame Member Incidences:\n\tMember\t\tEnd-1\t\tEnd-2\n");
        for (long i = 0; i < m.ne_fr; ++i)
            put(s, "\t%ld\t\t%ld\t\t%ld\n", i + 1, (long)m.fr_conn[2 * i] + 1, (long)m.fr_conn[2 * i + 1] + 1);
    }
    if (m.ne_sh > 0) {
        put(s, "\nShell Member Incidences:\n\tElement\t\tVertex-1\tVertex-2\tVertex-3\n");
        for (long i = 0; i < m.ne_sh; ++i)
            put(s, "\t%ld\t\t%ld\t\t%ld\t\t%ld\n", i + 1, (long)m.sh_conn[3 * i] + 1, (long)m.sh_conn[3 * i + 1] + 1,
                (long)m.sh_conn[3 * i + 2] + 1);
    }
    // constraints: every fixed DOF after the element-type pass, before the
    // equation numbering (a fixed DOF is the one without an equation)
    put(s, "\nJoint Constraints:\n\tJoint\t\tDirection\tWarping (optional)\n");
    for (long i = 0; i < m.nj; ++i) {
        for (int j = 0; j < 6; ++j)
            if (m.jcode[i * 7 + j] == 0) put(s, "\t%ld\t\t%ld\n", i + 1, (long)j + 1);
        // "j,7,1" (one warping DOF per member end) is a constraint line too,
        // though the numbering gives that joint's ends their own equations
        const int w = m.echo.wrp.empty() ? 0 : m.echo.wrp[i];
        if (m.jcode[i * 7 + 6] == 0 || w == 1) put(s, "\t%ld\t\t%ld\t\t%d\n", i + 1, 7L, w);
    }
    put(s, "\nNumber of equations (system DOFs): %ld\n", m.neq);
    put(s, "\nLength of stiffness array: %ld\n", m.lss);
    put(s, "\nJoint Coordinates:\n\tJoint\t\tDirection-1\tDirection-2\tDirection-3\n");
    for (long i = 0; i < m.nj; ++i)
        put(s, "\t%d\t\t%lf\t%lf\t%lf\n", (int)(i + 1), m.x0[i * 3], m.x0[i * 3 + 1], m.x0[i * 3 + 2]);
    put(s, "\nJoint Degrees of Freedom:\n\tJoint\t\tX-Translation\tY-Translation\tZ-Translation\tX-Rotation\t"
           "Y-Rotation\tZ-Rotation\tWarping\n");
    for (long i = 0; i < m.nj; ++i) {
        put(s, "\t%d\t\t", (int)(i + 1));
        for (int j = 0; j < 7; ++j) put(s, "%ld\t\t", m.jcode[i * 7 + j]);
        put(s, "\n");
    }

    const double *x = m.x0.data();
    if (m.ne_tr > 0) {
        put(s, "\nTruss Element Properties:\n\tElement\t\tModulus\t\tArea\t\tDensity\t\tLength\t\tYield Stress\n");
        for (long i = 0; i < m.ne_tr; ++i) {
            const int j = m.tr_conn[2 * i], k = m.tr_conn[2 * i + 1];
            const double el[3] = {x[k * 3] - x[j * 3], x[k * 3 + 1] - x[j * 3 + 1], x[k * 3 + 2] - x[j * 3 + 2]};
            put(s, "\t%ld\t\t%lf\t%lf\t%lf\t%lf\t%lf\n", i + 1, m.tr_e[i], m.tr_a[i], m.echo.tr_dens[i], norm3(el),
                m.echo.tr_yield[i]);
        }
    }
    if (m.ne_fr > 0) {
        put(s, "\nFrame Element Properties:\n\tElement\t\tElastic Modulus\t\tShear Modulus\t\tArea\t\t"
               "___________________________Moments of Inertia__________________________\n\t\t\t\t\t\t\t\t\t\t\t"
               "Strong-Axis Bending\tWeak-Axis Bending\tPolar\t\tWarping\n");
        for (long i = 0; i < m.ne_fr; ++i) {
            const double *p = &m.fr_prop[8 * i];  // E, G, rho, A, I strong, I weak, J, I warping
            put(s, "\t%ld\t\t%lf\t\t%lf\t\t%lf\t%lf\t\t%lf\t\t%lf\t%lf\n", i + 1, p[0], p[1], p[3], p[4], p[5], p[6],
                p[7]);
        }
        put(s, "\nFrame Element Orientation:\n\tElement\t\tLength\t\t______________Auxiliary Points_____________"
               "\n\t\t\t\t\tDirection-1\tDirection-2\tDirection-3\n");
        for (long i = 0; i < m.ne_fr; ++i) {
            const int j = m.fr_conn[2 * i], k = m.fr_conn[2 * i + 1];
            const double el[3] = {x[k * 3] - x[j * 3], x[k * 3 + 1] - x[j * 3 + 1], x[k * 3 + 2] - x[j * 3 + 2]};
            put(s, "\t%ld\t\t%lf\t%lf\t%lf\t%lf\n", i + 1, norm3(el), m.fr_aux[3 * i], m.fr_aux[3 * i + 1],
                m.fr_aux[3 * i + 2]);
        }
        put(s, "\nFrame Element Yield Criteria:\n\tElement\t\tYield Stress\t\t_____Plastic Section Moduli______"
               "\n\t\t\t\t\t\tStrong-Axis\t\tWeak-Axis\n");
        for (long i = 0; i < m.ne_fr; ++i)
            put(s, "\t%ld\t\t%lf\t\t%lf\t\t%lf\n", i + 1, m.echo.fr_yield[3 * i], m.echo.fr_yield[3 * i + 1],
                m.echo.fr_yield[3 * i + 2]);
    }
    if (m.ne_sh > 0) {
        put(s, "\nShell Element Properties:\n\tElement\t\tElastic Modulus\t\tPoisson's Ratio\t\tThickness\tDensity\t\t"
               "Area\t\tLength-12\tLength-23\tLength-31\tYield Stress\n");
        for (long i = 0; i < m.ne_sh; ++i) {
            const int j = m.sh_conn[3 * i], k = m.sh_conn[3 * i + 1], l = m.sh_conn[3 * i + 2];
            double e12[3], e23[3], e31[3];
            for (int a = 0; a < 3; ++a) {
                e23[a] = x[l * 3 + a] - x[k * 3 + a];
                e31[a] = x[l * 3 + a] - x[j * 3 + a];
                e12[a] = x[k * 3 + a] - x[j * 3 + a];
            }
            // face area from the normal e12 x e31
            const double nrm[3] = {e12[1] * e31[2] - e12[2] * e31[1], e12[2] * e31[0] - e12[0] * e31[2],
                                   e12[0] * e31[1] - e12[1] * e31[0]};
            const double area = 0.5 * norm3(nrm);
            put(s, "\t%ld\t\t%lf\t\t%lf\t%lf\t%lf\t%lf\t%lf\t%lf\t%lf\t%lf\n", i + 1, m.sh_e[i], m.sh_nu[i], m.sh_t[i],
                m.echo.sh_dens[i], area, norm3(e12), norm3(e23), norm3(e31), m.echo.sh_yield[i]);
        }
    }
    if (m.alg < 4 && !m.echo.load_jt.empty()) {
        put(s, "\nJoint Loads:\n\tGlobal Joint\tDirection\tForce\n");
        for (size_t i = 0; i < m.echo.load_jt.size(); ++i)
            put(s, "\t%ld\t\t%d\t\t%lf\n", m.echo.load_jt[i], m.echo.load_dir[i], m.echo.load_mag[i]);
    }
    if (m.alg == 3)
        put(s, "\nInitial Prescribed Displacement:\n\tGlobal Joint\tDirection\tDisplacement\n\t%ld\t\t%d\t\t%f\n",
            m.echo.dk_jt, m.echo.dk_dir, m.dk);
    return s;
}

}  // namespace cb

extern "C" int cb_input_echo(const char *text, size_t len, char *buf, size_t cap, size_t *needed)
{
    if (!text) return CB_ERR_ARG;
    cb::HostModel h;
    int status = CB_ERR_PARSE;
    const std::string err = cb::parse_model_def(text, len, h, status);
    if (!err.empty()) return status == CB_OK ? CB_ERR_PARSE : status;
    const std::string s = cb::input_echo(h);
    if (needed) *needed = s.size();
    if (buf && cap > 0) {
        const size_t n = std::min(cap - 1, s.size());
        std::memcpy(buf, s.data(), n);
        buf[n] = '\0';
    }
    return CB_OK;
}
