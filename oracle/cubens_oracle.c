/* CPU oracle for the CU-BENs nonlinear equilibrium-loop hot path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference's FP64
 * algorithms, used by the parity tests as the checker and by bench.py as the
 * CPU baseline. Each routine names the reference file:line it restates. The
 * restatement keeps the reference's arithmetic (including its quirks: the
 * drilling stiffness /1e4, the zeroed membrane part of the previous element
 * force, the root rule of quad, the three criteria of test) but is organised
 * around the 3x3 block structure of the element transformations.
 */
#define _POSIX_C_SOURCE 199309L
#include "cubens_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now_s(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* ------------------------------------------------------------------------ */
/* Model                                                                     */
/* ------------------------------------------------------------------------ */

struct orc_model {
    long nj, ne_tr, ne_fr, ne_sh, neq, lss;
    long *jcode;     /* NJ*7, 1-based equation numbers, 0 = fixed (model.c:937-961) */
    long *maxa;      /* NEQ+1, 1-based diagonal addresses (model.c:1264-1270) */
    double *x0;      /* NJ*3 initial coordinates */
    double *q;       /* NEQ reference load (model.c:1313-1335) */
    /* truss */
    long *tr_conn;   /* NE_TR*2 (0-based joints) */
    double *tr_e, *tr_a, *tr_len0, *tr_dir0; /* dir0: NE_TR*3 */
    /* shell */
    long *sh_conn;   /* NE_SH*3 (0-based joints) */
    double *sh_e, *sh_nu, *sh_t, *sh_dens;
    double *sh_xl;   /* NE_SH*3 local x2, x3, y3 of the initial geometry */
    double *sh_area0;
    double *sh_slen0; /* NE_SH*3 initial side lengths l12, l23, l31 */
    double *sh_c0;   /* NE_SH*9 initial triads (rows c1, c2, c3) */
    double *sh_kem;  /* NE_SH*36 membrane stiffness (stiffe_m_sh) */
    double *sh_keb;  /* NE_SH*81 plate bending stiffness (stiffe_b_sh) */
    /* frame (14 DOF: 7 per end incl. warping) */
    long *fr_conn;   /* NE_FR*2 (0-based joints) */
    double *fr_e, *fr_g, *fr_dens, *fr_a, *fr_iz, *fr_iy, *fr_ip, *fr_iw; /* iz strong, iy weak */
    double *fr_aux;  /* NE_FR*3 auxiliary points */
    double *fr_len0; /* NE_FR initial lengths */
    double *fr_c0;   /* NE_FR*9 initial triads */
    long *fr_mc;     /* NE_FR*14 1-based equation numbers (0 = fixed), warping numbered per member */
    int alg;         /* ALGFLAG: 3 (MSAL) or 5 (nonlinear Newmark) */
    /* MSAL controls (main.c:2240-2245, arc.c:48) */
    long dkdof;      /* 0-based */
    double dk, alpha, psi_thresh, lpfmax, dkimax, toldisp, tolforc, tolener;
    int iteopt, itemax, submax, imagmax, negmax;
    /* nonlinear Newmark input (main.c:3320-3326, model.c:1492-1609) */
    long ntin;       /* input time points (ntsteps + 1) */
    long nsteps;     /* NTSTPS = (long)(ttot/dt + 1) */
    double dt, ttot, numopt, spectrds, lpf0, dlpf0, dlpfmax, dlpfmin;
    int solmin;
    double *pinpt;   /* NEQ*ntin per-step joint forces */
    double *um0, *vm0, *am0; /* linear Newmark (ALGFLAG 4): NEQ initial displacements, velocities,
                                accelerations (load, model.c:1583-1604) */
};

/* ---- token reader: the model_def layout is positional numbers ---- */
typedef struct {
    const char *p;
    int ok;
} tok_t;

static double tok_num(tok_t *t)
{
    while (*t->p && (*t->p == ',' || *t->p == ' ' || *t->p == '\t' || *t->p == '\n' ||
                     *t->p == '\r'))
        t->p++;
    if (!*t->p) {
        t->ok = 0;
        return 0;
    }
    char *end;
    double v = strtod(t->p, &end);
    if (end == t->p) {
        t->ok = 0;
        return 0;
    }
    t->p = end;
    return v;
}

static void set_err(char *err, int errlen, const char *msg)
{
    if (err && errlen > 0) {
        strncpy(err, msg, (size_t)errlen - 1);
        err[errlen - 1] = 0;
    }
}

static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* cross product with optional normalisation (misc.c:264-282) */
static void cross3(const double *a, const double *b, double *c, int normalise)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
    if (normalise) {
        double l = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        c[0] /= l;
        c[1] /= l;
        c[2] /= l;
    }
}

static double vdot(long n, const double *a, const double *b)
{
    double s = 0;
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* Shell geometry from three vertex positions, as prop_sh (shell.c:61-91) and
 * updatc (misc.c:149-184) compute it: side lengths, face area and the triad
 * x^ = e12/|e12|, z^ = n/|n|, y^ = z^ x x^ (rows c1, c2, c3 of c). */
static void shell_geometry(const double *p1, const double *p2, const double *p3, double *c,
                           double *area, double *slen)
{
    double e12[3], e23[3], e31[3], nrm[3], lx[3], lz[3], ly[3];
    for (int m = 0; m < 3; ++m) {
        e23[m] = p3[m] - p2[m];
        e31[m] = p3[m] - p1[m];
        e12[m] = p2[m] - p1[m];
    }
    double l23 = sqrt(dot3(e23, e23));
    double l31 = sqrt(dot3(e31, e31));
    double l12 = sqrt(dot3(e12, e12));
    if (slen) {
        slen[0] = l12;
        slen[1] = l23;
        slen[2] = l31;
    }
    cross3(e12, e31, nrm, 0);
    double a = 0.5 * sqrt(dot3(nrm, nrm));
    *area = a;
    for (int m = 0; m < 3; ++m) {
        lx[m] = e12[m] / l12;
        lz[m] = nrm[m] / (2 * a);
    }
    cross3(lz, lx, ly, 1);
    for (int m = 0; m < 3; ++m) {
        c[m] = lx[m];
        c[3 + m] = ly[m];
        c[6 + m] = lz[m];
    }
}

/* Local membrane coordinates (mem_coord, shell.c:2402-2446): vertex 1 at the
 * origin, xl = (x2, x3, y3) = (c1.(p2-p1), c1.(p3-p1), c2.(p3-p1)). */
static void shell_local(const double *p1, const double *p2, const double *p3, const double *c,
                        double *xl)
{
    double X2[3], X3[3];
    for (int m = 0; m < 3; ++m) {
        X2[m] = p2[m] - p1[m];
        X3[m] = p3[m] - p1[m];
    }
    /* the reference sums sum_l T[j][l]*X[l][k] including the zero column of X */
    xl[0] = c[0] * X2[0] + c[1] * X2[1] + c[2] * X2[2];
    xl[1] = c[0] * X3[0] + c[1] * X3[1] + c[2] * X3[2];
    xl[2] = c[3] * X3[0] + c[4] * X3[1] + c[5] * X3[2];
}

/* Plane-stress matrix and membrane B of the constant-strain triangle
 * (stiffe_m_sh, shell.c:487-531; stiffg_sh, shell.c:660-686). */
static void plane_stress(double e, double nu, double C[3][3])
{
    double f = e / (1 - pow(nu, 2));
    C[0][2] = C[1][2] = C[2][0] = C[2][1] = 0;
    C[0][0] = C[1][1] = f;
    C[0][1] = C[1][0] = f * nu;
    C[2][2] = f * (1 - nu) / 2;
}

static void membrane_b(const double *xl, double area, double B[3][6])
{
    double x2 = xl[0], x3 = xl[1], y3 = xl[2];
    double a2 = 2 * area;
    memset(B, 0, sizeof(double) * 18);
    B[0][0] = B[2][1] = -(y3 / a2);
    B[0][2] = B[2][3] = y3 / a2;
    B[1][1] = B[2][0] = (x3 - x2) / a2;
    B[1][3] = B[2][2] = -(x3 / a2);
    B[1][5] = B[2][4] = x2 / a2;
}

/* Membrane stiffness t*A*B^T C B (stiffe_m_sh, shell.c:487-531). */
static void shell_kem(double e, double nu, double t, double area, const double *xl, double *kem)
{
    double C[3][3], B[3][6], BC[6][3];
    plane_stress(e, nu, C);
    membrane_b(xl, area, B);
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += B[k][i] * C[k][j];
            BC[i][j] = s;
        }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += BC[i][k] * B[k][j];
            kem[i * 6 + j] = t * area * s;
        }
}

/* Explicit DKT plate-bending stiffness of Batoz (1982), as stiffe_b_sh
 * evaluates it (shell.c:533-658): ke_b = Q alpha^T / (2A) with the transposed
 * 9x9 "alpha" matrix written in terms of the local coordinates and the
 * Batoz coefficients p4..p6, t4, t5, q4, q5, r4, r5. */
static void shell_keb(double e, double nu, double t, double area, const double *xl,
                      const double *slen, double *keb)
{
    double x2 = xl[0], x3 = xl[1], y3 = xl[2];
    double D = e * pow(t, 3) / (12 * (1 - pow(nu, 2)));
    double E1 = D, E3 = D, E2 = D * nu, E4 = D * (1 - nu) / 2;
    double x23 = x2 - x3;
    double L12 = pow(slen[0], 2), L23 = pow(slen[1], 2), L31 = pow(slen[2], 2);
    double p4 = -6 * x23 / L23, p5 = -6 * x3 / L31, p6 = 6 * x2 / L12;
    double t4 = 6 * y3 / L23, t5 = -6 * y3 / L31;
    double q4 = -3 * x23 * y3 / L23, q5 = 3 * x3 * y3 / L31;
    double r4 = 3 * pow(y3, 2) / L23, r5 = 3 * pow(y3, 2) / L31;
    /* row k of aT holds column k of Batoz's alpha matrix */
    double aT[9][9] = {
        {y3 * p6, -(y3 * p6), y3 * p5, -(x2 * t5), 0, x23 * t5, -(x3 * p6) - x2 * p5, -x23 * p6,
         x23 * p5 + y3 * t5},
        {0, 0, -(y3 * q5), x23 + x2 * r5, x23, x23 * (1 - r5), x2 * q5 + y3, y3,
         -x23 * q5 + y3 * (1 - r5)},
        {-4 * y3, 2 * y3, y3 * (2 - r5), -(x2 * q5), 0, x23 * q5, -4 * x23 + x2 * r5, 2 * x23,
         x23 * (2 - r5) + y3 * q5},
        {-(y3 * p6), y3 * p6, y3 * p4, 0, x2 * t4, -(x3 * t4), x3 * p6, x23 * p6 + x2 * p4,
         -(x3 * p4) + y3 * t4},
        {0, 0, y3 * q4, x3, x3 + x2 * r4, x3 * (1 - r4), -y3, -y3 + x2 * q4,
         y3 * (r4 - 1) - x3 * q4},
        {-2 * y3, 4 * y3, y3 * (r4 - 2), 0, -(x2 * q4), x3 * q4, 2 * x3, -4 * x3 + x2 * r4,
         x3 * (2 - r4) - y3 * q4},
        {0, 0, -(y3 * (p4 + p5)), x2 * t5, -(x2 * t4), -x23 * t5 + x3 * t4, x2 * p5, -(x2 * p4),
         -x23 * p5 + x3 * p4 - y3 * (t4 + t5)},
        {0, 0, y3 * (q4 - q5), x2 * (r5 - 1), x2 * (r4 - 1), -x23 * r5 - x3 * r4 - x2, x2 * q5,
         x2 * q4, -x23 * q5 - x3 * q4 + y3 * (r4 - r5)},
        {0, 0, y3 * (r4 - r5), -(x2 * q5), -(x2 * q4), x3 * q4 + x23 * q5, x2 * (r5 - 2),
         x2 * (r4 - 2), -x23 * r5 - x3 * r4 + 4 * x2 + y3 * (q5 - q4)}};
    /* Q = (block-wise) D-weighted alpha^T with the 1/24 integration weights */
    double Q[9][9];
    for (int g = 0; g < 3; ++g) {
        int o = 3 * g;
        for (int i = o; i < o + 3; ++i) {
            double b1 = 0, b2 = 0, b3 = 0;
            for (int j = 0; j < 3; ++j) {
                b1 += E1 * aT[i][j] + E2 * aT[i][j + 3];
                b2 += E2 * aT[i][j] + E3 * aT[i][j + 3];
                b3 += E4 * aT[i][j + 6];
            }
            for (int j = 0; j < 3; ++j) {
                Q[i][j] = (E1 * aT[i][j] + E2 * aT[i][j + 3] + b1) / 24;
                Q[i][j + 3] = (E2 * aT[i][j] + E3 * aT[i][j + 3] + b2) / 24;
                Q[i][j + 6] = (E4 * aT[i][j + 6] + b3) / 24;
            }
        }
    }
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) {
            double s = 0;
            for (int k = 0; k < 9; ++k) s += Q[i][k] * aT[j][k];
            keb[i * 9 + j] = s / (2 * area);
        }
}

/* The loop above reproduces the three row groups of stiffe_b_sh
 * (shell.c:609-650): for row group g the columns j, j+3 and j+6 of aT are read
 * at offsets relative to the group (g*3). */

void orc_free(orc_model *m)
{
    if (!m) return;
    free(m->jcode);
    free(m->maxa);
    free(m->x0);
    free(m->q);
    free(m->tr_conn);
    free(m->tr_e);
    free(m->tr_a);
    free(m->tr_len0);
    free(m->tr_dir0);
    free(m->sh_conn);
    free(m->sh_e);
    free(m->sh_nu);
    free(m->sh_t);
    free(m->sh_xl);
    free(m->sh_area0);
    free(m->sh_dens);
    free(m->sh_slen0);
    free(m->sh_c0);
    free(m->sh_kem);
    free(m->sh_keb);
    free(m->fr_conn);
    free(m->fr_e);
    free(m->fr_g);
    free(m->fr_dens);
    free(m->fr_a);
    free(m->fr_iz);
    free(m->fr_iy);
    free(m->fr_ip);
    free(m->fr_iw);
    free(m->fr_aux);
    free(m->fr_len0);
    free(m->fr_c0);
    free(m->fr_mc);
    free(m->pinpt);
    free(m->um0);
    free(m->vm0);
    free(m->am0);
    free(m);
}

/* Frame triad from prop_fr (frame.c:130-160) / updatc (misc.c:110-147):
 * x^ along the member, z^ = x^ x (aux - end 1) normalised, y^ = z^ x x^. */
static void frame_geometry(const double *pa, const double *pb, const double *aux, double *c, double *len)
{
    double el[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    double L = sqrt(dot3(el, el));
    double lx[3] = {el[0] / L, el[1] / L, el[2] / L};
    double tmp[3] = {aux[0] - pa[0], aux[1] - pa[1], aux[2] - pa[2]};
    double lz[3], ly[3];
    cross3(lx, tmp, lz, 1);
    cross3(lz, lx, ly, 1);
    for (int m = 0; m < 3; ++m) {
        c[m] = lx[m];
        c[3 + m] = ly[m];
        c[6 + m] = lz[m];
    }
    *len = L;
}

static orc_model *load_fail(orc_model *m, char *err, int errlen, const char *msg)
{
    set_err(err, errlen, msg);
    orc_free(m);
    return NULL;
}

orc_model *orc_load(const char *text, char *err, int errlen)
{
    tok_t t = {text, 1};
    orc_model *m = calloc(1, sizeof *m);
    int ana = (int)tok_num(&t);
    int alg = (int)tok_num(&t);
    if (!((ana == 2 && (alg == 3 || alg == 5)) || (ana == 1 && alg == 4)))
        return load_fail(m, err, errlen, "oracle supports ANAFLAG 2 with ALGFLAG 3 (MSAL) or 5 (Newmark), "
                                         "and ANAFLAG 1 with ALGFLAG 4 (linear Newmark)");
    m->alg = alg;
    if (alg > 3) {
        int chkpt = (int)tok_num(&t), rflag = (int)tok_num(&t);
        (void)chkpt;
        if (rflag != 0) return load_fail(m, err, errlen, "restart input (RFLAG 1) is not supported");
    }
    int slv = (int)tok_num(&t);
    int opt = (int)tok_num(&t);
    if (slv != 0 || opt != 1) return load_fail(m, err, errlen, "oracle supports SLVFLAG 0 and OPTFLAG 1");
    m->nj = (long)tok_num(&t);
    m->ne_tr = (long)tok_num(&t);
    m->ne_fr = (long)tok_num(&t);
    m->ne_sh = (long)tok_num(&t);
    long nsbr = (long)tok_num(&t), nfbr = (long)tok_num(&t);
    if (nsbr || nfbr || !t.ok) return load_fail(m, err, errlen, "brick elements are not supported");
    if (alg == 5 && (m->ne_tr || m->ne_sh))
        return load_fail(m, err, errlen, "the nonlinear Newmark oracle supports frame-only models");
    if (alg == 4 && (m->ne_tr || (m->ne_sh && m->ne_fr)))
        return load_fail(m, err, errlen, "the linear Newmark oracle supports frame-only or shell-only models");
    long NJ = m->nj;
    m->tr_conn = calloc((size_t)(2 * m->ne_tr + 1), sizeof(long));
    m->fr_conn = calloc((size_t)(2 * m->ne_fr + 1), sizeof(long));
    m->sh_conn = calloc((size_t)(3 * m->ne_sh + 1), sizeof(long));
    /* joint-element connectivity (model.c:95-133) and frames per joint */
    int *has_tr = calloc((size_t)NJ, sizeof(int)), *has_sh = calloc((size_t)NJ, sizeof(int));
    int *nfr = calloc((size_t)NJ, sizeof(int)), *wrp = calloc((size_t)NJ, sizeof(int));
    for (long i = 0; i < 2 * m->ne_tr; ++i) {
        m->tr_conn[i] = (long)tok_num(&t) - 1;
        has_tr[m->tr_conn[i]] = 1;
    }
    for (long i = 0; i < 2 * m->ne_fr; ++i) {
        m->fr_conn[i] = (long)tok_num(&t) - 1;
        nfr[m->fr_conn[i]]++;
    }
    for (long i = 0; i < 3 * m->ne_sh; ++i) {
        m->sh_conn[i] = (long)tok_num(&t) - 1;
        has_sh[m->sh_conn[i]] = 1;
    }
    /* constraints (model.c:216-264): free = -1, fixed = 0; "j,7,r" sets the
     * warping restraint flag r (1 = one warping DOF per member) */
    m->jcode = malloc(sizeof(long) * (size_t)NJ * 7);
    for (long i = 0; i < NJ * 7; ++i) m->jcode[i] = -1;
    for (;;) {
        long j = (long)tok_num(&t), k = (long)tok_num(&t);
        if (!t.ok || j == 0) break;
        if (k < 1 || k > 7 || j > NJ) {
            free(has_tr);
            free(has_sh);
            free(nfr);
            free(wrp);
            return load_fail(m, err, errlen, "bad constraint line");
        }
        if (k == 7) wrp[j - 1] = (int)tok_num(&t);
        m->jcode[(j - 1) * 7 + k - 1] = 0;
    }
    /* DOFs that no element type uses (model.c:267-285) */
    for (long i = 0; i < NJ; ++i) {
        if (nfr[i] == 0) {
            if (!has_sh[i]) {
                int from = has_tr[i] ? 3 : 0;
                for (int j = from; j < 7; ++j) m->jcode[i * 7 + j] = 0;
            } else {
                m->jcode[i * 7 + 6] = 0;
            }
        }
    }
    /* equation numbers (codes, model.c:941-961) */
    long neq = 0;
    for (long i = 0; i < NJ; ++i) {
        for (int j = 0; j < 6; ++j)
            if (m->jcode[i * 7 + j] != 0) m->jcode[i * 7 + j] = ++neq;
        if (m->jcode[i * 7 + 6] != 0) {
            m->jcode[i * 7 + 6] = ++neq;
        } else if (wrp[i] == 1) {
            m->jcode[i * 7 + 6] = ++neq;
            neq += nfr[i] - 1;
        }
    }
    m->neq = neq;
    /* frame member codes: the warping DOF of a joint with one warping DOF
     * per member counts up over the members in element order (model.c:1007-1032) */
    m->fr_mc = calloc((size_t)(14 * m->ne_fr + 1), sizeof(long));
    int *cnt = calloc((size_t)NJ, sizeof(int));
    for (long i = 0; i < NJ; ++i) cnt[i] = nfr[i];
    for (long e = 0; e < m->ne_fr; ++e)
        for (int a = 0; a < 2; ++a) {
            long j = m->fr_conn[e * 2 + a];
            for (int d = 0; d < 6; ++d) m->fr_mc[e * 14 + a * 7 + d] = m->jcode[j * 7 + d];
            if (wrp[j] == 1) {
                m->fr_mc[e * 14 + a * 7 + 6] = m->jcode[j * 7 + 6] + nfr[j] - cnt[j];
                cnt[j]--;
            } else {
                m->fr_mc[e * 14 + a * 7 + 6] = m->jcode[j * 7 + 6];
            }
        }
    free(cnt);
    free(has_tr);
    free(has_sh);
    free(nfr);
    free(wrp);
    /* prescribed motion list of dynamic analyses (skylin, model.c:1156-1201) */
    if (alg > 3) {
        long j = (long)tok_num(&t), k = (long)tok_num(&t);
        (void)k;
        if (j != 0) return load_fail(m, err, errlen, "prescribed support motion (NBC > 0) is not supported");
    }
    /* skyline profile (skylin, model.c:1204-1277): trusses, frames, shells */
    long *kht = calloc((size_t)neq + 1, sizeof(long));
    for (long e = 0; e < m->ne_tr + m->ne_fr + m->ne_sh; ++e) {
        long mc[18];
        int nd = 0;
        if (e < m->ne_tr) {
            for (int a = 0; a < 2; ++a)
                for (int d = 0; d < 3; ++d) mc[nd++] = m->jcode[m->tr_conn[e * 2 + a] * 7 + d];
        } else if (e < m->ne_tr + m->ne_fr) {
            long f = e - m->ne_tr;
            for (int k = 0; k < 14; ++k) mc[nd++] = m->fr_mc[f * 14 + k];
        } else {
            long s = e - m->ne_tr - m->ne_fr;
            for (int a = 0; a < 3; ++a)
                for (int d = 0; d < 6; ++d) mc[nd++] = m->jcode[m->sh_conn[s * 3 + a] * 7 + d];
        }
        long mn = neq;
        for (int k = 0; k < nd; ++k)
            if (mc[k] > 0 && mc[k] < mn) mn = mc[k];
        for (int k = 0; k < nd; ++k)
            if (mc[k] != 0 && mc[k] - mn > kht[mc[k] - 1]) kht[mc[k] - 1] = mc[k] - mn;
    }
    m->maxa = malloc(sizeof(long) * (size_t)(neq + 1));
    m->maxa[0] = 1;
    for (long i = 0; i < neq; ++i) m->maxa[i + 1] = m->maxa[i] + kht[i] + 1;
    m->lss = m->maxa[neq] - 1;
    free(kht);
    /* coordinates */
    m->x0 = malloc(sizeof(double) * (size_t)NJ * 3);
    for (long i = 0; i < NJ * 3; ++i) m->x0[i] = tok_num(&t);
    /* truss properties and geometry (prop_tr, truss.c:41-80) */
    m->tr_e = calloc((size_t)m->ne_tr + 1, sizeof(double));
    m->tr_a = calloc((size_t)m->ne_tr + 1, sizeof(double));
    m->tr_len0 = calloc((size_t)m->ne_tr + 1, sizeof(double));
    m->tr_dir0 = calloc((size_t)m->ne_tr * 3 + 1, sizeof(double));
    for (long i = 0; i < m->ne_tr; ++i) {
        const double *pa = m->x0 + m->tr_conn[i * 2] * 3, *pb = m->x0 + m->tr_conn[i * 2 + 1] * 3;
        double el[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
        m->tr_len0[i] = sqrt(dot3(el, el));
        for (int k = 0; k < 3; ++k) m->tr_dir0[i * 3 + k] = el[k] / m->tr_len0[i];
        m->tr_e[i] = tok_num(&t);
        m->tr_a[i] = tok_num(&t);
        (void)tok_num(&t); /* density */
        (void)tok_num(&t); /* yield */
    }
    /* frame properties (prop_fr, frame.c:43-224) */
    long F = m->ne_fr;
    double **fp[] = {&m->fr_e, &m->fr_g, &m->fr_dens, &m->fr_a, &m->fr_iz, &m->fr_iy, &m->fr_ip, &m->fr_iw};
    for (int k = 0; k < 8; ++k) *fp[k] = calloc((size_t)F + 1, sizeof(double));
    m->fr_aux = calloc((size_t)F * 3 + 1, sizeof(double));
    m->fr_len0 = calloc((size_t)F + 1, sizeof(double));
    m->fr_c0 = calloc((size_t)F * 9 + 1, sizeof(double));
    if (F > 0) {
        for (long i = 0; i < F; ++i)
            for (int k = 0; k < 8; ++k) (*fp[k])[i] = tok_num(&t);
        long j = (long)tok_num(&t);
        for (int k = 0; k < 6; ++k) (void)tok_num(&t);
        if (j != 0) return load_fail(m, err, errlen, "frame member end offsets are not supported");
        for (long i = 0; i < F * 3; ++i) m->fr_aux[i] = tok_num(&t);
        for (long i = 0; i < F * 3; ++i) (void)tok_num(&t); /* yield, plastic moduli */
        j = (long)tok_num(&t);
        for (int k = 0; k < 4; ++k) (void)tok_num(&t);
        if (j != 0) return load_fail(m, err, errlen, "frame member end releases are not supported");
        for (long i = 0; i < F; ++i)
            frame_geometry(m->x0 + m->fr_conn[i * 2] * 3, m->x0 + m->fr_conn[i * 2 + 1] * 3,
                           m->fr_aux + i * 3, m->fr_c0 + i * 9, m->fr_len0 + i);
    }
    /* shell properties and geometry (prop_sh, shell.c:43-108) */
    long E = m->ne_sh;
    m->sh_e = calloc((size_t)E + 1, sizeof(double));
    m->sh_nu = calloc((size_t)E + 1, sizeof(double));
    m->sh_t = calloc((size_t)E + 1, sizeof(double));
    m->sh_dens = calloc((size_t)E + 1, sizeof(double));
    m->sh_xl = calloc((size_t)E * 3 + 1, sizeof(double));
    m->sh_area0 = calloc((size_t)E + 1, sizeof(double));
    m->sh_slen0 = calloc((size_t)E * 3 + 1, sizeof(double));
    m->sh_c0 = calloc((size_t)E * 9 + 1, sizeof(double));
    m->sh_kem = calloc((size_t)E * 36 + 1, sizeof(double));
    m->sh_keb = calloc((size_t)E * 81 + 1, sizeof(double));
    for (long i = 0; i < E; ++i) {
        m->sh_e[i] = tok_num(&t);
        m->sh_nu[i] = tok_num(&t);
        m->sh_t[i] = tok_num(&t);
        m->sh_dens[i] = tok_num(&t); /* density (mass_sh) */
        (void)tok_num(&t);            /* yield */
        const double *p1 = m->x0 + m->sh_conn[i * 3] * 3, *p2 = m->x0 + m->sh_conn[i * 3 + 1] * 3,
                     *p3 = m->x0 + m->sh_conn[i * 3 + 2] * 3;
        shell_geometry(p1, p2, p3, m->sh_c0 + i * 9, m->sh_area0 + i, m->sh_slen0 + i * 3);
        shell_local(p1, p2, p3, m->sh_c0 + i * 9, m->sh_xl + i * 3);
        shell_kem(m->sh_e[i], m->sh_nu[i], m->sh_t[i], m->sh_area0[i], m->sh_xl + i * 3,
                  m->sh_kem + i * 36);
        shell_keb(m->sh_e[i], m->sh_nu[i], m->sh_t[i], m->sh_area0[i], m->sh_xl + i * 3,
                  m->sh_slen0 + i * 3, m->sh_keb + i * 81);
    }
    m->q = calloc((size_t)neq + 1, sizeof(double));
    if (alg == 3) {
        /* joint loads (load, model.c:1313-1335), then frame distributed loads */
        for (;;) {
            long jt = (long)tok_num(&t);
            long dir = (long)tok_num(&t);
            double mag = tok_num(&t);
            if (!t.ok || jt == 0) break;
            long k = m->jcode[(jt - 1) * 7 + dir - 1];
            if (k != 0) m->q[k - 1] = mag;
        }
        if (F > 0) {
            long fr = (long)tok_num(&t);
            (void)tok_num(&t);
            (void)tok_num(&t);
            if (fr != 0) return load_fail(m, err, errlen, "frame distributed loads are not supported");
        }
        /* MSAL controls (msal, arc.c:41-68; main.c:2240-2245) */
        long jt = (long)tok_num(&t);
        long dir = (long)tok_num(&t);
        m->dk = tok_num(&t);
        m->alpha = tok_num(&t);
        m->psi_thresh = tok_num(&t);
        m->iteopt = (int)tok_num(&t);
        m->lpfmax = tok_num(&t);
        m->dkimax = tok_num(&t);
        m->itemax = (int)tok_num(&t);
        m->submax = (int)tok_num(&t);
        m->imagmax = (int)tok_num(&t);
        m->negmax = (int)tok_num(&t);
        m->toldisp = tok_num(&t);
        m->tolforc = tok_num(&t);
        m->tolener = tok_num(&t);
        if (!t.ok) return load_fail(m, err, errlen, "model_def ended early");
        m->dkdof = m->jcode[(jt - 1) * 7 + dir - 1] - 1;
        if (m->dkdof < 0) return load_fail(m, err, errlen, "initially prescribed displacement at a fixed DOF");
    } else {
        /* time points (main.c:1600-1607) */
        long ntsteps = (long)tok_num(&t);
        m->ttot = tok_num(&t);
        m->dt = m->ttot / (double)ntsteps;
        m->ntin = ntsteps + 1;
        m->nsteps = (long)(m->ttot / m->dt + 1);
        /* per-step joint forces (load, model.c:1516-1549): lines of one DOF
         * are consecutive time points; a zero force is stored as 1e-30 */
        m->pinpt = calloc((size_t)(neq * m->ntin + 1), sizeof(double));
        long kps = 0, i = 0;
        for (;;) {
            long jt = (long)tok_num(&t);
            long dir = (long)tok_num(&t);
            double mag = tok_num(&t);
            if (!t.ok || jt == 0) break;
            if (alg == 5 && mag == 0) mag = 1e-30;
            long ks = m->jcode[(jt - 1) * 7 + dir - 1];
            if (ks != kps) i = 0;
            if (ks != 0 && i < m->ntin) m->pinpt[(ks - 1) * m->ntin + i] = mag;
            kps = ks;
            ++i;
        }
        /* prescribed support displacements (none supported) and initial conditions */
        long jt = (long)tok_num(&t);
        (void)tok_num(&t);
        (void)tok_num(&t);
        if (jt != 0) return load_fail(m, err, errlen, "prescribed displacements are not supported");
        /* initial conditions: kept by the linear driver only, since the
         * nonlinear one zeroes its motion before the first step */
        m->um0 = calloc((size_t)neq + 1, sizeof(double));
        m->vm0 = calloc((size_t)neq + 1, sizeof(double));
        m->am0 = calloc((size_t)neq + 1, sizeof(double));
        for (;;) {
            jt = (long)tok_num(&t);
            long dir = (long)tok_num(&t);
            double d0 = tok_num(&t), v0 = tok_num(&t), a0 = tok_num(&t);
            if (!t.ok || jt == 0) break;
            if (jt < 1 || jt > NJ || dir < 1 || dir > 7) return load_fail(m, err, errlen, "bad initial condition");
            long k = m->jcode[(jt - 1) * 7 + dir - 1];
            if (k != 0) {
                if (d0 != 0) m->um0[k - 1] = d0;
                if (v0 != 0) m->vm0[k - 1] = v0;
                if (a0 != 0) m->am0[k - 1] = a0;
            }
        }
        if (alg == 4) {
            /* linear Newmark controls (main.c:3184, 3192) */
            m->numopt = tok_num(&t);
            m->spectrds = tok_num(&t);
            m->lpfmax = tok_num(&t);
            if (!t.ok) return load_fail(m, err, errlen, "model_def ended early");
            if (m->numopt == 0 && m->spectrds != 1)
                return load_fail(m, err, errlen, "invalid spectral radius for Newmark without dissipation");
            return m;
        }
        /* Newmark controls (main.c:3320-3326) */
        m->numopt = tok_num(&t);
        m->spectrds = tok_num(&t);
        m->lpfmax = tok_num(&t);
        m->lpf0 = tok_num(&t);
        m->dlpf0 = tok_num(&t);
        m->dlpfmax = tok_num(&t);
        m->dlpfmin = tok_num(&t);
        m->itemax = (int)tok_num(&t);
        m->submax = (int)tok_num(&t);
        m->solmin = (int)tok_num(&t);
        m->toldisp = tok_num(&t);
        m->tolforc = tok_num(&t);
        m->tolener = tok_num(&t);
        if (!t.ok) return load_fail(m, err, errlen, "model_def ended early");
        if (m->numopt == 0 && m->spectrds != 1)
            return load_fail(m, err, errlen, "invalid spectral radius for Newmark without dissipation");
    }
    return m;
}

void orc_sizes(const orc_model *m, long *out)
{
    out[0] = m->nj;
    out[1] = m->ne_tr;
    out[2] = m->ne_fr;
    out[3] = m->ne_sh;
    out[4] = m->neq;
    out[5] = m->lss;
    out[6] = m->dkdof;
    out[7] = m->itemax;
}

void orc_dyn_sizes(const orc_model *m, long *nsteps, double *dt)
{
    *nsteps = m->nsteps;
    *dt = m->dt;
}

void orc_topology(const orc_model *m, long *jcode, double *q)
{
    memcpy(jcode, m->jcode, sizeof(long) * (size_t)m->nj * 7);
    memcpy(q, m->q, sizeof(double) * (size_t)m->neq);
}

void orc_shell_initial(const orc_model *m, double *c, double *area)
{
    memcpy(c, m->sh_c0, sizeof(double) * (size_t)m->ne_sh * 9);
    memcpy(area, m->sh_area0, sizeof(double) * (size_t)m->ne_sh);
}

/* ------------------------------------------------------------------------ */
/* Element forces                                                            */
/* ------------------------------------------------------------------------ */

static void shell_mcode(const orc_model *m, long s, long *mc)
{
    for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 6; ++d) mc[a * 6 + d] = m->jcode[m->sh_conn[s * 3 + a] * 7 + d];
}

/* One DKT element of forces_sh, ANAFLAG 2 branch (shell.c:1728-1785 and
 * 2305-2397): membrane force from the total local displacement, bending force
 * from the incremental displacement rotated into the previous frame, both
 * carried into the current frame by R_i R_ip^T and scattered as T_i^T ef_i.
 * ef_ip_mem_zeroed mirrors the reference zeroing ef_ip's membrane entries
 * (shell.c:1773) before it is rotated. */
static void shell_force_element(const orc_model *m, long s, const double *x_temp,
                                const double *dd, const double *cip, const double *efip,
                                double *ci, double *area_i, double *efi, double *fe)
{
    static const int flagm[6] = {0, 1, 6, 7, 12, 13};
    const long *cn = m->sh_conn + s * 3;
    const double *p1 = x_temp + cn[0] * 3, *p2 = x_temp + cn[1] * 3, *p3 = x_temp + cn[2] * 3;
    shell_geometry(p1, p2, p3, ci, area_i, NULL);
    double xlc[3];
    shell_local(p1, p2, p3, ci, xlc);
    const double *xl = m->sh_xl + s * 3;
    double dm[6] = {0, 0, xlc[0] - xl[0], 0, xlc[1] - xl[1], xlc[2] - xl[2]};
    long mc[18];
    shell_mcode(m, s, mc);
    double DD[18];
    for (int i = 0; i < 18; ++i) DD[i] = mc[i] ? dd[mc[i] - 1] : 0.0;
    /* ddb = rows {2,3,4} of each node block of T_ip applied to DD */
    double ddb[9];
    for (int a = 0; a < 3; ++a) {
        const double *u = DD + 6 * a, *r = DD + 6 * a + 3;
        ddb[3 * a] = cip[6] * u[0] + cip[7] * u[1] + cip[8] * u[2];
        ddb[3 * a + 1] = cip[0] * r[0] + cip[1] * r[1] + cip[2] * r[2];
        ddb[3 * a + 2] = cip[3] * r[0] + cip[4] * r[1] + cip[5] * r[2];
    }
    double ef_temp[18] = {0}, def[18] = {0}, efp[18];
    memcpy(efp, efip, sizeof efp);
    const double *kem = m->sh_kem + s * 36, *keb = m->sh_keb + s * 81;
    for (int i = 0; i < 6; ++i) {
        double sum = 0;
        for (int j = 0; j < 6; ++j) sum += kem[i * 6 + j] * dm[j];
        efp[flagm[i]] = 0;
        ef_temp[flagm[i]] = sum;
    }
    static const int flagb[9] = {2, 3, 4, 8, 9, 10, 14, 15, 16};
    for (int i = 0; i < 9; ++i) {
        double sum = 0;
        for (int j = 0; j < 9; ++j) sum += keb[i * 9 + j] * ddb[j];
        def[flagb[i]] = sum;
    }
    /* R_rel = R_i R_ip^T (the 3x3 block of T_i T_ip^T) */
    double Rr[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            Rr[r][c] = ci[r * 3] * cip[c * 3] + ci[r * 3 + 1] * cip[c * 3 + 1] +
                       ci[r * 3 + 2] * cip[c * 3 + 2];
    for (int b = 0; b < 6; ++b)
        for (int r = 0; r < 3; ++r) {
            double sum = 0;
            for (int c = 0; c < 3; ++c) sum += Rr[r][c] * (def[3 * b + c] + efp[3 * b + c]);
            efi[3 * b + r] = ef_temp[3 * b + r] + sum;
        }
    /* T_i^T ef_i */
    for (int b = 0; b < 6; ++b)
        for (int c = 0; c < 3; ++c)
            fe[3 * b + c] = ci[c] * efi[3 * b] + ci[3 + c] * efi[3 * b + 1] + ci[6 + c] * efi[3 * b + 2];
}

void orc_shell_forces(const orc_model *m, const double *x_temp, const double *dd,
                      const double *c_ip, const double *ef_ip, double *c_i, double *area_i,
                      double *ef_i, double *f)
{
    memset(f, 0, sizeof(double) * (size_t)m->neq);
    for (long s = 0; s < m->ne_sh; ++s) {
        double fe[18];
        long mc[18];
        shell_force_element(m, s, x_temp, dd, c_ip + s * 9, ef_ip + s * 18, c_i + s * 9, area_i + s,
                            ef_i + s * 18, fe);
        shell_mcode(m, s, mc);
        for (int i = 0; i < 18; ++i)
            if (mc[i]) f[mc[i] - 1] += fe[i];
    }
}

/* Truss geometry update (misc.c:95-107) and force (truss.c:326-375). */
static void truss_force_element(const orc_model *m, long e, const double *x_temp, double *len_i,
                                double *dir_i, double *ef)
{
    const double *pa = x_temp + m->tr_conn[e * 2] * 3, *pb = x_temp + m->tr_conn[e * 2 + 1] * 3;
    double el[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    double L = sqrt(dot3(el, el));
    *len_i = L;
    for (int k = 0; k < 3; ++k) dir_i[k] = el[k] / L;
    double L0 = m->tr_len0[e];
    double strain = (L - L0) / L0;
    ef[0] = m->tr_e[e] * m->tr_a[e] * (strain + 0.5 * pow(strain, 2)) * L / L0;
    ef[1] = -ef[0];
}

void orc_truss_forces(const orc_model *m, const double *x_temp, double *length_i, double *dir_i,
                      double *ef_i, double *f)
{
    for (long e = 0; e < m->ne_tr; ++e) {
        truss_force_element(m, e, x_temp, length_i + e, dir_i + e * 3, ef_i + e * 2);
        for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 3; ++d) {
                long k = m->jcode[m->tr_conn[e * 2 + a] * 7 + d];
                if (k) f[k - 1] -= ef_i[e * 2 + a] * dir_i[e * 3 + d];
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Frame element (14 DOF)                                                    */
/* ------------------------------------------------------------------------ */

/* Local 14x14 stiffness of the frame: elastic part (stiffe_fr,
 * frame.c:364-408) with reference length L0, plus the geometric part
 * (stiffg_fr, frame.c:410-579) from the previous total end forces ef and
 * deformed length L. DOFs per end: u, v, w, thx, thy, thz, warping. */
#define KSYM(i, j, v)                 \
    do {                              \
        double v_ = (v);              \
        k[i][j] += v_;                \
        if ((i) != (j)) k[j][i] += v_; \
    } while (0)

static void frame_klocal(const orc_model *m, long e, double L0, const double *ef, double L,
                         double k[14][14])
{
    const double E = m->fr_e[e], G = m->fr_g[e], A = m->fr_a[e], Iz = m->fr_iz[e], Iy = m->fr_iy[e],
                 J = m->fr_ip[e], Iw = m->fr_iw[e];
    memset(k, 0, sizeof(double) * 196);
    k[0][0] = k[7][7] = E * A / L0;
    k[7][0] = k[0][7] = -k[0][0];
    k[1][1] = k[8][8] = 12 * E * Iz / pow(L0, 3);
    k[8][1] = k[1][8] = -k[1][1];
    k[2][2] = k[9][9] = 12 * E * Iy / pow(L0, 3);
    k[9][2] = k[2][9] = -k[2][2];
    k[3][3] = k[10][10] = 6 * G * J / (5 * L0) + 12 * E * Iw / pow(L0, 3);
    k[10][3] = k[3][10] = -k[3][3];
    k[5][5] = k[12][12] = 4 * E * Iz / L0;
    k[4][4] = k[11][11] = 4 * E * Iy / L0;
    k[6][6] = k[13][13] = 2 * G * J * L0 / 15 + 4 * E * Iw / L0;
    k[5][1] = k[1][5] = k[12][1] = k[1][12] = 6 * E * Iz / pow(L0, 2);
    k[8][5] = k[5][8] = k[12][8] = k[8][12] = -k[5][1];
    k[9][4] = k[4][9] = k[11][9] = k[9][11] = 6 * E * Iy / pow(L0, 2);
    k[4][2] = k[2][4] = k[11][2] = k[2][11] = -k[9][4];
    k[6][3] = k[3][6] = k[13][3] = k[3][13] = G * J / 10 + 6 * E * Iw / pow(L0, 2);
    k[10][6] = k[6][10] = k[13][10] = k[10][13] = -k[6][3];
    k[12][5] = k[5][12] = 2 * E * Iz / L0;
    k[11][4] = k[4][11] = 2 * E * Iy / L0;
    k[13][6] = k[6][13] = -(G * J * L0 / 30 - 2 * E * Iw / L0);
    /* geometric stiffness of the axial force P = ef[7] and the end moments */
    const double P = ef[7], e4 = ef[4], e5 = ef[5], e10 = ef[10], e11 = ef[11], e12 = ef[12];
    k[0][0] += P / L;
    k[7][7] += P / L;
    KSYM(7, 0, -(P / L));
    k[1][1] += 6 * P / (5 * L);
    k[8][8] += 6 * P / (5 * L);
    k[2][2] += 6 * P / (5 * L);
    k[9][9] += 6 * P / (5 * L);
    KSYM(8, 1, -(6 * P / (5 * L)));
    KSYM(9, 2, -(6 * P / (5 * L)));
    k[3][3] += 6 * P * J / (5 * A * L);
    k[10][10] += 6 * P * J / (5 * A * L);
    KSYM(10, 3, -(6 * P * J / (5 * A * L)));
    k[4][4] += 2 * P * L / 15;
    k[11][11] += 2 * P * L / 15;
    k[5][5] += 2 * P * L / 15;
    k[12][12] += 2 * P * L / 15;
    k[6][6] += 2 * P * J / (15 * A);
    k[13][13] += 2 * P * J / (15 * A);
    KSYM(3, 1, (11 * e4 - e11) / (10 * L));
    KSYM(8, 3, -((11 * e4 - e11) / (10 * L)));
    KSYM(4, 1, e10 / L);
    KSYM(5, 2, e10 / L);
    KSYM(11, 8, e10 / L);
    KSYM(12, 9, e10 / L);
    KSYM(11, 1, -(e10 / L));
    KSYM(12, 2, -(e10 / L));
    KSYM(8, 4, -(e10 / L));
    KSYM(9, 5, -(e10 / L));
    KSYM(5, 1, P / 10);
    KSYM(12, 1, P / 10);
    KSYM(9, 4, P / 10);
    KSYM(11, 9, P / 10);
    KSYM(4, 2, -(P / 10));
    KSYM(11, 2, -(P / 10));
    KSYM(8, 5, -(P / 10));
    KSYM(12, 8, -(P / 10));
    KSYM(6, 1, e4 / 10);
    KSYM(8, 6, -(e4 / 10));
    KSYM(10, 8, (e4 - 11 * e11) / (10 * L));
    KSYM(10, 1, -((e4 - 11 * e11) / (10 * L)));
    KSYM(13, 8, e11 / 10);
    KSYM(13, 1, -(e11 / 10));
    KSYM(3, 2, (11 * e5 - e12) / (10 * L));
    KSYM(9, 3, -((11 * e5 - e12) / (10 * L)));
    KSYM(6, 2, e5 / 10);
    KSYM(9, 6, -(e5 / 10));
    KSYM(10, 9, (e5 - 11 * e12) / (10 * L));
    KSYM(10, 2, -((e5 - 11 * e12) / (10 * L)));
    KSYM(13, 9, e12 / 10);
    KSYM(13, 2, -(e12 / 10));
    KSYM(4, 3, -((2 * e5 - e12) / 5));
    KSYM(5, 3, (2 * e4 - e11) / 5);
    KSYM(6, 3, P * J / (10 * A));
    KSYM(13, 3, P * J / (10 * A));
    KSYM(10, 6, -(P * J / (10 * A)));
    KSYM(13, 10, -(P * J / (10 * A)));
    KSYM(11, 3, -((2 * e5 + e12) / 10));
    KSYM(12, 3, (2 * e4 + e11) / 10);
    KSYM(6, 4, -((3 * e5 - e12) * L / 30));
    KSYM(10, 4, -((e5 + 2 * e12) / 10));
    KSYM(11, 4, -(P * L / 30));
    KSYM(12, 5, -(P * L / 30));
    KSYM(12, 4, e10 / 2);
    KSYM(11, 5, -(e10 / 2));
    KSYM(13, 4, e5 * L / 30);
    KSYM(6, 5, (3 * e4 - e11) * L / 30);
    KSYM(10, 5, (e4 + 2 * e11) / 10);
    KSYM(13, 5, -(e4 * L / 30));
    KSYM(11, 6, -(e12 * L / 30));
    KSYM(12, 6, e11 * L / 30);
    KSYM(13, 6, -(P * J / (30 * A)));
    KSYM(11, 10, (e5 - 2 * e12) / 5);
    KSYM(12, 10, -((e4 - 2 * e11) / 5));
    KSYM(13, 11, -((e5 - 3 * e12) * L / 30));
    KSYM(13, 12, (e4 - 3 * e11) * L / 30);
}
#undef KSYM

/* 14x14 frame transformation T: the triad on the four 3x3 translation and
 * rotation blocks, 1 on the two warping DOFs (frame.c:284-296). */
static void frame_T(const double *c, double T[14][14])
{
    memset(T, 0, sizeof(double) * 196);
    static const int base[4] = {0, 3, 7, 10};
    for (int b = 0; b < 4; ++b)
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) T[base[b] + r][base[b] + q] = c[r * 3 + q];
    T[6][6] = T[13][13] = 1;
}

/* One frame of forces_fr, ANAFLAG 2, no offsets (frame.c:902-1312) with the
 * frame part of updatc (misc.c:108-147). */
static void frame_force_element(const orc_model *m, long e, const double *x_temp, const double *dd,
                                const double *cip, const double *efip, double len_ip, double lref,
                                double *ci, double *len_i, double *efi, double *fe)
{
    const long *cn = m->fr_conn + e * 2;
    frame_geometry(x_temp + cn[0] * 3, x_temp + cn[1] * 3, m->fr_aux + e * 3, ci, len_i);
    double k[14][14], Tip[14][14], Ti[14][14];
    frame_klocal(m, e, lref, efip, len_ip, k);
    frame_T(cip, Tip);
    frame_T(ci, Ti);
    double DD[14], dl[14], def[14];
    for (int i = 0; i < 14; ++i) {
        long q = m->fr_mc[e * 14 + i];
        DD[i] = q ? dd[q - 1] : 0.0;
    }
    for (int i = 0; i < 14; ++i) {
        double sum = 0;
        for (int j = 0; j < 14; ++j) sum += Tip[i][j] * DD[j];
        dl[i] = sum;
    }
    for (int i = 0; i < 14; ++i) {
        double sum = 0;
        for (int j = 0; j < 14; ++j) sum += k[i][j] * dl[j];
        def[i] = sum;
    }
    double TT[14][14];
    for (int i = 0; i < 14; ++i)
        for (int j = 0; j < 14; ++j) {
            double sum = 0;
            for (int q = 0; q < 14; ++q) sum += Ti[i][q] * Tip[j][q];
            TT[i][j] = sum;
        }
    for (int i = 0; i < 14; ++i) {
        double sum = 0;
        for (int j = 0; j < 14; ++j) sum += TT[i][j] * (efip[j] + def[j]);
        efi[i] = sum;
    }
    for (int i = 0; i < 14; ++i) {
        double sum = 0;
        for (int j = 0; j < 14; ++j) sum += Ti[j][i] * efi[j];
        fe[i] = sum;
    }
}

/* Frame tangent K = T^T k T (stiff_fr, frame.c:226-362, transform misc.c:41-69). */
static void frame_tangent_element(const orc_model *m, long e, const double *c, const double *ef,
                                  double len, double lref, double K[14][14])
{
    double k[14][14], T[14][14], tmp[14][14];
    frame_klocal(m, e, lref, ef, len, k);
    frame_T(c, T);
    for (int i = 0; i < 14; ++i)
        for (int j = 0; j < 14; ++j) {
            double sum = 0;
            for (int q = 0; q < 14; ++q) sum += T[q][i] * k[q][j];
            tmp[i][j] = sum;
        }
    for (int i = 0; i < 14; ++i)
        for (int j = 0; j < 14; ++j) {
            double sum = 0;
            for (int q = 0; q < 14; ++q) sum += tmp[i][q] * T[q][j];
            K[i][j] = sum;
        }
}

/* Lumped frame mass (mass_fr, frame.c:1314-1391): rho A L / 24 * 12 on the
 * translations, rho A L / 24 * L^2 on the rotations, nothing on warping,
 * with L the member length at the coordinates x; also returns L. */
static double frame_mass_element(const orc_model *m, long e, const double *x, double *mt, double *mr)
{
    const long *cn = m->fr_conn + e * 2;
    double el[3];
    for (int k = 0; k < 3; ++k) el[k] = x[cn[1] * 3 + k] - x[cn[0] * 3 + k];
    double L = sqrt(dot3(el, el));
    double rAL = m->fr_dens[e] * m->fr_a[e] * L;
    *mt = rAL / 24 * 12;
    *mr = rAL / 24 * pow(L, 2);
    return L;
}

/* ------------------------------------------------------------------------ */
/* Tangent stiffness                                                         */
/* ------------------------------------------------------------------------ */

static void sky_add(const orc_model *m, double *ss, const long *mc, int nd, const double *K)
{
    /* element (ie <= je) entries into the 1-based skyline (truss.c:170-193) */
    for (int je = 0; je < nd; ++je) {
        long j = mc[je];
        if (!j) continue;
        for (int ie = 0; ie <= je; ++ie) {
            long i = mc[ie];
            if (!i) continue;
            long k = i > j ? m->maxa[i - 1] + (i - j) : m->maxa[j - 1] + (j - i);
            ss[k - 1] += K[ie * nd + je];
        }
    }
}

/* 18x18 local DKT tangent (stiffe_sh shell.c:346-485 plus stiffg_sh
 * shell.c:660-840) for converged coordinates x, triad c and area. */
static void shell_local_tangent(const orc_model *m, long s, const double *x, const double *c,
                                double area_c, double k[18][18])
{
    memset(k, 0, sizeof(double) * 324);
    static const int mem[6] = {0, 1, 6, 7, 12, 13};
    static const int ben[9] = {2, 3, 4, 8, 9, 10, 14, 15, 16};
    const double *kem = m->sh_kem + s * 36, *keb = m->sh_keb + s * 81;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) k[mem[i]][mem[j]] = kem[i * 6 + j];
    for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j) k[ben[i]][ben[j]] = keb[i * 9 + j];
    k[5][5] = keb[1 * 9 + 1] / 10000;
    k[11][11] = keb[4 * 9 + 4] / 10000;
    k[17][17] = keb[7 * 9 + 7] / 10000;
    /* geometric stiffness from the membrane force of the converged state */
    const long *cn = m->sh_conn + s * 3;
    double xlc[3];
    shell_local(x + cn[0] * 3, x + cn[1] * 3, x + cn[2] * 3, c, xlc);
    const double *xl = m->sh_xl + s * 3;
    double dm[6] = {0, 0, xlc[0] - xl[0], 0, xlc[1] - xl[1], xlc[2] - xl[2]};
    double C[3][3], B[3][6];
    plane_stress(m->sh_e[s], m->sh_nu[s], C);
    membrane_b(xl, area_c, B);
    double CB[3][6], Nm[3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 6; ++j) {
            double sum = 0;
            for (int q = 0; q < 3; ++q) sum += C[i][q] * B[q][j];
            CB[i][j] = sum;
        }
    for (int i = 0; i < 3; ++i) {
        double sum = 0;
        for (int j = 0; j < 6; ++j) sum += CB[i][j] * dm[j];
        Nm[i] = m->sh_t[s] * sum;
    }
    /* kg = A Bnl^T N Bnl; Bnl acts identically on u, v and w of each vertex */
    double a2 = 2 * area_c;
    double bx[3] = {-(xl[2] / a2), xl[2] / a2, 0};
    double by[3] = {(xl[1] - xl[0]) / a2, -(xl[1] / a2), xl[0] / a2};
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            /* (Bnl^T N)[a][.] then times Bnl, in the reference's summation order */
            double t0 = bx[a] * Nm[0] + by[a] * Nm[2];
            double t1 = bx[a] * Nm[2] + by[a] * Nm[1];
            double g = area_c * (t0 * bx[b] + t1 * by[b]);
            for (int p = 0; p < 3; ++p) k[6 * a + p][6 * b + p] += g;
        }
}

/* Tangent of the whole model in the skyline: stiff_tr, stiff_fr, stiff_sh in
 * that order (main.c:2716-2734). Frame state may be NULL when NE_FR == 0. */
static void tangent_all(const orc_model *m, const double *x, const double *c_sh, const double *area_sh,
                        const double *len_tr, const double *dir_tr, const double *ef_tr,
                        const double *c_fr, const double *ef_fr, const double *len_fr,
                        const double *lref_fr, double *ss)
{
    memset(ss, 0, sizeof(double) * (size_t)m->lss);
    /* truss: EA L^2/L0^3 axial plus N/L geometric term (truss.c:100-166) */
    for (long e = 0; e < m->ne_tr; ++e) {
        double kax = m->tr_e[e] * m->tr_a[e] * pow(len_tr[e], 2) / pow(m->tr_len0[e], 3);
        const double *c = dir_tr + e * 3;
        double K[36];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                /* T^T k T with T = [[c,0],[0,c]] and k = kax [[1,-1],[-1,1]] */
                double tk = (i < 3 ? c[i] * kax : c[i - 3] * -kax);
                double tk2 = (i < 3 ? c[i] * -kax : c[i - 3] * kax);
                K[i * 6 + j] = j < 3 ? tk * c[j] : tk2 * c[j - 3];
            }
        double g = ef_tr[e * 2] / len_tr[e];
        for (int i = 0; i < 6; ++i) K[i * 6 + i] += g;
        for (int d = 0; d < 3; ++d) {
            K[d * 6 + d + 3] -= g;
            K[(d + 3) * 6 + d] -= g;
        }
        long mc[6];
        for (int a = 0; a < 2; ++a)
            for (int d = 0; d < 3; ++d) mc[a * 3 + d] = m->jcode[m->tr_conn[e * 2 + a] * 7 + d];
        sky_add(m, ss, mc, 6, K);
    }
    for (long e = 0; e < m->ne_fr; ++e) {
        double K[14][14];
        frame_tangent_element(m, e, c_fr + e * 9, ef_fr + e * 14, len_fr[e], lref_fr[e], K);
        sky_add(m, ss, m->fr_mc + e * 14, 14, &K[0][0]);
    }
    /* shell: T^T k T with T = diag(R, ..., R) (misc.c:41-69) */
    for (long s = 0; s < m->ne_sh; ++s) {
        double k[18][18], K[324];
        const double *R = c_sh + s * 9;
        shell_local_tangent(m, s, x, R, area_sh[s], k);
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b) {
                double tmp[3][3];
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q)
                        tmp[p][q] = R[p] * k[3 * a][3 * b + q] + R[3 + p] * k[3 * a + 1][3 * b + q] +
                                    R[6 + p] * k[3 * a + 2][3 * b + q];
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q)
                        K[(3 * a + p) * 18 + 3 * b + q] =
                            tmp[p][0] * R[q] + tmp[p][1] * R[3 + q] + tmp[p][2] * R[6 + q];
            }
        long mc[18];
        shell_mcode(m, s, mc);
        sky_add(m, ss, mc, 18, K);
    }
}

void orc_tangent(const orc_model *m, const double *x, const double *c_sh, const double *area_sh,
                 const double *len_tr, const double *dir_tr, const double *ef_tr, long *maxa,
                 double *ss)
{
    memcpy(maxa, m->maxa, sizeof(long) * (size_t)(m->neq + 1));
    double *ef0 = calloc((size_t)(14 * m->ne_fr + 1), sizeof(double));
    tangent_all(m, x, c_sh, area_sh, len_tr, dir_tr, ef_tr, m->fr_c0, ef0, m->fr_len0, m->fr_len0, ss);
    free(ef0);
}

void orc_tangent_fr(const orc_model *m, const double *c_fr, const double *ef_fr, const double *len_fr,
                    const double *lref_fr, long *maxa, double *ss)
{
    memcpy(maxa, m->maxa, sizeof(long) * (size_t)(m->neq + 1));
    tangent_all(m, m->x0, NULL, NULL, NULL, NULL, NULL, c_fr, ef_fr, len_fr, lref_fr, ss);
}

void orc_frame_forces(const orc_model *m, const double *x_temp, const double *dd, const double *c_ip,
                      const double *ef_ip, const double *len_ip, const double *lref, double *c_i,
                      double *len_i, double *ef_i, double *f)
{
    memset(f, 0, sizeof(double) * (size_t)m->neq);
    for (long e = 0; e < m->ne_fr; ++e) {
        double fe[14];
        frame_force_element(m, e, x_temp, dd, c_ip + e * 9, ef_ip + e * 14, len_ip[e], lref[e], c_i + e * 9,
                            len_i + e, ef_i + e * 14, fe);
        for (int i = 0; i < 14; ++i) {
            long q = m->fr_mc[e * 14 + i];
            if (q) f[q - 1] += fe[i];
        }
    }
}

void orc_shell_geometry0(const orc_model *m, double *xl, double *slen)
{
    memcpy(xl, m->sh_xl, sizeof(double) * 3 * (size_t)m->ne_sh);
    memcpy(slen, m->sh_slen0, sizeof(double) * 3 * (size_t)m->ne_sh);
}

void orc_frame_mcode(const orc_model *m, long *mc)
{
    memcpy(mc, m->fr_mc, sizeof(long) * 14 * (size_t)m->ne_fr);
}

void orc_frame_initial(const orc_model *m, double *c, double *len)
{
    memcpy(c, m->fr_c0, sizeof(double) * 9 * (size_t)m->ne_fr);
    memcpy(len, m->fr_len0, sizeof(double) * (size_t)m->ne_fr);
}

void orc_frame_mass(const orc_model *m, const double *x, double *sm)
{
    memset(sm, 0, sizeof(double) * (size_t)m->neq);
    for (long e = 0; e < m->ne_fr; ++e) {
        double mt, mr;
        frame_mass_element(m, e, x, &mt, &mr);
        for (int i = 0; i < 14; ++i) {
            long q = m->fr_mc[e * 14 + i];
            int d = i % 7;
            if (q && d < 6) sm[q - 1] += d < 3 ? mt : mr;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Skyline LDL^T (Bathe's active-column COLSOL; solve.c:539-698)             */
/* ------------------------------------------------------------------------ */

/* a(i, n) for the upper triangle, i <= n, 1-based; only valid inside column n */
#define SKY(ss, maxa, i, n) ((ss)[(maxa)[(n)-1] + ((n) - (i)) - 1])

/* stop_nonpos: the ALGFLAG != 3 behaviour, returning at the first pivot <= 0
 * and leaving the later columns unfactored (solve.c:558-561, 608-611). */
static int sky_factor(long neq, const long *maxa, double *ss, double *ssd, int *det, int stop_nonpos)
{
    *det = 0;
    for (long n = 1; n <= neq; ++n) {
        long h = maxa[n] - maxa[n - 1] - 1; /* column height */
        long top = n - h;                   /* first row stored in column n */
        /* g(i,n) = a(i,n) - sum_{r} l(r,i) g(r,n), rows top+1 .. n-1 */
        for (long i = top + 1; i <= n - 1; ++i) {
            long hi = maxa[i] - maxa[i - 1] - 1;
            long topi = i - hi;
            long r0 = topi > top ? topi : top;
            if (r0 > i - 1) continue;
            double c = 0;
            for (long r = i - 1; r >= r0; --r) c += SKY(ss, maxa, r, i) * SKY(ss, maxa, r, n);
            SKY(ss, maxa, i, n) -= c;
        }
        /* l(i,n) = g(i,n)/d(i); d(n) = a(n,n) - sum l(i,n) g(i,n) */
        double b = 0;
        for (long i = n - 1; i >= top; --i) {
            double g = SKY(ss, maxa, i, n);
            double c = g / SKY(ss, maxa, i, i);
            b += c * g;
            SKY(ss, maxa, i, n) = c;
        }
        SKY(ss, maxa, n, n) -= b;
        double piv = SKY(ss, maxa, n, n);
        if (stop_nonpos) {
            if (!(piv > 0)) return 1;
            continue;
        }
        ssd[n - 1] = piv;
        if (piv == 0) return 1;
        if (!(piv > 0)) *det = 1;
    }
    return 0;
}

static void sky_solve(long neq, const long *maxa, const double *ss, double *v)
{
    for (long n = 1; n <= neq; ++n) {
        long h = maxa[n] - maxa[n - 1] - 1;
        double c = 0;
        for (long i = n - 1; i >= n - h; --i) c += SKY(ss, maxa, i, n) * v[i - 1];
        v[n - 1] -= c;
    }
    for (long n = 0; n < neq; ++n) v[n] /= ss[maxa[n] - 1];
    for (long n = neq; n >= 2; --n) {
        long h = maxa[n] - maxa[n - 1] - 1;
        for (long i = n - 1; i >= n - h; --i) v[i - 1] -= SKY(ss, maxa, i, n) * v[n - 1];
    }
}

void orc_skyline_solve(const orc_model *m, double *ss, double *rhs, double *ssd, int *det,
                       int fact)
{
    if (fact == 0) sky_factor(m->neq, m->maxa, ss, ssd, det, 0);
    else *det = 0;
    sky_solve(m->neq, m->maxa, ss, rhs);
}

/* ------------------------------------------------------------------------ */
/* quad (arc.c:70-157) and test (misc.c:187-250)                             */
/* ------------------------------------------------------------------------ */

int orc_quad(long neq, double a, double b, double c, double *dt, const double *dp,
             const double *ddr, const double *ddq, double *dd, double *dlpf, double *lpft)
{
    double rad = b * b - 4 * a * c;
    if (!(rad > 0)) return 2;
    double root[2] = {(-b + sqrt(b * b - 4 * a * c)) / (2 * a), (-b - sqrt(b * b - 4 * a * c)) / (2 * a)};
    double gam[2] = {0, 0};
    for (int k = 0; k < 2; ++k)
        for (long i = 0; i < neq; ++i) {
            double di = dt[i] - dp[i] + ddr[i] + root[k] * ddq[i];
            gam[k] += (dt[i] - dp[i]) * di;
        }
    int pick;
    if (gam[0] > gam[1] && gam[0] > 0) pick = 0;
    else if (gam[1] > gam[0] && gam[1] > 0) pick = 1;
    else return 3;
    for (long i = 0; i < neq; ++i) {
        double di = dt[i] - dp[i] + ddr[i] + root[pick] * ddq[i];
        dt[i] = di + dp[i];
        dd[i] = ddr[i] + root[pick] * ddq[i];
    }
    *dlpf = root[pick];
    *lpft += *dlpf;
    return 0;
}

int orc_test(long neq, const double *d_temp, const double *dd, const double *f_temp,
             const double *fp, const double *qtot, const double *f_ip, double intener1,
             int *convchk, double toldisp, double tolforc, double tolener)
{
    *convchk = 0;
    if (toldisp < 1) {
        double dl = vdot(neq, dd, dd), tot = vdot(neq, d_temp, d_temp);
        if (tot == 0) return 1;
        if (sqrt(dl) / sqrt(tot) > toldisp) *convchk += 10;
    }
    if (tolforc < 1) {
        double ui = 0, up = 0;
        for (long i = 0; i < neq; ++i) {
            ui += (qtot[i] - f_temp[i]) * (qtot[i] - f_temp[i]);
            up += (qtot[i] - fp[i]) * (qtot[i] - fp[i]);
        }
        if (up == 0) return 1;
        if (sqrt(ui) / sqrt(up) > tolforc) *convchk += 100;
    }
    if (tolener < 1) {
        double en = 0;
        for (long i = 0; i < neq; ++i) en += dd[i] * (qtot[i] - f_ip[i]);
        if (intener1 == 0) return 1;
        if (fabs(en / intener1) > tolener) *convchk += 1000;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MSAL driver (main.c:2158-3141)                                            */
/* ------------------------------------------------------------------------ */

typedef struct {
    /* per-element state: converged (c), previous iteration (ip), current (i) */
    double *sh_c_c, *sh_c_ip, *sh_c_i, *sh_a_c, *sh_a_ip, *sh_a_i;
    double *sh_ef_c, *sh_ef_ip, *sh_ef_i;
    double *tr_l_c, *tr_l_i, *tr_d_c, *tr_d_i, *tr_ef_c, *tr_ef_i;
    double *fr_c_c, *fr_c_ip, *fr_c_i, *fr_ef_c, *fr_ef_ip, *fr_ef_i, *fr_l_c, *fr_l_ip, *fr_l_i;
    double *fr_lref;  /* reference (undeformed) length used by the frame stiffness */
    double *x, *x_temp;
} state_t;

static void state_alloc(const orc_model *m, state_t *s)
{
    size_t E = (size_t)m->ne_sh + 1, T = (size_t)m->ne_tr + 1;
    s->sh_c_c = malloc(sizeof(double) * 9 * E);
    s->sh_c_ip = malloc(sizeof(double) * 9 * E);
    s->sh_c_i = malloc(sizeof(double) * 9 * E);
    s->sh_a_c = malloc(sizeof(double) * E);
    s->sh_a_ip = malloc(sizeof(double) * E);
    s->sh_a_i = malloc(sizeof(double) * E);
    s->sh_ef_c = calloc(18 * E, sizeof(double));
    s->sh_ef_ip = calloc(18 * E, sizeof(double));
    s->sh_ef_i = calloc(18 * E, sizeof(double));
    s->tr_l_c = malloc(sizeof(double) * T);
    s->tr_l_i = malloc(sizeof(double) * T);
    s->tr_d_c = malloc(sizeof(double) * 3 * T);
    s->tr_d_i = malloc(sizeof(double) * 3 * T);
    s->tr_ef_c = calloc(2 * T, sizeof(double));
    s->tr_ef_i = calloc(2 * T, sizeof(double));
    size_t F = (size_t)m->ne_fr + 1;
    s->fr_c_c = malloc(sizeof(double) * 9 * F);
    s->fr_c_ip = malloc(sizeof(double) * 9 * F);
    s->fr_c_i = malloc(sizeof(double) * 9 * F);
    s->fr_ef_c = calloc(14 * F, sizeof(double));
    s->fr_ef_ip = calloc(14 * F, sizeof(double));
    s->fr_ef_i = calloc(14 * F, sizeof(double));
    s->fr_l_c = malloc(sizeof(double) * F);
    s->fr_l_ip = malloc(sizeof(double) * F);
    s->fr_l_i = malloc(sizeof(double) * F);
    s->fr_lref = malloc(sizeof(double) * F);
    s->x = malloc(sizeof(double) * 3 * (size_t)m->nj);
    s->x_temp = malloc(sizeof(double) * 3 * (size_t)m->nj);
}

static void state_free(state_t *s)
{
    double **p[] = {&s->sh_c_c, &s->sh_c_ip, &s->sh_c_i, &s->sh_a_c, &s->sh_a_ip, &s->sh_a_i,
                    &s->sh_ef_c, &s->sh_ef_ip, &s->sh_ef_i, &s->tr_l_c, &s->tr_l_i, &s->tr_d_c,
                    &s->tr_d_i, &s->tr_ef_c, &s->tr_ef_i, &s->x, &s->x_temp, &s->fr_c_c, &s->fr_c_ip,
                    &s->fr_c_i, &s->fr_ef_c, &s->fr_ef_ip, &s->fr_ef_i, &s->fr_l_c, &s->fr_l_ip,
                    &s->fr_l_i, &s->fr_lref};
    for (size_t i = 0; i < sizeof p / sizeof p[0]; ++i) {
        free(*p[i]);
        *p[i] = NULL;
    }
}

/* updatc translation update (misc.c:82-93): x_temp += dd on free translations */
static void update_coords(const orc_model *m, double *x_temp, const double *dd)
{
    for (long i = 0; i < m->nj; ++i)
        for (int j = 0; j < 3; ++j) {
            long k = m->jcode[i * 7 + j];
            if (k) x_temp[i * 3 + j] += dd[k - 1];
        }
}

/* internal force of the whole model: updatc geometry + forces_tr + forces_sh */
static void internal_force(const orc_model *m, state_t *s, const double *dd, double *f)
{
    memset(f, 0, sizeof(double) * (size_t)m->neq);
    if (m->ne_tr) orc_truss_forces(m, s->x_temp, s->tr_l_i, s->tr_d_i, s->tr_ef_i, f);
    for (long e = 0; e < m->ne_fr; ++e) {
        double fe[14];
        frame_force_element(m, e, s->x_temp, dd, s->fr_c_ip + e * 9, s->fr_ef_ip + e * 14, s->fr_l_ip[e],
                            s->fr_lref[e], s->fr_c_i + e * 9, s->fr_l_i + e, s->fr_ef_i + e * 14, fe);
        for (int i = 0; i < 14; ++i) {
            long q = m->fr_mc[e * 14 + i];
            if (q) f[q - 1] += fe[i];
        }
    }
    for (long e = 0; e < m->ne_sh; ++e) {
        double fe[18];
        long mc[18];
        shell_force_element(m, e, s->x_temp, dd, s->sh_c_ip + e * 9, s->sh_ef_ip + e * 18,
                            s->sh_c_i + e * 9, s->sh_a_i + e, s->sh_ef_i + e * 18, fe);
        shell_mcode(m, e, mc);
        for (int i = 0; i < 18; ++i)
            if (mc[i]) f[mc[i] - 1] += fe[i];
    }
}

/* "ip <- i" after an iteration (main.c:2399-2428) */
static void advance_iteration(const orc_model *m, state_t *s)
{
    memcpy(s->sh_ef_ip, s->sh_ef_i, sizeof(double) * 18 * (size_t)m->ne_sh);
    memcpy(s->sh_c_ip, s->sh_c_i, sizeof(double) * 9 * (size_t)m->ne_sh);
    memcpy(s->sh_a_ip, s->sh_a_i, sizeof(double) * (size_t)m->ne_sh);
    memcpy(s->fr_ef_ip, s->fr_ef_i, sizeof(double) * 14 * (size_t)m->ne_fr);
    memcpy(s->fr_c_ip, s->fr_c_i, sizeof(double) * 9 * (size_t)m->ne_fr);
    memcpy(s->fr_l_ip, s->fr_l_i, sizeof(double) * (size_t)m->ne_fr);
}

/* "i, ip <- converged" at the start of an increment (main.c:2582-2623) */
static void reset_to_converged(const orc_model *m, state_t *s)
{
    memcpy(s->x_temp, s->x, sizeof(double) * 3 * (size_t)m->nj);
    size_t E = (size_t)m->ne_sh, T = (size_t)m->ne_tr;
    memcpy(s->sh_ef_i, s->sh_ef_c, sizeof(double) * 18 * E);
    memcpy(s->sh_ef_ip, s->sh_ef_c, sizeof(double) * 18 * E);
    memcpy(s->sh_c_i, s->sh_c_c, sizeof(double) * 9 * E);
    memcpy(s->sh_c_ip, s->sh_c_c, sizeof(double) * 9 * E);
    memcpy(s->sh_a_i, s->sh_a_c, sizeof(double) * E);
    memcpy(s->sh_a_ip, s->sh_a_c, sizeof(double) * E);
    memcpy(s->tr_ef_i, s->tr_ef_c, sizeof(double) * 2 * T);
    memcpy(s->tr_l_i, s->tr_l_c, sizeof(double) * T);
    memcpy(s->tr_d_i, s->tr_d_c, sizeof(double) * 3 * T);
    size_t F = (size_t)m->ne_fr;
    memcpy(s->fr_c_i, s->fr_c_c, sizeof(double) * 9 * F);
    memcpy(s->fr_c_ip, s->fr_c_c, sizeof(double) * 9 * F);
    memcpy(s->fr_ef_i, s->fr_ef_c, sizeof(double) * 14 * F);
    memcpy(s->fr_ef_ip, s->fr_ef_c, sizeof(double) * 14 * F);
    memcpy(s->fr_l_i, s->fr_l_c, sizeof(double) * F);
    memcpy(s->fr_l_ip, s->fr_l_c, sizeof(double) * F);
}

/* "converged <- i" when an increment is accepted (main.c:3060-3105) */
static void accept_state(const orc_model *m, state_t *s)
{
    memcpy(s->x, s->x_temp, sizeof(double) * 3 * (size_t)m->nj);
    size_t E = (size_t)m->ne_sh, T = (size_t)m->ne_tr;
    memcpy(s->sh_ef_c, s->sh_ef_i, sizeof(double) * 18 * E);
    memcpy(s->sh_c_c, s->sh_c_i, sizeof(double) * 9 * E);
    memcpy(s->sh_a_c, s->sh_a_i, sizeof(double) * E);
    memcpy(s->tr_ef_c, s->tr_ef_i, sizeof(double) * 2 * T);
    memcpy(s->tr_l_c, s->tr_l_i, sizeof(double) * T);
    memcpy(s->tr_d_c, s->tr_d_i, sizeof(double) * 3 * T);
    size_t F = (size_t)m->ne_fr;
    memcpy(s->fr_c_c, s->fr_c_i, sizeof(double) * 9 * F);
    memcpy(s->fr_ef_c, s->fr_ef_i, sizeof(double) * 14 * F);
    memcpy(s->fr_l_c, s->fr_l_i, sizeof(double) * F);
}

static double rel_residual(long neq, const double *q, double lpf, const double *f)
{
    double num = 0, den = 0;
    for (long i = 0; i < neq; ++i) {
        double qt = q[i] * lpf;
        num += (qt - f[i]) * (qt - f[i]);
        den += qt * qt;
    }
    return den > 0 ? sqrt(num / den) : 0;
}

int orc_msal(orc_model *m, int max_steps, double *lam, int *its, double *dout, double *res,
             char *err, int errlen)
{
    return orc_msal_timed(m, max_steps, lam, its, dout, res, NULL, err, errlen);
}

int orc_msal_timed(orc_model *m, int max_steps, double *lam, int *its, double *dout, double *res,
                   double *tstamp, char *err, int errlen)
{
    long N = m->neq;
    size_t nb = sizeof(double) * (size_t)(N + 1);
    double *d = calloc(1, nb), *dp = calloc(1, nb), *dpp = calloc(1, nb), *ddq = calloc(1, nb),
           *ddr = calloc(1, nb), *dd = calloc(1, nb), *d_temp = calloc(1, nb), *f = calloc(1, nb),
           *fp = calloc(1, nb), *f_ip = calloc(1, nb), *f_temp = calloc(1, nb), *r = calloc(1, nb),
           *qtot = calloc(1, nb), *ssd = calloc(1, nb), *ssd_o = calloc(1, nb),
           *ss = malloc(sizeof(double) * (size_t)m->lss);
    long *maxa = malloc(sizeof(long) * (size_t)(N + 1));
    const double *q = m->q;
    state_t s;
    state_alloc(m, &s);
    int nconv = 0, rc = 0, det = 0, convchk = 1;
    memcpy(s.x, m->x0, sizeof(double) * 3 * (size_t)m->nj);
    memcpy(s.sh_c_c, m->sh_c0, sizeof(double) * 9 * (size_t)m->ne_sh);
    memcpy(s.sh_a_c, m->sh_area0, sizeof(double) * (size_t)m->ne_sh);
    memcpy(s.tr_l_c, m->tr_len0, sizeof(double) * (size_t)m->ne_tr);
    memcpy(s.tr_d_c, m->tr_dir0, sizeof(double) * 3 * (size_t)m->ne_tr);
    memcpy(s.fr_c_c, m->fr_c0, sizeof(double) * 9 * (size_t)m->ne_fr);
    memcpy(s.fr_l_c, m->fr_len0, sizeof(double) * (size_t)m->ne_fr);
    memcpy(s.fr_lref, m->fr_len0, sizeof(double) * (size_t)m->ne_fr);
    reset_to_converged(m, &s);

    /* ---- first increment: displacement control at dkdof (main.c:2296-2560) ---- */
    tangent_all(m, s.x, s.sh_c_c, s.sh_a_c, s.tr_l_c, s.tr_d_c, s.tr_ef_c, s.fr_c_c, s.fr_ef_c, s.fr_l_c,
                s.fr_lref, ss);
    memcpy(ddq, q, sizeof(double) * (size_t)N);
    orc_skyline_solve(m, ss, ddq, ssd, &det, 0);
    double lpf = m->dk / ddq[m->dkdof];
    double intener1 = 0;
    for (long i = 0; i < N; ++i) {
        d[i] = dd[i] = lpf * ddq[i];
        intener1 += dd[i] * (lpf * q[i]);
        ssd_o[i] = ssd[i];
    }
    update_coords(m, s.x_temp, dd);
    internal_force(m, &s, dd, f);
    int itecnt = 1;
    advance_iteration(m, &s);
    do {
        for (long i = 0; i < N; ++i) {
            qtot[i] = q[i] * lpf;
            r[i] = qtot[i] - f[i];
        }
        memcpy(ddr, r, sizeof(double) * (size_t)N);
        orc_skyline_solve(m, ss, ddr, ssd, &det, 1);
        double dl = -ddr[m->dkdof] / ddq[m->dkdof];
        lpf += dl;
        for (long i = 0; i < N; ++i) {
            dd[i] = ddr[i] + dl * ddq[i];
            d[i] += dd[i];
            f_ip[i] = f[i];
        }
        update_coords(m, s.x_temp, dd);
        internal_force(m, &s, dd, f);
        if (orc_test(N, d, dd, f, fp, qtot, f_ip, intener1, &convchk, m->toldisp, m->tolforc,
                     m->tolener)) {
            set_err(err, errlen, "zero norm in the convergence test");
            rc = -1;
            goto done;
        }
        itecnt++;
        advance_iteration(m, &s);
    } while (convchk != 0 && itecnt <= m->itemax);
    if (convchk != 0) {
        set_err(err, errlen, "initially prescribed displacement too large");
        rc = -2;
        goto done;
    }
    accept_state(m, &s);
    if (nconv < max_steps) {
        lam[nconv] = lpf;
        its[nconv] = itecnt;
        if (dout) memcpy(dout + (size_t)nconv * N, d, sizeof(double) * (size_t)N);
        res[nconv] = rel_residual(N, q, lpf, f);
        if (tstamp) tstamp[nconv] = now_s();
        nconv++;
    }
    double dkc = fabs(d[m->dkdof]), lpfc = fabs(lpf);
    for (long i = 0; i < N; ++i) {
        dpp[i] = dp[i];
        dp[i] = d[i];
        fp[i] = f[i];
    }
    double lpfpp = 0, lpfp = lpf;
    reset_to_converged(m, &s);
    double dnorm = sqrt(vdot(N, dp, dp));
    double dnormallow = m->alpha * sqrt(vdot(N, dp, dp));
    double beta = sqrt((double)m->iteopt / (double)itecnt) * (dnormallow / dnorm);
    double psi = 1;
    for (long i = 0; i < N; ++i) {
        double tq = fabs(ssd[i] / ssd_o[i]);
        if (tq < psi) psi = tq;
    }
    double qq = vdot(N, q, q);

    /* ---- arc-length increments (main.c:2647-3134) ---- */
    int errchk2 = 0, subcnt = 0, imagcnt = 0, negcnt = 0;
    double arc = 0;
    while (lpfc <= m->lpfmax && dkc <= m->dkimax && nconv < max_steps) {
        memcpy(d_temp, d, sizeof(double) * (size_t)N);
        double lpf_temp = lpf;
        if (errchk2 == 0) {
            double dot = 0;
            for (long i = 0; i < N; ++i) dot += (dp[i] - dpp[i]) * (dp[i] - dpp[i]);
            arc = psi >= m->psi_thresh ? beta * sqrt(dot + (lpfp - lpfpp) * (lpfp - lpfpp))
                                       : beta * sqrt(dot);
        } else {
            reset_to_converged(m, &s);
            errchk2 = 0;
        }
        tangent_all(m, s.x, s.sh_c_c, s.sh_a_c, s.tr_l_c, s.tr_d_c, s.tr_ef_c, s.fr_c_c, s.fr_ef_c, s.fr_l_c,
                    s.fr_lref, ss);
        memcpy(ddq, q, sizeof(double) * (size_t)N);
        orc_skyline_solve(m, ss, ddq, ssd, &det, 0);
        double a = psi >= m->psi_thresh ? qq + vdot(N, ddq, ddq) : vdot(N, ddq, ddq);
        double dlpf = det == 0 ? arc * sqrt(1 / a) : -arc * sqrt(1 / a);
        lpf_temp += dlpf;
        intener1 = 0;
        for (long i = 0; i < N; ++i) {
            dd[i] = dlpf * ddq[i];
            d_temp[i] += dd[i];
            intener1 += dd[i] * (dlpf * q[i]);
        }
        update_coords(m, s.x_temp, dd);
        internal_force(m, &s, dd, f_temp);
        advance_iteration(m, &s);
        itecnt = 1;
        do {
            for (long i = 0; i < N; ++i) {
                qtot[i] = q[i] * lpf_temp;
                r[i] = qtot[i] - f_temp[i];
                f_ip[i] = f_temp[i];
            }
            memcpy(ddr, r, sizeof(double) * (size_t)N);
            orc_skyline_solve(m, ss, ddr, ssd, &det, 1);
            double b, c;
            if (psi >= m->psi_thresh) {
                b = 2 * (vdot(N, d_temp, ddq) - vdot(N, dp, ddq) + vdot(N, ddr, ddq) +
                         (lpf_temp - lpfp) * qq);
                c = 2 * (vdot(N, d_temp, ddr) - vdot(N, dp, ddr) - vdot(N, d_temp, dp)) +
                    vdot(N, d_temp, d_temp) + vdot(N, dp, dp) + vdot(N, ddr, ddr) +
                    (lpf_temp - lpfp) * (lpf_temp - lpfp) * qq - arc * arc;
            } else {
                b = 2 * (vdot(N, d_temp, ddq) - vdot(N, dp, ddq) + vdot(N, ddr, ddq));
                c = 2 * (vdot(N, d_temp, ddr) - vdot(N, dp, ddr) - vdot(N, d_temp, dp)) +
                    vdot(N, d_temp, d_temp) + vdot(N, dp, dp) + vdot(N, ddr, ddr) - arc * arc;
            }
            errchk2 = orc_quad(N, a, b, c, d_temp, dp, ddr, ddq, dd, &dlpf, &lpf_temp);
            if (errchk2 == 0) {
                update_coords(m, s.x_temp, dd);
                internal_force(m, &s, dd, f_temp);
                if (orc_test(N, d_temp, dd, f_temp, fp, qtot, f_ip, intener1, &convchk,
                             m->toldisp, m->tolforc, m->tolener)) {
                    set_err(err, errlen, "zero norm in the convergence test");
                    rc = -1;
                    goto done;
                }
                if (convchk == 0) {
                    dnorm = 0;
                    for (long i = 0; i < N; ++i) dnorm += (d_temp[i] - dp[i]) * (d_temp[i] - dp[i]);
                    dnorm = sqrt(dnorm);
                    if (dnorm > 100 * dnormallow) {
                        arc /= beta;
                        beta = dnormallow / dnorm;
                        arc *= beta;
                        memcpy(f_temp, f, sizeof(double) * (size_t)N);
                        errchk2 = 1;
                    }
                } else {
                    itecnt++;
                    if (itecnt > m->itemax) {
                        arc *= 0.5;
                        memcpy(f_temp, f, sizeof(double) * (size_t)N);
                        subcnt++;
                        errchk2 = 1;
                    }
                    advance_iteration(m, &s);
                }
            } else if (errchk2 == 2) {
                arc *= 0.5;
                memcpy(f_temp, f, sizeof(double) * (size_t)N);
                imagcnt++;
            } else if (errchk2 == 3) {
                arc *= 0.5;
                memcpy(f_temp, f, sizeof(double) * (size_t)N);
                negcnt++;
            }
        } while (convchk != 0 && errchk2 == 0 && subcnt <= m->submax && imagcnt <= m->imagmax &&
                 negcnt <= m->negmax);
        if (subcnt > m->submax || imagcnt > m->imagmax || negcnt > m->negmax) {
            set_err(err, errlen, "maximum allowable number of subdivisions exceeded");
            rc = -3;
            goto done;
        } else if (errchk2 == 0) {
            beta = sqrt((double)m->iteopt / (double)itecnt) * (dnormallow / dnorm);
            for (long i = 0; i < N; ++i) {
                dpp[i] = dp[i];
                d[i] = dp[i] = d_temp[i];
                f[i] = fp[i] = f_temp[i];
            }
            lpfpp = lpfp;
            lpf = lpfp = lpf_temp;
            accept_state(m, &s);
            dkc = fabs(d[m->dkdof]);
            lpfc = fabs(lpf);
            psi = 1;
            for (long i = 0; i < N; ++i) {
                double tq = fabs(ssd[i] / ssd_o[i]);
                if (tq < psi) psi = tq;
            }
            subcnt = imagcnt = negcnt = 0;
            lam[nconv] = lpf;
            its[nconv] = itecnt;
            if (dout) memcpy(dout + (size_t)nconv * N, d, sizeof(double) * (size_t)N);
            res[nconv] = rel_residual(N, q, lpf, f);
            if (tstamp) tstamp[nconv] = now_s();
            nconv++;
            /* No reset here: like the reference, the next increment's predictor
             * starts from the previous-iteration shell state (c_ip, ef_ip) that
             * the converged iteration left untouched (main.c:2987-3033 update
             * "ip" only on non-converged iterations; main.c:2655 skips the
             * reset when errchk2 == 0). */
        }
    }
done:
    state_free(&s);
    free(d);
    free(dp);
    free(dpp);
    free(ddq);
    free(ddr);
    free(dd);
    free(d_temp);
    free(f);
    free(fp);
    free(f_ip);
    free(f_temp);
    free(r);
    free(qtot);
    free(ssd);
    free(ssd_o);
    free(ss);
    free(maxa);
    return rc < 0 ? rc : nconv;
}

/* ------------------------------------------------------------------------ */
/* Nonlinear Newmark driver (main.c:3305-3960, solve.c:139-222, 469-533)     */
/* ------------------------------------------------------------------------ */

/* Runs the reference's ALGFLAG 5 time loop for frame-only models (SLVFLAG 0,
 * no prescribed motion, NBC = 0) and records, for each of the first
 * max_steps time steps k: time[k] = k dt, its[k] = the iteration count of the
 * accepted pass, d[k*NEQ ...] (may be NULL), res[k] = |dyn - f| / |dyn| with
 * dyn = qtot - M a (the dynamic equilibrium the convergence test judges).
 * Returns the number of steps recorded, or -(error code) with err set. */
/* Lumped shell mass (mass_sh, shell.c:1505-1592): Mtot = rho A t with the
 * face area from the coordinates x, Mtot/3 at each vertex's translations and
 * Mtot/3 t^2/12 at its rotations, added to sm[eq] element by element. */
static void shell_mass(const orc_model *m, const double *x, double *sm)
{
    for (long s = 0; s < m->ne_sh; ++s) {
        const double *p0 = x + m->sh_conn[s * 3] * 3, *p1 = x + m->sh_conn[s * 3 + 1] * 3,
                     *p2 = x + m->sh_conn[s * 3 + 2] * 3;
        double el12[3], el31[3], nrm[3];
        for (int k = 0; k < 3; ++k) {
            el31[k] = p2[k] - p0[k];
            el12[k] = p1[k] - p0[k];
        }
        cross3(el12, el31, nrm, 0);
        const double area = 0.5 * sqrt(dot3(nrm, nrm));
        const double t = m->sh_t[s], mtot = m->sh_dens[s] * area * t;
        const double mt = mtot / 3, mr = mtot / 3 * pow(t, 2) / 12;
        long mc[18];
        shell_mcode(m, s, mc);
        for (int i = 0; i < 18; ++i)
            if (mc[i]) sm[mc[i] - 1] += (i % 6) < 3 ? mt : mr;
    }
}

/* y = K x for the symmetric skyline K (skymult, solve.c:700-757): column n
 * holds K(n, n) at maxa[n-1] and the entries above it after; the upper
 * triangle's columns are applied from the last one, then the diagonal, then
 * the lower triangle row by row. */
static void sky_mult(long neq, const long *maxa, const double *ss, const double *x, double *y)
{
    for (long i = 0; i < neq; ++i) y[i] = 0;
    for (long n = neq; n >= 2; --n) {
        long k = n;
        for (long kk = maxa[n - 1] + 1; kk <= maxa[n] - 1; ++kk) {
            --k;
            y[k - 1] += ss[kk - 1] * x[n - 1];
        }
    }
    for (long n = 0; n < neq; ++n) y[n] += x[n] * ss[maxa[n] - 1];
    for (long n = neq; n >= 1; --n) {
        if (maxa[n] - 1 < maxa[n - 1] + 1) continue;
        long k = n;
        double c = 0;
        for (long kk = maxa[n - 1] + 1; kk <= maxa[n] - 1; ++kk) {
            --k;
            c += ss[kk - 1] * x[k - 1];
        }
        y[n - 1] += c;
    }
}

/* Linear Newmark (ANAFLAG 1, ALGFLAG 4; main.c:3143-3302 with the effective
 * stiffness of solve.c:139-222 and the time loop of solve.c:246-467, SLVFLAG
 * 0, no prescribed motion, no restart): the stiffness of the initial state
 * and the lumped mass are formed once, K_eff = K + a0 (1 - am) / (1 - af) M
 * is factored once, and every time step k solves
 *   K_eff u = p_k [+ af / (1 - af) p_(k-1)] + M_eff(u_m, v_m, a_m)
 *             [- af / (1 - af) K u_m]
 * followed by the Newmark kinematics. Writes per step the time k dt and u. */
int orc_linear_newmark(orc_model *m, long max_steps, double *time_out, double *dout, char *err, int errlen)
{
    if (m->alg != 4) {
        set_err(err, errlen, "model is not a linear Newmark model (ALGFLAG 4)");
        return -1;
    }
    long N = m->neq, F = m->ne_fr, NT = m->nsteps;
    if (NT != m->ntin) {
        set_err(err, errlen, "ttot/dt + 1 differs from the number of input time points");
        return -1;
    }
    size_t nb = sizeof(double) * (size_t)(N + 1);
    double *ss = malloc(sizeof(double) * (size_t)m->lss), *keff = malloc(sizeof(double) * (size_t)m->lss),
           *sm = calloc(1, nb), *ssd = calloc(1, nb), *um = calloc(1, nb), *vm = calloc(1, nb),
           *am = calloc(1, nb), *uc = calloc(1, nb), *vc = calloc(1, nb), *ac = calloc(1, nb),
           *reff = calloc(1, nb), *ku = calloc(1, nb), *ef0 = calloc((size_t)(14 * F + 1), sizeof(double));
    double alpham = 0, alphaf = 0;
    if (m->numopt == 1) {
        alpham = (2 * m->spectrds - 1) / (m->spectrds + 1);
        alphaf = m->spectrds / (m->spectrds + 1);
    } else if (m->numopt == 2) {
        alphaf = (1 - m->spectrds) / (1 + m->spectrds);
    } else if (m->numopt == 3) {
        alpham = (m->spectrds - 1) / (m->spectrds + 1);
    }
    const double alpha = pow(1 - alpham + alphaf, 2) / 4, delta = 0.5 - alpham + alphaf;
    const double dt = m->dt, dt_temp = 1 * dt;
    const double a0 = 1 / (alpha * pow(dt_temp, 2)), a2 = 1 / (alpha * dt_temp), a3 = 1 / (2 * alpha) - 1;
    const double a6 = (dt_temp) * (1 - delta), a7 = delta * (dt_temp);
    /* stiffness of the initial state (the element forces are zero, so the
     * geometric terms vanish: stiffe alone, as ANAFLAG 1 forms it) and the
     * lumped mass (mass_fr or mass_sh) */
    tangent_all(m, m->x0, m->sh_c0, m->sh_area0, NULL, NULL, NULL, m->fr_c0, ef0, m->fr_len0, m->fr_len0, ss);
    if (m->ne_fr) orc_frame_mass(m, m->x0, sm);
    if (m->ne_sh) shell_mass(m, m->x0, sm);
    memcpy(keff, ss, sizeof(double) * (size_t)m->lss);
    for (long i = 0; i < N; ++i) keff[m->maxa[i] - 1] += a0 * (1 - alpham) * sm[i] / (1 - alphaf);
    int det = 0;
    sky_factor(N, m->maxa, keff, ssd, &det, 1);
    memcpy(um, m->um0, nb - sizeof(double));
    memcpy(vm, m->vm0, nb - sizeof(double));
    memcpy(am, m->am0, nb - sizeof(double));
    const double *pq = m->pinpt;
    long k = 0;
    for (; k < NT && k < max_steps; ++k) {
        for (long i = 0; i < N; ++i) {
            const double meff = sm[i] * ((1 - alpham) * (um[i] * a0 + vm[i] * a2 + am[i] * a3) - alpham * am[i]) /
                                (1 - alphaf);
            reff[i] = k == 0 ? pq[i * NT + k] + meff
                             : pq[i * NT + k] + alphaf / (1 - alphaf) * pq[i * NT + k - 1] + meff;
        }
        if (alphaf != 0) {
            sky_mult(N, m->maxa, ss, um, ku);
            for (long i = 0; i < N; ++i) reff[i] -= alphaf / (1 - alphaf) * ku[i];
        }
        sky_solve(N, m->maxa, keff, reff);
        for (long i = 0; i < N; ++i) {
            uc[i] = reff[i];
            ac[i] = a0 * (uc[i] - um[i]) - a2 * vm[i] - a3 * am[i];
            vc[i] = vm[i] + a6 * am[i] + a7 * ac[i];
        }
        time_out[k] = k * dt;
        if (dout) memcpy(dout + (size_t)k * N, uc, sizeof(double) * (size_t)N);
        for (long i = 0; i < N; ++i) {
            um[i] = uc[i];
            vm[i] = vc[i];
            am[i] = ac[i];
        }
    }
    free(ss);
    free(keff);
    free(sm);
    free(ssd);
    free(um);
    free(vm);
    free(am);
    free(uc);
    free(vc);
    free(ac);
    free(reff);
    free(ku);
    free(ef0);
    return (int)k;
}

int orc_newmark(orc_model *m, long max_steps, double *time_out, int *its_out, double *dout,
                double *res_out, char *err, int errlen)
{
    if (m->alg != 5) {
        set_err(err, errlen, "model is not a nonlinear Newmark model (ALGFLAG 5)");
        return -1;
    }
    long N = m->neq, F = m->ne_fr, NT = m->nsteps;
    if (NT != m->ntin) {
        set_err(err, errlen, "ttot/dt + 1 differs from the number of input time points");
        return -1;
    }
    size_t nb = sizeof(double) * (size_t)(N + 1);
    double *d = calloc(1, nb), *f = calloc(1, nb), *d_temp = calloc(1, nb), *f_temp = calloc(1, nb),
           *fp = calloc(1, nb), *f_ip = calloc(1, nb), *dd = calloc(1, nb), *r = calloc(1, nb),
           *qtot = calloc(1, nb), *dyn = calloc(1, nb), *uc = calloc(1, nb), *vc = calloc(1, nb),
           *ac = calloc(1, nb), *uc_i = calloc(1, nb), *vc_i = calloc(1, nb), *ac_i = calloc(1, nb),
           *um = calloc(1, nb), *vm = calloc(1, nb), *am = calloc(1, nb), *sm = calloc(1, nb),
           *ssd = calloc(1, nb), *ss = malloc(sizeof(double) * (size_t)m->lss),
           *lt = malloc(sizeof(double) * (size_t)(F + 1));
    const double *pin = m->pinpt;
    state_t s;
    state_alloc(m, &s);
    int rc = 0, nrec = 0, det = 0;
    /* Newmark / HHT / WBZ parameters (main.c:3329-3343) */
    double alpham = 0, alphaf = 0;
    if (m->numopt == 1) {
        alpham = (2 * m->spectrds - 1) / (m->spectrds + 1);
        alphaf = m->spectrds / (m->spectrds + 1);
    } else if (m->numopt == 2) {
        alphaf = (1 - m->spectrds) / (1 + m->spectrds);
    } else if (m->numopt == 3) {
        alpham = (m->spectrds - 1) / (m->spectrds + 1);
    }
    const double alpha = pow(1 - alpham + alphaf, 2) / 4;
    const double delta = 0.5 - alpham + alphaf;
    const double dt = m->dt;
    double ddt = 1, sub_dt = 1, dt_temp = dt, tsflag = 0;
    const double lpfi = m->lpf0, dlpfi = m->dlpf0, lpfmax = m->lpfmax;
    double lpf = lpfi, dlpf = dlpfi, dlpfp = dlpf, intener1 = 0;
    int convchk = 1, itecnt = 0;
    /* initial state (main.c:3398-3447): zero motion, frame lengths L0 */
    memcpy(s.x, m->x0, sizeof(double) * 3 * (size_t)m->nj);
    memcpy(s.fr_c_c, m->fr_c0, sizeof(double) * 9 * (size_t)F);
    memcpy(s.fr_l_c, m->fr_len0, sizeof(double) * (size_t)F);
    memcpy(lt, m->fr_len0, sizeof(double) * (size_t)F);
    long k = 0;
    do {
        dt_temp = ddt * dt;
        sub_dt = ddt;
        tsflag = 0;
        do {
            const double a0 = 1 / (alpha * pow(dt_temp, 2));
            const double a2 = 1 / (alpha * dt_temp);
            const double a3 = 1 / (2 * alpha) - 1;
            const double a6 = (dt_temp) * (1 - delta);
            const double a7 = delta * (dt_temp);
            int solcnt = 0, subcnt = 0;
            lpf = lpfi;
            dlpf = dlpfi;
            do {
                if (lpf > lpfmax) lpf = lpfmax;
                for (long i = 0; i < N; ++i) {
                    fp[i] = f[i];
                    d_temp[i] = d[i];
                    f_temp[i] = f[i];
                }
                dlpfp = dlpf;
                reset_to_converged(m, &s);
                for (long i = 0; i < N; ++i) {
                    um[i] = uc_i[i] = uc[i];
                    vm[i] = vc_i[i] = vc[i];
                    am[i] = ac_i[i] = ac[i];
                }
                itecnt = 0;
                do {
                    if (itecnt == 0) {
                        if (k == 0) {
                            for (long i = 0; i < N; ++i) {
                                qtot[i] = pin[i * NT + k] * sub_dt * lpf;
                                r[i] = qtot[i] - f_temp[i];
                            }
                        } else {
                            for (long i = 0; i < N; ++i) {
                                qtot[i] = (pin[i * NT + k - 1] + (pin[i * NT + k] - pin[i * NT + k - 1]) * (sub_dt)) * lpf;
                                r[i] = (qtot[i] - f_temp[i]) + alphaf / (1 - alphaf) * (pin[i * NT + k - 1] - f_temp[i]);
                            }
                        }
                    } else {
                        for (long i = 0; i < N; ++i) {
                            r[i] = (f_temp[i] - qtot[i]);
                            r[i] = r[i] + sm[i] * ac_i[i] -
                                   sm[i] * ((a2 * vc_i[i] + a3 * ac_i[i]) * (1 - alpham) - ac_i[i] * alpham) /
                                       (1 - alphaf);
                        }
                    }
                    /* tangent from the previous iteration's state, lengths lt from
                     * the last mass_fr call; mass at the converged coordinates,
                     * which also rewrites lt (frame.c:1339) */
                    tangent_all(m, s.x, NULL, NULL, NULL, NULL, NULL, s.fr_c_ip, s.fr_ef_ip, s.fr_l_ip, lt, ss);
                    memset(sm, 0, nb);
                    for (long e = 0; e < F; ++e) {
                        double mt, mr;
                        lt[e] = frame_mass_element(m, e, s.x, &mt, &mr);
                        for (int i = 0; i < 14; ++i) {
                            long q = m->fr_mc[e * 14 + i];
                            int dof = i % 7;
                            if (q && dof < 6) sm[q - 1] += dof < 3 ? mt : mr;
                        }
                    }
                    if (m->lss == 1) {
                        dd[0] = r[0] / ss[0];
                    } else {
                        /* Keff = K + a0 (1 - am) / (1 - af) M on the diagonal
                         * (solve.c:203-210), factored every iteration */
                        for (long i = 0; i < N; ++i) ss[m->maxa[i] - 1] += a0 * (1 - alpham) * sm[i] / (1 - alphaf);
                        sky_factor(N, m->maxa, ss, ssd, &det, 1);
                        /* Reff (solve.c:478-487); inside solve the "m" vectors are
                         * the current uc_i, vc_i, ac_i */
                        for (long i = 0; i < N; ++i)
                            dd[i] = r[i] + sm[i] * ((1 - alpham) * (vc_i[i] * a2 + ac_i[i] * a3) - alpham * ac_i[i]) /
                                               (1 - alphaf);
                        sky_solve(N, m->maxa, ss, dd);
                    }
                    for (long i = 0; i < N; ++i) {
                        if (itecnt > 0) dd[i] = dd[i] * (-1);
                        d_temp[i] += dd[i];
                        f_ip[i] = f_temp[i];
                        f_temp[i] = 0;
                    }
                    for (long i = 0; i < N; ++i) {
                        uc_i[i] = d_temp[i];
                        ac_i[i] = (uc_i[i] - um[i]) * a0 - a2 * vm[i] - a3 * am[i];
                        vc_i[i] = vm[i] + a6 * am[i] + a7 * ac_i[i];
                    }
                    update_coords(m, s.x_temp, dd);
                    for (long e = 0; e < F; ++e) {
                        double fe[14];
                        frame_force_element(m, e, s.x_temp, dd, s.fr_c_ip + e * 9, s.fr_ef_ip + e * 14,
                                            s.fr_l_ip[e], lt[e], s.fr_c_i + e * 9, s.fr_l_i + e,
                                            s.fr_ef_i + e * 14, fe);
                        for (int i = 0; i < 14; ++i) {
                            long q = m->fr_mc[e * 14 + i];
                            if (q) f_temp[q - 1] += fe[i];
                        }
                    }
                    for (long i = 0; i < N; ++i) dyn[i] = qtot[i] - sm[i] * ac_i[i];
                    if (itecnt == 0) {
                        intener1 = 0;
                        for (long i = 0; i < N; ++i) intener1 += dd[i] * (dyn[i] - fp[i]);
                    }
                    if (orc_test(N, d_temp, dd, f_temp, fp, dyn, f_ip, intener1, &convchk, m->toldisp,
                                 m->tolforc, m->tolener)) {
                        set_err(err, errlen, "zero norm in the convergence test");
                        rc = -1;
                        goto done;
                    }
                    advance_iteration(m, &s);
                    itecnt++;
                } while (convchk != 0 && itecnt <= m->itemax);
                if (convchk != 0 && subcnt <= m->submax) {
                    if (lpf == lpfmax) break;
                    else if (dlpfp == m->dlpfmin) break;
                    dlpf = dlpfp / 2;
                    if (dlpf < m->dlpfmin) dlpf = m->dlpfmin;
                    lpf = lpf - dlpfp + dlpf;
                    subcnt++;
                    solcnt = 0;
                } else if (subcnt > m->submax) {
                    break;
                } else {
                    solcnt++;
                    subcnt = 0;
                    if (solcnt >= m->solmin) {
                        dlpf *= 2;
                        solcnt = 0;
                    }
                    lpf += dlpf;
                }
            } while (lpf <= lpfmax);
            if (convchk != 0) {
                ddt = ddt / 2;
                dt_temp = ddt * dt;
                if (tsflag == 0) sub_dt = ddt;
                else if (tsflag == 1) sub_dt = sub_dt - ddt;
            } else {
                memcpy(d, d_temp, nb);
                memcpy(f, f_temp, nb);
                memcpy(uc, uc_i, nb);
                memcpy(vc, vc_i, nb);
                memcpy(ac, ac_i, nb);
                accept_state(m, &s);
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
        if (convchk != 0) {
            set_err(err, errlen, "minimum time increment interval reached without convergence");
            rc = -2;
            goto done;
        }
        if (nrec < max_steps) {
            time_out[nrec] = (double)k * dt;
            its_out[nrec] = itecnt;
            if (dout) memcpy(dout + (size_t)nrec * N, d, sizeof(double) * (size_t)N);
            double num = 0, den = 0;
            for (long i = 0; i < N; ++i) {
                num += (dyn[i] - f[i]) * (dyn[i] - f[i]);
                den += dyn[i] * dyn[i];
            }
            res_out[nrec] = den > 0 ? sqrt(num / den) : 0;
            nrec++;
        }
        ++k;
    } while (k < NT && nrec < max_steps);
done:
    state_free(&s);
    double *bufs[] = {d, f, d_temp, f_temp, fp, f_ip, dd, r, qtot, dyn, uc, vc, ac, uc_i, vc_i, ac_i,
                      um, vm, am, sm, ssd, ss, lt};
    for (size_t i = 0; i < sizeof bufs / sizeof bufs[0]; ++i) free(bufs[i]);
    return rc < 0 ? rc : nrec;
}
