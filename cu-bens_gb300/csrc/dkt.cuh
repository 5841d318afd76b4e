// Element mathematics of the co-rotational truss and DKT shell, shared by the
// setup, internal-force and tangent kernels. Everything is written for one
// element held in registers; T is double or float.
//
// Reference formulas restated here:
//   shell geometry and triad      prop_sh shell.c:61-91, updatc misc.c:149-184
//   local membrane coordinates    mem_coord shell.c:2402-2446
//   CST membrane stiffness        stiffe_m_sh shell.c:487-531
//   explicit DKT bending          stiffe_b_sh shell.c:533-658 (Batoz 1982)
//   membrane geometric stiffness  stiffg_sh shell.c:660-840
//   truss force / stiffness       forces_tr truss.c:326-375, stiff_tr truss.c:100-166
#pragma once

#include <cuda_runtime.h>

#ifndef CB_HD
#define CB_HD __host__ __device__ __forceinline__
#endif

namespace cb {

template <typename T>
CB_HD T dot3(const T *a, const T *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Side lengths (l12, l23, l31), face area and triad c (rows x^, y^, z^) of a
// triangle: x^ along edge 1-2, z^ along (p2-p1) x (p3-p1), y^ = z^ x x^.
template <typename T>
CB_HD void shell_geometry(const T *p1, const T *p2, const T *p3, T *c, T &area, T *slen)
{
    T e12[3], e23[3], e31[3], n[3];
    for (int m = 0; m < 3; ++m) {
        e23[m] = p3[m] - p2[m];
        e31[m] = p3[m] - p1[m];
        e12[m] = p2[m] - p1[m];
    }
    T l12 = sqrt(dot3(e12, e12));
    if (slen) {
        slen[0] = l12;
        slen[1] = sqrt(dot3(e23, e23));
        slen[2] = sqrt(dot3(e31, e31));
    }
    n[0] = e12[1] * e31[2] - e12[2] * e31[1];
    n[1] = e12[2] * e31[0] - e12[0] * e31[2];
    n[2] = e12[0] * e31[1] - e12[1] * e31[0];
    T a = T(0.5) * sqrt(dot3(n, n));
    area = a;
    T lz[3], lx[3];
    for (int m = 0; m < 3; ++m) {
        lx[m] = e12[m] / l12;
        lz[m] = n[m] / (2 * a);
    }
    T ly[3] = {lz[1] * lx[2] - lz[2] * lx[1], lz[2] * lx[0] - lz[0] * lx[2],
               lz[0] * lx[1] - lz[1] * lx[0]};
    T ll = sqrt(dot3(ly, ly));
    for (int m = 0; m < 3; ++m) {
        c[m] = lx[m];
        c[3 + m] = ly[m] / ll;
        c[6 + m] = lz[m];
    }
}

// Local membrane coordinates (x2, x3, y3) with vertex 1 at the origin.
template <typename T>
CB_HD void shell_local(const T *p1, const T *p2, const T *p3, const T *c, T *xl)
{
    T X2[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    T X3[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    xl[0] = c[0] * X2[0] + c[1] * X2[1] + c[2] * X2[2];
    xl[1] = c[0] * X3[0] + c[1] * X3[1] + c[2] * X3[2];
    xl[2] = c[3] * X3[0] + c[4] * X3[1] + c[5] * X3[2];
}

template <typename T>
CB_HD void plane_stress(T e, T nu, T C[3][3])
{
    T f = e / (1 - nu * nu);
    C[0][2] = C[1][2] = C[2][0] = C[2][1] = 0;
    C[0][0] = C[1][1] = f;
    C[0][1] = C[1][0] = f * nu;
    C[2][2] = f * (1 - nu) / 2;
}

// Strain-displacement matrix of the constant-strain triangle (u1 v1 u2 v2 u3 v3).
template <typename T>
CB_HD void membrane_b(const T *xl, T area, T B[3][6])
{
    T x2 = xl[0], x3 = xl[1], y3 = xl[2], a2 = 2 * area;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 6; ++j) B[i][j] = 0;
    B[0][0] = B[2][1] = -(y3 / a2);
    B[0][2] = B[2][3] = y3 / a2;
    B[1][1] = B[2][0] = (x3 - x2) / a2;
    B[1][3] = B[2][2] = -(x3 / a2);
    B[1][5] = B[2][4] = x2 / a2;
}

// kem = t A B^T C B (6x6, row-major)
template <typename T>
CB_HD void shell_kem(T e, T nu, T t, T area, const T *xl, T *kem)
{
    T C[3][3], B[3][6], BC[6][3];
    plane_stress(e, nu, C);
    membrane_b(xl, area, B);
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 3; ++j) BC[i][j] = B[0][i] * C[0][j] + B[1][i] * C[1][j] + B[2][i] * C[2][j];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j)
            kem[i * 6 + j] = t * area * (BC[i][0] * B[0][j] + BC[i][1] * B[1][j] + BC[i][2] * B[2][j]);
}

// Explicit DKT plate bending stiffness (9x9, row-major), w/thx/thy per vertex.
// keb = Q alpha^T / (2A); row k of aT is column k of Batoz's alpha matrix,
// written with the Batoz coefficients p4..p6, t4, t5, q4, q5, r4, r5.
template <typename T>
CB_HD void shell_keb(T e, T nu, T t, T area, const T *xl, const T *slen, T *keb)
{
    const T x2 = xl[0], x3 = xl[1], y3 = xl[2];
    const T D = e * t * t * t / (12 * (1 - nu * nu));
    const T E1 = D, E3 = D, E2 = D * nu, E4 = D * (1 - nu) / 2;
    const T x23 = x2 - x3;
    const T L12 = slen[0] * slen[0], L23 = slen[1] * slen[1], L31 = slen[2] * slen[2];
    const T p4 = -6 * x23 / L23, p5 = -6 * x3 / L31, p6 = 6 * x2 / L12;
    const T t4 = 6 * y3 / L23, t5 = -6 * y3 / L31;
    const T q4 = -3 * x23 * y3 / L23, q5 = 3 * x3 * y3 / L31;
    const T r4 = 3 * y3 * y3 / L23, r5 = 3 * y3 * y3 / L31;
    const T aT[9][9] = {
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
    T Q[9][9];
    for (int g = 0; g < 3; ++g) {
        for (int i = 3 * g; i < 3 * g + 3; ++i) {
            T b1 = 0, b2 = 0, b3 = 0;
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
            T s = 0;
            for (int k = 0; k < 9; ++k) s += Q[i][k] * aT[j][k];
            keb[i * 9 + j] = s / (2 * area);
        }
}

}  // namespace cb
