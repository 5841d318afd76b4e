// Co-rotational 14-DOF frame members (7 per end: 3 translations, 3
// rotations, warping), ANAFLAG 2, on the GPU. One thread per member, FP64.
//
//   frame_geometry   triad and length from the end coordinates and the
//                    member's fixed auxiliary point: prop_fr frame.c:130-160,
//                    updatc misc.c:108-147
//   frame_klocal     ke (stiffe_fr, frame.c:364-408) + kg of the axial force
//                    and end moments (stiffg_fr, frame.c:410-579)
//   frame_forces     forces_fr (frame.c:902-1312): ef_i = T_i T_ip^T (ef_ip
//                    + k T_ip DD), element force T_i^T ef_i
//   frame_tangent    stiff_fr (frame.c:226-362): K = T^T k T, packed upper
//                    triangle K[ie][je], ie <= je
//   frame_mass       mass_fr (frame.c:1314-1391): lumped rho A L / 24 * 12 on
//                    translations and rho A L / 24 * L^2 on rotations, with L
//                    the member length at the given coordinates
//
// T is block diagonal (the triad on DOFs 0-2, 3-5, 7-9, 10-12 and 1 on the
// warping DOFs 6 and 13), so every product with T runs over the three
// non-zero terms of a block, in the order the full 14-term sums meet them.
//
// Algorithmic work per member and force evaluation: reads 2 joint indices,
// 14 equation numbers, 7 section constants, aux point, 6 coordinates, 14
// increments, c_ip 9, ef_ip 14, 2 lengths (~ 500 B); writes c_i 9, len_i,
// ef_i 14, 14 element forces (~ 300 B); about 1.2 kFLOP (k dl 196 FMA, the
// triad products 4 x 2 x 9 FMA, kg entries ~ 150).
#include <cuda_runtime.h>

#include "frame.cuh"
#include "internal.hpp"

namespace cb {

namespace {

constexpr int kFT = 128;

struct Section {
    double E, G, A, Iz, Iy, J, Iw;
};

__device__ __forceinline__ Section load_section(const double *prop, long e, long F)
{
    // prop rows: E, G, rho, A, I strong (z), I weak (y), J, I warping
    return Section{prop[e], prop[F + e], prop[3 * F + e], prop[4 * F + e], prop[5 * F + e],
                   prop[6 * F + e], prop[7 * F + e]};
}

#define KSYM(i, j, v)                  \
    do {                               \
        const double v_ = (v);         \
        k[i][j] += v_;                 \
        if ((i) != (j)) k[j][i] += v_; \
    } while (0)

// Local 14x14 stiffness: elastic part on the reference length L0, geometric
// part of the previous iteration's forces ef on the deformed length L.
__device__ void frame_klocal(const Section &s, double L0, const double *ef, double L, double k[14][14])
{
    const double E = s.E, G = s.G, A = s.A, Iz = s.Iz, Iy = s.Iy, J = s.J, Iw = s.Iw;
    for (int i = 0; i < 14; ++i)
        for (int j = 0; j < 14; ++j) k[i][j] = 0;
    const double L2 = pow(L0, 2), L3 = pow(L0, 3);
    k[0][0] = k[7][7] = E * A / L0;
    k[7][0] = k[0][7] = -k[0][0];
    k[1][1] = k[8][8] = 12 * E * Iz / L3;
    k[8][1] = k[1][8] = -k[1][1];
    k[2][2] = k[9][9] = 12 * E * Iy / L3;
    k[9][2] = k[2][9] = -k[2][2];
    k[3][3] = k[10][10] = 6 * G * J / (5 * L0) + 12 * E * Iw / L3;
    k[10][3] = k[3][10] = -k[3][3];
    k[5][5] = k[12][12] = 4 * E * Iz / L0;
    k[4][4] = k[11][11] = 4 * E * Iy / L0;
    k[6][6] = k[13][13] = 2 * G * J * L0 / 15 + 4 * E * Iw / L0;
    k[5][1] = k[1][5] = k[12][1] = k[1][12] = 6 * E * Iz / L2;
    k[8][5] = k[5][8] = k[12][8] = k[8][12] = -k[5][1];
    k[9][4] = k[4][9] = k[11][9] = k[9][11] = 6 * E * Iy / L2;
    k[4][2] = k[2][4] = k[11][2] = k[2][11] = -k[9][4];
    k[6][3] = k[3][6] = k[13][3] = k[3][13] = G * J / 10 + 6 * E * Iw / L2;
    k[10][6] = k[6][10] = k[13][10] = k[10][13] = -k[6][3];
    k[12][5] = k[5][12] = 2 * E * Iz / L0;
    k[11][4] = k[4][11] = 2 * E * Iy / L0;
    k[13][6] = k[6][13] = -(G * J * L0 / 30 - 2 * E * Iw / L0);
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

// first DOF of the 3x3 triad block that DOF i belongs to, or -1 (warping)
__device__ __forceinline__ int block_base(int i) { return i == 6 || i == 13 ? -1 : (i < 6 ? (i / 3) * 3 : 7 + ((i - 7) / 3) * 3); }

__global__ void __launch_bounds__(kFT) frame_geometry_kernel(DevFrame fr, const double *__restrict__ x,
                                                             double *__restrict__ c, double *__restrict__ len,
                                                             long F)
{
    long e = blockIdx.x * (long)kFT + threadIdx.x;
    if (e >= F) return;
    const int na = fr.conn[e], nb = fr.conn[F + e];
    double pa[3] = {x[na * 3], x[na * 3 + 1], x[na * 3 + 2]};
    double pb[3] = {x[nb * 3], x[nb * 3 + 1], x[nb * 3 + 2]};
    double aux[3] = {fr.aux[e], fr.aux[F + e], fr.aux[2 * F + e]};
    double cc[9], L;
    frame_geometry(pa, pb, aux, cc, &L);
    for (int k = 0; k < 9; ++k) c[k * F + e] = cc[k];
    len[e] = L;
}

// forces_fr for member e with the current triad ci given: ef_i, and the
// element force in global axes T_i^T ef_i into fe.
__device__ __forceinline__ void frame_force_member(const DevFrame &fr, long e, const double *ci,
                                                   const double *__restrict__ dd, const double *__restrict__ lref,
                                                   double *__restrict__ fe, long F)
{
    double cp[9], efp[14], DD[14];
    for (int k = 0; k < 9; ++k) cp[k] = fr.c_ip[k * F + e];
    for (int k = 0; k < 14; ++k) {
        efp[k] = fr.ef_ip[k * F + e];
        const int q = fr.eq[k * F + e];
        DD[k] = q >= 0 ? dd[q] : 0.0;
    }
    double k[14][14];
    frame_klocal(load_section(fr.prop, e, F), lref[e], efp, fr.len_ip[e], k);
    // dl = T_ip DD
    double dl[14];
    for (int i = 0; i < 14; ++i) {
        const int b = block_base(i);
        if (b < 0) {
            dl[i] = DD[i];
            continue;
        }
        const int r = i - b;
        double sum = 0;
        for (int q = 0; q < 3; ++q) sum += cp[r * 3 + q] * DD[b + q];
        dl[i] = sum;
    }
    // t = ef_ip + k dl
    double t[14];
    for (int i = 0; i < 14; ++i) {
        double sum = 0;
        for (int j = 0; j < 14; ++j) sum += k[i][j] * dl[j];
        t[i] = efp[i] + sum;
    }
    // R = c_i c_ip^T per block; ef_i = blockdiag(R, 1) t
    double R[9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double sum = 0;
            for (int q = 0; q < 3; ++q) sum += ci[a * 3 + q] * cp[b * 3 + q];
            R[a * 3 + b] = sum;
        }
    double efi[14];
    for (int i = 0; i < 14; ++i) {
        const int b = block_base(i);
        if (b < 0) {
            efi[i] = t[i];
            continue;
        }
        const int r = i - b;
        double sum = 0;
        for (int q = 0; q < 3; ++q) sum += R[r * 3 + q] * t[b + q];
        efi[i] = sum;
    }
    // element force in global axes: T_i^T ef_i
    for (int i = 0; i < 14; ++i) {
        const int b = block_base(i);
        double v;
        if (b < 0) {
            v = efi[i];
        } else {
            const int c = i - b;
            v = 0;
            for (int r = 0; r < 3; ++r) v += ci[r * 3 + c] * efi[b + r];
        }
        fe[(long)i * F + e] = v;
        fr.ef_i[(long)i * F + e] = efi[i];
    }
}

__global__ void __launch_bounds__(kFT) frame_forces_kernel(DevFrame fr, const double *__restrict__ x_t,
                                                           const double *__restrict__ dd,
                                                           const double *__restrict__ lref,
                                                           double *__restrict__ fe, long F)
{
    long e = blockIdx.x * (long)kFT + threadIdx.x;
    if (e >= F) return;
    const int na = fr.conn[e], nb = fr.conn[F + e];
    double pa[3] = {x_t[na * 3], x_t[na * 3 + 1], x_t[na * 3 + 2]};
    double pb[3] = {x_t[nb * 3], x_t[nb * 3 + 1], x_t[nb * 3 + 2]};
    double aux[3] = {fr.aux[e], fr.aux[F + e], fr.aux[2 * F + e]};
    double ci[9], Li;
    frame_geometry(pa, pb, aux, ci, &Li);
    frame_force_member(fr, e, ci, dd, lref, fe, F);
    for (int q = 0; q < 9; ++q) fr.c_i[q * F + e] = ci[q];
    fr.len_i[e] = Li;
}

// The same with the current triads given (c_i[q*F + e], as updatc formed them).
__global__ void __launch_bounds__(kFT) frame_forces_triads_kernel(DevFrame fr, const double *__restrict__ c_i,
                                                                  const double *__restrict__ dd,
                                                                  const double *__restrict__ lref,
                                                                  double *__restrict__ fe, long F)
{
    long e = blockIdx.x * (long)kFT + threadIdx.x;
    if (e >= F) return;
    double ci[9];
    for (int q = 0; q < 9; ++q) ci[q] = c_i[q * F + e];
    frame_force_member(fr, e, ci, dd, lref, fe, F);
}

// Tangent from the state (c, ef, len) with reference lengths lref; writes
// the 105 entries K[ie][je], ie <= je, at kel[p*F + e], p the packed index.
template <typename T>
__global__ void __launch_bounds__(kFT) frame_tangent_kernel(DevFrame fr, const double *__restrict__ c_s,
                                                            const double *__restrict__ ef_s,
                                                            const double *__restrict__ len_s,
                                                            const double *__restrict__ lref,
                                                            T *__restrict__ kel, long F)
{
    long e = blockIdx.x * (long)kFT + threadIdx.x;
    if (e >= F) return;
    double c[9], ef[14];
    for (int q = 0; q < 9; ++q) c[q] = c_s[q * F + e];
    for (int q = 0; q < 14; ++q) ef[q] = ef_s[q * F + e];
    double k[14][14];
    frame_klocal(load_section(fr.prop, e, F), lref[e], ef, len_s[e], k);
    const int bases[4] = {0, 3, 7, 10};
    // tmp = T^T k, in place by rows of each block
    for (int bi = 0; bi < 4; ++bi) {
        const int b = bases[bi];
        for (int j = 0; j < 14; ++j) {
            const double k0 = k[b][j], k1 = k[b + 1][j], k2 = k[b + 2][j];
            for (int i = 0; i < 3; ++i) k[b + i][j] = c[i] * k0 + c[3 + i] * k1 + c[6 + i] * k2;
        }
    }
    // K = tmp T, in place by columns of each block; store the upper triangle
    for (int bi = 0; bi < 4; ++bi) {
        const int b = bases[bi];
        for (int i = 0; i < 14; ++i) {
            const double t0 = k[i][b], t1 = k[i][b + 1], t2 = k[i][b + 2];
            for (int j = 0; j < 3; ++j) k[i][b + j] = t0 * c[j] + t1 * c[3 + j] + t2 * c[6 + j];
        }
    }
    int p = 0;
    for (int ie = 0; ie < 14; ++ie)
        for (int je = ie; je < 14; ++je, ++p) kel[(long)p * F + e] = (T)k[ie][je];
}

__global__ void __launch_bounds__(kFT) frame_mass_kernel(DevFrame fr, const double *__restrict__ x,
                                                         double *__restrict__ lt, double *__restrict__ me, long F)
{
    long e = blockIdx.x * (long)kFT + threadIdx.x;
    if (e >= F) return;
    const int na = fr.conn[e], nb = fr.conn[F + e];
    double el[3];
    for (int q = 0; q < 3; ++q) el[q] = x[nb * 3 + q] - x[na * 3 + q];
    const double L = sqrt(el[0] * el[0] + el[1] * el[1] + el[2] * el[2]);
    lt[e] = L;
    const double rAL = fr.prop[2 * F + e] * fr.prop[3 * F + e] * L;
    const double mt = rAL / 24 * 12, mr = rAL / 24 * pow(L, 2);
    for (int i = 0; i < 14; ++i) {
        const int d = i % 7;
        me[(long)i * F + e] = d < 3 ? mt : (d < 6 ? mr : 0.0);
    }
}

inline unsigned nblk(long n) { return (unsigned)((n + kFT - 1) / kFT); }

}  // namespace

void launch_frame_geometry(const DevFrame &fr, const double *x, double *c, double *len, long F, cudaStream_t st)
{
    if (F) frame_geometry_kernel<<<nblk(F), kFT, 0, st>>>(fr, x, c, len, F);
}

void launch_frame_forces(const DevFrame &fr, const double *x_t, const double *dd, const double *lref, double *fe,
                         long F, cudaStream_t st)
{
    if (F) frame_forces_kernel<<<nblk(F), kFT, 0, st>>>(fr, x_t, dd, lref, fe, F);
}

void launch_frame_forces_given_triads(const DevFrame &fr, const double *c_i, const double *dd, const double *lref,
                                      double *fe, long F, cudaStream_t st)
{
    if (F) frame_forces_triads_kernel<<<nblk(F), kFT, 0, st>>>(fr, c_i, dd, lref, fe, F);
}

template <typename T>
void launch_frame_tangent(const DevFrame &fr, const double *c, const double *ef, const double *len,
                          const double *lref, T *kel, long F, cudaStream_t st)
{
    if (F) frame_tangent_kernel<T><<<nblk(F), kFT, 0, st>>>(fr, c, ef, len, lref, kel, F);
}
template void launch_frame_tangent<float>(const DevFrame &, const double *, const double *, const double *,
                                          const double *, float *, long, cudaStream_t);
template void launch_frame_tangent<double>(const DevFrame &, const double *, const double *, const double *,
                                           const double *, double *, long, cudaStream_t);

void launch_frame_mass(const DevFrame &fr, const double *x, double *lt, double *me, long F, cudaStream_t st)
{
    if (F) frame_mass_kernel<<<nblk(F), kFT, 0, st>>>(fr, x, lt, me, F);
}

}  // namespace cb
