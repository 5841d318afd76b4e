// Element kernels: DKT shell and truss internal forces (FP64), element
// tangents (FP64 or FP32), and the deterministic gather assembly.
//
// Layout: per-element arrays are structure-of-arrays, value k of element e
// at [k*E + e], so a warp of consecutive elements reads contiguous memory.
// One thread owns one element: on GB300 the FP64 pipe (about 1/64 of the
// FP32 rate) bounds these kernels, and thread-per-element spends no FP64
// instruction on redundancy or cross-lane reduction.
#include <cuda_runtime.h>

#include "dkt.cuh"
#include "internal.hpp"

namespace cb {

namespace {

constexpr int kThreads = 128;

inline unsigned blocks_for(long n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

// Initial shell geometry, local coordinates and element stiffnesses
// (prop_sh shell.c:61-95, stiffe_m_sh, stiffe_b_sh), once per model.
// Lumped shell mass (mass_sh, shell.c:1505-1592), one thread per element:
// Mtot = rho A t with the face area from the coordinates x, Mtot/3 at each
// vertex's translations and Mtot/3 t^2/12 at its rotations, in the element
// force buffer's layout [k * E + e] (gathered into the equations like forces).
__global__ void shell_mass_kernel(DevShell s, const double *__restrict__ x, const double *__restrict__ dens,
                                  double *__restrict__ me, long E)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    double p[3][3];
    for (int a = 0; a < 3; ++a) {
        int n = s.conn[a * E + e];
        for (int m = 0; m < 3; ++m) p[a][m] = x[n * 3 + m];
    }
    double el12[3], el31[3];
    for (int m = 0; m < 3; ++m) {
        el31[m] = p[2][m] - p[0][m];
        el12[m] = p[1][m] - p[0][m];
    }
    const double n0 = el12[1] * el31[2] - el12[2] * el31[1], n1 = el12[2] * el31[0] - el12[0] * el31[2],
                 n2 = el12[0] * el31[1] - el12[1] * el31[0];
    const double area = 0.5 * sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    const double t = s.prop[2 * E + e], mtot = dens[e] * area * t;
    const double mt = mtot / 3, mr = mtot / 3 * (t * t) / 12;
    for (int k = 0; k < 18; ++k) me[k * E + e] = (k % 6) < 3 ? mt : mr;
}

__global__ void shell_setup_kernel(DevShell s, const double *__restrict__ x0, long E)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    double p[3][3];
    for (int a = 0; a < 3; ++a) {
        int n = s.conn[a * E + e];
        for (int m = 0; m < 3; ++m) p[a][m] = x0[n * 3 + m];
    }
    double c[9], area, slen[3], xl[3];
    shell_geometry(p[0], p[1], p[2], c, area, slen);
    shell_local(p[0], p[1], p[2], c, xl);
    double em = s.prop[e], nu = s.prop[E + e], t = s.prop[2 * E + e];
    double kem[36], keb[81];
    shell_kem(em, nu, t, area, xl, kem);
    shell_keb(em, nu, t, area, xl, slen, keb);
    for (int k = 0; k < 9; ++k) s.c_c[k * E + e] = c[k];
    s.a_c[e] = area;
    for (int k = 0; k < 3; ++k) s.xl[k * E + e] = xl[k];
    for (int k = 0; k < 36; ++k) s.kem[k * E + e] = kem[k];
    for (int k = 0; k < 81; ++k) s.keb[k * E + e] = keb[k];
}

// One DKT element of forces_sh, ANAFLAG 2 (shell.c:1728-1785, 2305-2397),
// with the shell part of updatc (misc.c:149-184) fused in front:
//   c_i, a_i   triad and area of the current coordinates x_t
//   dm         total local membrane displacement (mem_coord - initial)
//   ddb        incremental bending displacement in the previous frame c_ip
//   ef_i       = ke_m dm + R_i R_ip^T (ke_b ddb + ef_ip with membrane part zeroed)
//   fe         = T_i^T ef_i, the element's contribution to f
// FP64 work per element: about 400 FMA plus 4 sqrt and 9 divisions.
__global__ void __launch_bounds__(kThreads) shell_forces_kernel(DevShell s,
                                                                const double *__restrict__ x_t,
                                                                const double *__restrict__ dd,
                                                                double *__restrict__ fe, long E)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    double p[3][3];
    for (int a = 0; a < 3; ++a) {
        int n = s.conn[a * E + e];
        for (int m = 0; m < 3; ++m) p[a][m] = x_t[n * 3 + m];
    }
    double ci[9], area;
    shell_geometry(p[0], p[1], p[2], ci, area, (double *)nullptr);
    double xlc[3];
    shell_local(p[0], p[1], p[2], ci, xlc);
    const double dm2 = xlc[0] - s.xl[e], dm4 = xlc[1] - s.xl[E + e], dm5 = xlc[2] - s.xl[2 * E + e];
    double cip[9];
    for (int k = 0; k < 9; ++k) cip[k] = s.c_ip[k * E + e];
    // incremental bending displacements w, thx, thy per vertex (rows 2,3,4 of T_ip)
    double ddb[9];
    for (int a = 0; a < 3; ++a) {
        double u[6];
        for (int d = 0; d < 6; ++d) {
            int q = s.eq[(a * 6 + d) * E + e];
            u[d] = q >= 0 ? dd[q] : 0.0;
        }
        ddb[3 * a] = cip[6] * u[0] + cip[7] * u[1] + cip[8] * u[2];
        ddb[3 * a + 1] = cip[0] * u[3] + cip[1] * u[4] + cip[2] * u[5];
        ddb[3 * a + 2] = cip[3] * u[3] + cip[4] * u[4] + cip[5] * u[5];
    }
    // local element force: membrane part (u, v of each vertex) from ke_m dm,
    // bending increment (w, thx, thy) from ke_b ddb; dm has only entries 2, 4, 5
    double loc[18];
    const int mrow[6] = {0, 1, 6, 7, 12, 13};
    double eft[18];
    for (int k = 0; k < 18; ++k) eft[k] = 0.0;
    for (int i = 0; i < 6; ++i) {
        const double *km = s.kem + (long)(i * 6) * E + e;
        // sum over j of kem[i][j] dm[j]; entries 0, 1, 3 of dm are zero
        eft[mrow[i]] = km[2 * E] * dm2 + km[4 * E] * dm4 + km[5 * E] * dm5;
    }
    double def[18];
    for (int k = 0; k < 18; ++k) def[k] = 0.0;
    const int brow[9] = {2, 3, 4, 8, 9, 10, 14, 15, 16};
    for (int i = 0; i < 9; ++i) {
        const double *kb = s.keb + (long)(i * 9) * E + e;
        double v = 0.0;
#pragma unroll
        for (int j = 0; j < 9; ++j) v += kb[(long)j * E] * ddb[j];
        def[brow[i]] = v;
    }
    // previous element force with its membrane entries zeroed (shell.c:1773)
    for (int k = 0; k < 18; ++k) loc[k] = s.ef_ip[k * E + e];
    for (int i = 0; i < 6; ++i) loc[mrow[i]] = 0.0;
    // R_rel = R_i R_ip^T
    double Rr[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            Rr[r][c] = ci[r * 3] * cip[c * 3] + ci[r * 3 + 1] * cip[c * 3 + 1] + ci[r * 3 + 2] * cip[c * 3 + 2];
    double efi[18];
    for (int b = 0; b < 6; ++b)
        for (int r = 0; r < 3; ++r) {
            double v = Rr[r][0] * (def[3 * b] + loc[3 * b]) + Rr[r][1] * (def[3 * b + 1] + loc[3 * b + 1]) +
                       Rr[r][2] * (def[3 * b + 2] + loc[3 * b + 2]);
            efi[3 * b + r] = eft[3 * b + r] + v;
        }
    for (int k = 0; k < 9; ++k) s.c_i[k * E + e] = ci[k];
    s.a_i[e] = area;
    for (int k = 0; k < 18; ++k) s.ef_i[k * E + e] = efi[k];
    for (int b = 0; b < 6; ++b)
        for (int c = 0; c < 3; ++c)
            fe[(3 * b + c) * E + e] = ci[c] * efi[3 * b] + ci[3 + c] * efi[3 * b + 1] + ci[6 + c] * efi[3 * b + 2];
}

// Truss geometry update (misc.c:95-107) and axial force (truss.c:326-375):
// N = EA (eps + eps^2/2) L/L0; the element adds -N c to end 1 and +N c to end 2.
__global__ void truss_forces_kernel(DevTruss t, const double *__restrict__ x_t,
                                    double *__restrict__ fe, long T)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= T) return;
    int na = t.conn[e], nb = t.conn[T + e];
    double el[3] = {x_t[nb * 3] - x_t[na * 3], x_t[nb * 3 + 1] - x_t[na * 3 + 1],
                    x_t[nb * 3 + 2] - x_t[na * 3 + 2]};
    double L = sqrt(dot3(el, el));
    double c[3] = {el[0] / L, el[1] / L, el[2] / L};
    double L0 = t.len0[e];
    double eps = (L - L0) / L0;
    double N = t.ea[e] * (eps + 0.5 * (eps * eps)) * L / L0;
    t.len_i[e] = L;
    for (int d = 0; d < 3; ++d) t.dir_i[d * T + e] = c[d];
    t.n_i[e] = N;
    for (int d = 0; d < 3; ++d) {
        fe[d * T + e] = -(N * c[d]);
        fe[(3 + d) * T + e] = -((-N) * c[d]);
    }
}

__device__ __forceinline__ int packed_idx(int ie, int je, int nd) { return ie * nd - ie * (ie - 1) / 2 + (je - ie); }

// Element tangent of the DKT shell (stiff_sh shell.c:110-344 with
// stiffe_sh shell.c:346-485 and stiffg_sh shell.c:660-840) in precision T:
// local k = ke (membrane, bending, drilling = ke_b[ii]/1e4) + kg (membrane
// force of the converged state), rotated block by block, K_ab = R^T k_ab R,
// and written as a packed upper triangle (171 values).
template <typename T>
__global__ void __launch_bounds__(kThreads) shell_tangent_kernel(DevShell s,
                                                                 const double *__restrict__ x_c,
                                                                 T *__restrict__ kel, long E)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    double pd[3][3];
    for (int a = 0; a < 3; ++a) {
        int n = s.conn[a * E + e];
        for (int m = 0; m < 3; ++m) pd[a][m] = x_c[n * 3 + m];
    }
    T R[9];
    for (int k = 0; k < 9; ++k) R[k] = (T)s.c_c[k * E + e];
    // membrane force of the converged configuration (stiffg_sh): Nm = t C B(A_c) dm
    double Rd[9];
    for (int k = 0; k < 9; ++k) Rd[k] = s.c_c[k * E + e];
    double xlc[3];
    shell_local(pd[0], pd[1], pd[2], Rd, xlc);
    const double xl0 = s.xl[e], xl1 = s.xl[E + e], xl2 = s.xl[2 * E + e];
    const double xld[3] = {xl0, xl1, xl2};
    const double dm[6] = {0, 0, xlc[0] - xl0, 0, xlc[1] - xl1, xlc[2] - xl2};
    double Cm[3][3], Bm[3][6];
    const double ac = s.a_c[e];
    plane_stress(s.prop[e], s.prop[E + e], Cm);
    membrane_b(xld, ac, Bm);
    double Nm[3];
    for (int i = 0; i < 3; ++i) {
        double sum = 0;
        for (int j = 0; j < 6; ++j) {
            double cb = Cm[i][0] * Bm[0][j] + Cm[i][1] * Bm[1][j] + Cm[i][2] * Bm[2][j];
            sum += cb * dm[j];
        }
        Nm[i] = s.prop[2 * E + e] * sum;
    }
    const double a2 = 2 * ac;
    const double bx[3] = {-(xl2 / a2), xl2 / a2, 0.0};
    const double by[3] = {(xl1 - xl0) / a2, -(xl1 / a2), xl0 / a2};
    double G[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double t0 = bx[a] * Nm[0] + by[a] * Nm[2];
            double t1 = bx[a] * Nm[2] + by[a] * Nm[1];
            G[a][b] = ac * (t0 * bx[b] + t1 * by[b]);
        }
    // local entry k(l, l') for l = 6*vertex + component (u, v, w, thx, thy, thz)
    auto kloc = [&](int l, int lp) -> T {
        int va = l / 6, ca = l % 6, vb = lp / 6, cbb = lp % 6;
        double v = 0.0;
        bool any = false;
        if (ca < 2 && cbb < 2) {
            v = s.kem[(long)((2 * va + ca) * 6 + (2 * vb + cbb)) * E + e];
            any = true;
        } else if (ca >= 2 && ca <= 4 && cbb >= 2 && cbb <= 4) {
            v = s.keb[(long)((3 * va + ca - 2) * 9 + (3 * vb + cbb - 2)) * E + e];
            any = true;
        } else if (ca == 5 && cbb == 5 && va == vb) {
            v = s.keb[(long)((3 * va + 1) * 9 + (3 * va + 1)) * E + e] / 10000;
            any = true;
        }
        if (ca < 3 && ca == cbb) v = any ? v + G[va][vb] : G[va][vb];
        return (T)v;
    };
    for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b) {
            T k[3][3];
            for (int r = 0; r < 3; ++r)
                for (int q = 0; q < 3; ++q) k[r][q] = kloc(3 * a + r, 3 * b + q);
            T tmp[3][3];
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) tmp[p][q] = R[p] * k[0][q] + R[3 + p] * k[1][q] + R[6 + p] * k[2][q];
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) {
                    int ie = 3 * a + p, je = 3 * b + q;
                    if (ie > je) continue;
                    T v = tmp[p][0] * R[q] + tmp[p][1] * R[3 + q] + tmp[p][2] * R[6 + q];
                    kel[(long)packed_idx(ie, je, 18) * E + e] = v;
                }
        }
}

// Truss tangent (stiff_tr truss.c:100-166): T^T k T with k = EA L^2/L0^3
// [[1,-1],[-1,1]], plus N/L on the translational diagonal and -N/L between
// the ends; packed upper triangle (21 values).
template <typename T>
__global__ void truss_tangent_kernel(DevTruss t, T *__restrict__ kel, long NT)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= NT) return;
    double L = t.len_c[e], L0 = t.len0[e];
    double kax = t.ea[e] * (L * L) / (L0 * L0 * L0);
    double c[3] = {t.dir_c[e], t.dir_c[NT + e], t.dir_c[2 * NT + e]};
    double g = t.n_c[e] / L;
    for (int je = 0; je < 6; ++je)
        for (int ie = 0; ie <= je; ++ie) {
            double tk = ie < 3 ? c[ie] * kax : c[ie - 3] * -kax;
            double tk2 = ie < 3 ? c[ie] * -kax : c[ie - 3] * kax;
            double v = je < 3 ? tk * c[je] : tk2 * c[je - 3];
            if (ie == je) v += g;
            if (je == ie + 3) v -= g;
            kel[(long)packed_idx(ie, je, 6) * NT + e] = (T)v;
        }
}

__global__ void gather_f64_kernel(const int *__restrict__ ptr, const int *__restrict__ src,
                                  const double *__restrict__ in, double *__restrict__ out, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += in[src[k]];
    out[i] = s;
}

template <typename T>
__global__ void gather_band_kernel(const int *__restrict__ ptr, const int *__restrict__ src,
                                   const int64_t *__restrict__ dst, const T *__restrict__ in,
                                   T *__restrict__ band, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    T s = 0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += in[src[k]];
    band[dst[i]] = s;
}

__global__ void update_coords_kernel(const int *__restrict__ eq_x, const double *__restrict__ dd,
                                     double *__restrict__ x_t, long neq)
{
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= neq) return;
    int xi = eq_x[q];
    if (xi >= 0) x_t[xi] += dd[q];
}

}  // namespace

void launch_shell_mass(const DevShell &s, const double *x, const double *dens, double *me, long ne,
                       cudaStream_t st)
{
    if (ne > 0) shell_mass_kernel<<<blocks_for(ne), kThreads, 0, st>>>(s, x, dens, me, ne);
}
void launch_shell_setup(const DevShell &s, const double *x0, long ne, cudaStream_t st)
{
    if (ne > 0) shell_setup_kernel<<<blocks_for(ne, 64), 64, 0, st>>>(s, x0, ne);
}
void launch_shell_forces(const DevShell &s, const double *x_t, const double *dd, double *fe, long ne,
                         cudaStream_t st)
{
    if (ne > 0) shell_forces_kernel<<<blocks_for(ne), kThreads, 0, st>>>(s, x_t, dd, fe, ne);
}
void launch_truss_forces(const DevTruss &t, const double *x_t, double *fe, long nt, cudaStream_t st)
{
    if (nt > 0) truss_forces_kernel<<<blocks_for(nt), kThreads, 0, st>>>(t, x_t, fe, nt);
}
template <typename T>
void launch_shell_tangent(const DevShell &s, const double *x_c, T *kel, long ne, cudaStream_t st)
{
    if (ne > 0) shell_tangent_kernel<T><<<blocks_for(ne), kThreads, 0, st>>>(s, x_c, kel, ne);
}
template <typename T>
void launch_truss_tangent(const DevTruss &t, T *kel, long nt, cudaStream_t st)
{
    if (nt > 0) truss_tangent_kernel<T><<<blocks_for(nt), kThreads, 0, st>>>(t, kel, nt);
}
void launch_gather_f64(const int *ptr, const int *src, const double *in, double *out, long n,
                       cudaStream_t st)
{
    if (n > 0) gather_f64_kernel<<<blocks_for(n, 256), 256, 0, st>>>(ptr, src, in, out, n);
}
template <typename T>
void launch_gather_band(const int *ptr, const int *src, const int64_t *dst, const T *in, T *band,
                        long nslots, cudaStream_t st)
{
    if (nslots > 0)
        gather_band_kernel<T><<<blocks_for(nslots, 256), 256, 0, st>>>(ptr, src, dst, in, band, nslots);
}
void launch_update_coords(const int *eq_x, const double *dd, double *x_t, long neq, cudaStream_t st)
{
    update_coords_kernel<<<blocks_for(neq, 256), 256, 0, st>>>(eq_x, dd, x_t, neq);
}

template void launch_shell_tangent<double>(const DevShell &, const double *, double *, long, cudaStream_t);
template void launch_shell_tangent<float>(const DevShell &, const double *, float *, long, cudaStream_t);
template void launch_truss_tangent<double>(const DevTruss &, double *, long, cudaStream_t);
template void launch_truss_tangent<float>(const DevTruss &, float *, long, cudaStream_t);
template void launch_gather_band<double>(const int *, const int *, const int64_t *, const double *,
                                         double *, long, cudaStream_t);
template void launch_gather_band<float>(const int *, const int *, const int64_t *, const float *,
                                        float *, long, cudaStream_t);

}  // namespace cb
