// FP64 vector algebra of the arc-length iteration, fused into few passes,
// with deterministic reductions (fixed grid, fixed summation order, no
// atomics) so that two runs give bit-identical results.
//
//   residual     r = lpf_temp q - f                      main.c:2845-2855
//   quad dots    the 9 dot products of b and c plus the  main.c:2873-2889
//                3 sums behind quad's gammas             arc.c:96-107
//   quad         root selection by the larger gamma      arc.c:70-157
//   update       dd, d_temp and the coordinate update    arc.c:111-124, misc.c:82-93
//   test         displacement / force / energy criteria  misc.c:187-250
#include <cuda_runtime.h>

#include "internal.hpp"

namespace cb {

namespace {

constexpr int kT = 256;

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-level reduction of K per-thread sums into partial[k*kRedBlocks + block].
template <int K>
__device__ __forceinline__ void block_partials(double (&acc)[K], double *partial)
{
    __shared__ double sm[K][kT / 32];
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double v = warp_sum(acc[k]);
        if (lane == 0) sm[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double s = 0;
        for (int w = 0; w < kT / 32; ++w) s += sm[threadIdx.x][w];
        partial[threadIdx.x * kRedBlocks + blockIdx.x] = s;
    }
}

// Warp k sums partial[k][*] (lane-strided, shuffle tree) into out[k].
template <int K>
__device__ __forceinline__ void finalize_partials(const double *partial, double *out)
{
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    if (warp < K) {
        double s = 0;
        for (int b = lane; b < kRedBlocks; b += 32) s += partial[warp * kRedBlocks + b];
        s = warp_sum(s);
        if (lane == 0) out[warp] = s;
    }
}

__global__ void residual_kernel(const double *__restrict__ q, const double *__restrict__ f,
                                double *__restrict__ r, MsalScalars *sc, long n)
{
    const double lam = sc->lam_t;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i == 0) sc->lam_old = lam;
    if (i < n) r[i] = q[i] * lam - f[i];
}

__global__ void __launch_bounds__(kT) quad_dots_kernel(const double *__restrict__ dt,
                                                       const double *__restrict__ dp,
                                                       const double *__restrict__ ddr,
                                                       const double *__restrict__ ddq,
                                                       double *partial, long n)
{
    double acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = 0;
    for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)kRedBlocks * kT) {
        double a = dt[i], p = dp[i], r = ddr[i], q = ddq[i], g = a - p;
        acc[0] += a * q;
        acc[1] += p * q;
        acc[2] += r * q;
        acc[3] += a * r;
        acc[4] += p * r;
        acc[5] += a * p;
        acc[6] += a * a;
        acc[7] += p * p;
        acc[8] += r * r;
        acc[9] += g * g;
        acc[10] += g * r;
        acc[11] += g * q;
    }
    block_partials<12>(acc, partial);
}

// quad (arc.c:70-157): b and c as main.c:2873-2889 form them, then the
// root whose displacement increment makes the larger positive angle
// measure gamma = (d_t - d_p).(d_t - d_p + ddr + root ddq).
__global__ void quad_kernel(const double *partial, MsalScalars *sc)
{
    __shared__ double d[12];
    finalize_partials<12>(partial, d);
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int k = 0; k < 12; ++k) sc->dots[k] = d[k];
    const double a = sc->a, arc = sc->arc, dl = sc->lam_t - sc->lamp, qq = sc->qq;
    double b, c;
    if (sc->psi_ge) {
        b = 2 * (d[0] - d[1] + d[2] + dl * qq);
        c = 2 * (d[3] - d[4] - d[5]) + d[6] + d[7] + d[8] + dl * dl * qq - arc * arc;
    } else {
        b = 2 * (d[0] - d[1] + d[2]);
        c = 2 * (d[3] - d[4] - d[5]) + d[6] + d[7] + d[8] - arc * arc;
    }
    sc->dots[12] = b;
    sc->dots[13] = c;
    double rad = b * b - 4 * a * c;
    if (!(rad > 0)) {
        sc->quad_status = 2;
        return;
    }
    double root1 = (-b + sqrt(b * b - 4 * a * c)) / (2 * a);
    double root2 = (-b - sqrt(b * b - 4 * a * c)) / (2 * a);
    double g1 = d[9] + d[10] + root1 * d[11];
    double g2 = d[9] + d[10] + root2 * d[11];
    if (g1 > g2 && g1 > 0) {
        sc->root = root1;
    } else if (g2 > g1 && g2 > 0) {
        sc->root = root2;
    } else {
        sc->quad_status = 3;
        return;
    }
    sc->quad_status = 0;
    sc->lam_t += sc->root;
}

__global__ void quad_update_kernel(const double *__restrict__ ddr, const double *__restrict__ ddq,
                                   const double *__restrict__ dp, double *__restrict__ dt,
                                   double *__restrict__ dd, const int *__restrict__ eq_x,
                                   double *__restrict__ x_t, const MsalScalars *sc, long n)
{
    if (sc->quad_status != 0) return;
    const double root = sc->root;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double p = dp[i];
    double d1 = dt[i] - p + ddr[i] + root * ddq[i];
    dt[i] = d1 + p;
    double inc = ddr[i] + root * ddq[i];
    dd[i] = inc;
    int xi = eq_x[i];
    if (xi >= 0) x_t[xi] += inc;
}

__global__ void __launch_bounds__(kT) test_dots_kernel(const double *__restrict__ dd,
                                                       const double *__restrict__ dt,
                                                       const double *__restrict__ dp,
                                                       const double *__restrict__ q,
                                                       const double *__restrict__ f,
                                                       const double *__restrict__ fp,
                                                       const double *__restrict__ fip,
                                                       const MsalScalars *sc, double *partial,
                                                       long n)
{
    const double lam = sc->lam_old;
    double acc[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) acc[k] = 0;
    for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)kRedBlocks * kT) {
        double qt = q[i] * lam, x = dd[i], t = dt[i];
        double r = qt - f[i], rp = qt - fp[i], g = t - dp[i];
        acc[0] += x * x;
        acc[1] += t * t;
        acc[2] += r * r;
        acc[3] += rp * rp;
        acc[4] += x * (qt - fip[i]);
        acc[5] += g * g;
        acc[6] += qt * qt;
    }
    block_partials<7>(acc, partial);
}

// test (misc.c:187-250)
__global__ void test_kernel(const double *partial, MsalScalars *sc)
{
    __shared__ double d[7];
    finalize_partials<7>(partial, d);
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int k = 0; k < 7; ++k) sc->dots[k] = d[k];
    if (sc->intener_first) {
        // first iteration of a Newton-Raphson increment: intener1 = dd . (qtot - fp), and fp
        // is f_ip then (main.c:1975-1981)
        sc->intener1 = d[4];
        sc->intener_first = 0;
    }
    int conv = 0, err = 0;
    if (sc->toldisp < 1) {
        if (d[1] != 0) {
            if (sqrt(d[0]) / sqrt(d[1]) > sc->toldisp) conv += 10;
        } else {
            err = 1;
        }
    }
    if (!err && sc->tolforc < 1) {
        if (d[3] != 0) {
            if (sqrt(d[2]) / sqrt(d[3]) > sc->tolforc) conv += 100;
        } else {
            err = 2;
        }
    }
    if (!err && sc->tolener < 1) {
        if (sc->intener1 != 0) {
            if (fabs(d[4] / sc->intener1) > sc->tolener) conv += 1000;
        } else {
            err = 3;
        }
    }
    sc->convchk = conv;
    sc->test_err = err;
}

__global__ void __launch_bounds__(kT) dot_kernel(const double *__restrict__ a,
                                                 const double *__restrict__ b, double *partial, long n,
                                                 int diff)
{
    double acc[1] = {0};
    for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)kRedBlocks * kT) {
        if (diff) {
            double g = a[i] - b[i];
            acc[0] += g * g;
        } else {
            acc[0] += a[i] * (b ? b[i] : a[i]);
        }
    }
    block_partials<1>(acc, partial);
}

__global__ void first_update_kernel(const double *__restrict__ ddr, const double *__restrict__ ddq,
                                    long kdof, double *__restrict__ d, double *__restrict__ dd,
                                    const int *__restrict__ eq_x, double *__restrict__ x_t,
                                    MsalScalars *sc, long n)
{
    const double dl = -ddr[kdof] / ddq[kdof];
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i == 0) {
        sc->root = dl;
        sc->lam_t = sc->lam_old + dl;
    }
    if (i >= n) return;
    double inc = ddr[i] + dl * ddq[i];
    dd[i] = inc;
    d[i] += inc;
    int xi = eq_x[i];
    if (xi >= 0) x_t[xi] += inc;
}

__global__ void __launch_bounds__(kT) psi_kernel(const double *__restrict__ ssd,
                                                 const double *__restrict__ ssd_o, double *partial, long n)
{
    __shared__ double sm[kT];
    double m = 1.0;
    for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)kRedBlocks * kT) {
        double t = fabs(ssd[i] / ssd_o[i]);
        if (t < m) m = t;
    }
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = fmin(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

__global__ void psi_final_kernel(const double *partial, MsalScalars *sc, int slot)
{
    if (threadIdx.x != 0) return;
    double m = 1.0;
    for (int b = 0; b < kRedBlocks; ++b) m = fmin(m, partial[b]);
    sc->dots[slot] = m;
}

__global__ void dot_final_kernel(const double *partial, MsalScalars *sc, int slot)
{
    __shared__ double d[1];
    finalize_partials<1>(partial, d);
    __syncthreads();
    if (threadIdx.x == 0) sc->dots[slot] = d[0];
}

__global__ void scale_kernel(const double *__restrict__ x, double alpha, double *__restrict__ y, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = alpha * x[i];
}

__global__ void axpy_kernel(const double *__restrict__ x, double alpha, double *__restrict__ y, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) y[i] += alpha * x[i];
}

// ---- nonlinear Newmark (main.c:3553-3588, 3639-3688; solve.c:203-210, 478-487) ----

// Residual of main.c:3553-3588 and the effective right-hand side Reff of
// solve.c:478-487 in one pass. mode 0: predictor of the first time step,
// 1: predictor of a later step (HHT load interpolation), 2: corrector. The
// reference passes uc_i, vc_i, ac_i as solve's "m" vectors, so Reff uses the
// current iteration's velocity and acceleration.
__global__ void nm_reff_kernel(int mode, double sub_dt, double lpf, double alpham, double alphaf, double a2,
                               double a3, const double *__restrict__ pin_km1, const double *__restrict__ pin_k,
                               const double *__restrict__ f_temp, const double *__restrict__ sm,
                               const double *__restrict__ vc_i, const double *__restrict__ ac_i,
                               double *__restrict__ qtot, double *__restrict__ reff, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double f = f_temp[i], m = sm[i], v = vc_i[i], a = ac_i[i];
    double r;
    if (mode == 0) {
        const double qt = pin_k[i] * sub_dt * lpf;
        qtot[i] = qt;
        r = qt - f;
    } else if (mode == 1) {
        const double pm = pin_km1[i];
        const double qt = (pm + (pin_k[i] - pm) * (sub_dt)) * lpf;
        qtot[i] = qt;
        r = (qt - f) + alphaf / (1 - alphaf) * (pm - f);
    } else {
        r = f - qtot[i];
        r = r + m * a - m * ((a2 * v + a3 * a) * (1 - alpham) - a * alpham) / (1 - alphaf);
    }
    reff[i] = r + m * ((1 - alpham) * (v * a2 + a * a3) - alpham * a) / (1 - alphaf);
}

// Keff = K + a0 (1 - alpha_m) / (1 - alpha_f) M on the band diagonal
// (solve.c:203-210); c0 = a0 (1 - alpha_m), den = 1 - alpha_f.
template <typename T>
__global__ void nm_keff_kernel(T *__restrict__ band, long ld, const double *__restrict__ sm, double c0,
                               double den, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double add = c0 * sm[i] / den;
    band[i * ld] = (T)((double)band[i * ld] + add);
}

// Linear Newmark effective load (solve.c:349-385; i-th equation):
// M_eff = sm ((1 - am)(um a0 + vm a2 + am a3) - am am) / (1 - af),
// reff = p_k + M_eff on the first step, p_k + af/(1-af) p_(k-1) + M_eff after,
// then reff -= af/(1-af) (K um) when af != 0 (nku holds -K um).
__global__ void lin_reff_kernel(int first, double alpham, double alphaf, double a0, double a2, double a3,
                                const double *__restrict__ pin_km1, const double *__restrict__ pin_k,
                                const double *__restrict__ sm, const double *__restrict__ um,
                                const double *__restrict__ vm, const double *__restrict__ am,
                                const double *__restrict__ nku, double *__restrict__ reff, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double meff = sm[i] * ((1 - alpham) * (um[i] * a0 + vm[i] * a2 + am[i] * a3) - alpham * am[i]) /
                        (1 - alphaf);
    const double c = alphaf / (1 - alphaf);
    double r = first ? pin_k[i] + meff : pin_k[i] + c * pin_km1[i] + meff;
    if (nku) r -= c * (-nku[i]);
    reff[i] = r;
}

// Linear Newmark kinematics (solve.c:434-452): ac, vc from the solution uc,
// then the step's motion becomes the previous one; d mirrors uc.
__global__ void lin_update_kernel(const double *__restrict__ uc, double *__restrict__ um, double *__restrict__ vm,
                                  double *__restrict__ am, double *__restrict__ vc, double *__restrict__ ac,
                                  double *__restrict__ d, double a0, double a2, double a3, double a6, double a7,
                                  long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double u = uc[i], uo = um[i], vo = vm[i], ao = am[i];
    const double a = a0 * (u - uo) - a2 * vo - a3 * ao;
    const double v = vo + a6 * ao + a7 * a;
    ac[i] = a;
    vc[i] = v;
    um[i] = u;
    vm[i] = v;
    am[i] = a;
    d[i] = u;
}

// dd sign (correctors solve for -dd, main.c:3625-3631), d_temp += dd, the
// Newmark kinematics of main.c:3634-3639 and x_temp += dd (updatc).
__global__ void nm_update_kernel(double *__restrict__ dd, int neg, double *__restrict__ d_temp,
                                 const double *__restrict__ um, const double *__restrict__ vm,
                                 const double *__restrict__ am, double *__restrict__ uc_i,
                                 double *__restrict__ vc_i, double *__restrict__ ac_i, double a0, double a2,
                                 double a3, double a6, double a7, const int *__restrict__ eq_x,
                                 double *__restrict__ x_t, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x = dd[i];
    if (neg) {
        x = x * (-1);
        dd[i] = x;
    }
    const double u = d_temp[i] + x;
    d_temp[i] = u;
    uc_i[i] = u;
    const double acc = (u - um[i]) * a0 - a2 * vm[i] - a3 * am[i];
    ac_i[i] = acc;
    vc_i[i] = vm[i] + a6 * am[i] + a7 * acc;
    const int xi = eq_x[i];
    if (xi >= 0) x_t[xi] += x;
}

// dyn = qtot - M a (main.c:3684-3688) and the sums of the convergence test
// with dyn as the external force: [0] dd.dd, [1] d.d, [2] |dyn - f|^2,
// [3] |dyn - fp|^2, [4] dd.(dyn - f_ip), [5] dd.(dyn - fp) (intener1 of the
// first iteration, main.c:3690-3696), [6] dyn.dyn
__global__ void __launch_bounds__(kT) nm_test_dots_kernel(const double *__restrict__ dd,
                                                          const double *__restrict__ dt,
                                                          const double *__restrict__ f,
                                                          const double *__restrict__ fp,
                                                          const double *__restrict__ fip,
                                                          const double *__restrict__ qtot,
                                                          const double *__restrict__ sm,
                                                          const double *__restrict__ ac_i,
                                                          double *__restrict__ dyn, double *partial, long n)
{
    double acc[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) acc[k] = 0;
    for (long i = blockIdx.x * (long)kT + threadIdx.x; i < n; i += (long)kRedBlocks * kT) {
        const double y = qtot[i] - sm[i] * ac_i[i];
        dyn[i] = y;
        const double x = dd[i], t = dt[i], r = y - f[i], rp = y - fp[i];
        acc[0] += x * x;
        acc[1] += t * t;
        acc[2] += r * r;
        acc[3] += rp * rp;
        acc[4] += x * (y - fip[i]);
        acc[5] += x * (y - fp[i]);
        acc[6] += y * y;
    }
    block_partials<7>(acc, partial);
}

__global__ void nm_test_kernel(const double *partial, MsalScalars *sc, int first)
{
    __shared__ double d[7];
    finalize_partials<7>(partial, d);
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int k = 0; k < 7; ++k) sc->dots[k] = d[k];
    if (first) sc->intener1 = d[5];
    int conv = 0, err = 0;
    if (sc->toldisp < 1) {
        if (d[1] != 0) {
            if (sqrt(d[0]) / sqrt(d[1]) > sc->toldisp) conv += 10;
        } else {
            err = 1;
        }
    }
    if (!err && sc->tolforc < 1) {
        if (d[3] != 0) {
            if (sqrt(d[2]) / sqrt(d[3]) > sc->tolforc) conv += 100;
        } else {
            err = 2;
        }
    }
    if (!err && sc->tolener < 1) {
        if (sc->intener1 != 0) {
            if (fabs(d[4] / sc->intener1) > sc->tolener) conv += 1000;
        } else {
            err = 3;
        }
    }
    sc->convchk = conv;
    sc->test_err = err;
}

inline unsigned nb(long n) { return (unsigned)((n + kT - 1) / kT); }

}  // namespace

void launch_residual(const double *q, const double *f, double *r, MsalScalars *sc, long n, cudaStream_t st)
{
    residual_kernel<<<nb(n), kT, 0, st>>>(q, f, r, sc, n);
}
void launch_quad_dots(const double *dt, const double *dp, const double *ddr, const double *ddq,
                      double *partial, MsalScalars *sc, long n, cudaStream_t st)
{
    quad_dots_kernel<<<kRedBlocks, kT, 0, st>>>(dt, dp, ddr, ddq, partial, n);
    (void)sc;
}
void launch_quad(const double *partial, MsalScalars *sc, cudaStream_t st)
{
    quad_kernel<<<1, 12 * 32, 0, st>>>(partial, sc);
}
void launch_quad_update(const double *ddr, const double *ddq, const double *dp, double *dt, double *dd,
                        const int *eq_x, double *x_t, const MsalScalars *sc, long n, cudaStream_t st)
{
    quad_update_kernel<<<nb(n), kT, 0, st>>>(ddr, ddq, dp, dt, dd, eq_x, x_t, sc, n);
}
void launch_test(const double *dd, const double *dt, const double *dp, const double *q, const double *f,
                 const double *fp, const double *fip, double *partial, MsalScalars *sc, long n,
                 cudaStream_t st)
{
    test_dots_kernel<<<kRedBlocks, kT, 0, st>>>(dd, dt, dp, q, f, fp, fip, sc, partial, n);
    test_kernel<<<1, 7 * 32, 0, st>>>(partial, sc);
}
void launch_dot(const double *a, const double *b, double *partial, MsalScalars *sc, int slot, long n,
                cudaStream_t st, bool diff)
{
    dot_kernel<<<kRedBlocks, kT, 0, st>>>(a, b, partial, n, diff ? 1 : 0);
    dot_final_kernel<<<1, 32, 0, st>>>(partial, sc, slot);
}
void launch_first_update(const double *ddr, const double *ddq, long kdof, double *d, double *dd,
                         const int *eq_x, double *x_t, MsalScalars *sc, long n, cudaStream_t st)
{
    first_update_kernel<<<nb(n), kT, 0, st>>>(ddr, ddq, kdof, d, dd, eq_x, x_t, sc, n);
}
void launch_psi(const double *ssd, const double *ssd_o, double *partial, MsalScalars *sc, int slot, long n,
                cudaStream_t st)
{
    psi_kernel<<<kRedBlocks, kT, 0, st>>>(ssd, ssd_o, partial, n);
    psi_final_kernel<<<1, 32, 0, st>>>(partial, sc, slot);
}
void launch_scale(const double *x, double alpha, double *y, long n, cudaStream_t st)
{
    scale_kernel<<<nb(n), kT, 0, st>>>(x, alpha, y, n);
}
void launch_axpy(const double *x, double alpha, double *y, long n, cudaStream_t st)
{
    axpy_kernel<<<nb(n), kT, 0, st>>>(x, alpha, y, n);
}

void launch_nm_reff(int mode, double sub_dt, double lpf, double alpham, double alphaf, double a2, double a3,
                    const double *pin_km1, const double *pin_k, const double *f_temp, const double *sm,
                    const double *vc_i, const double *ac_i, double *qtot, double *reff, long n, cudaStream_t st)
{
    nm_reff_kernel<<<nb(n), kT, 0, st>>>(mode, sub_dt, lpf, alpham, alphaf, a2, a3, pin_km1, pin_k, f_temp, sm,
                                         vc_i, ac_i, qtot, reff, n);
}
void launch_lin_reff(int first, double alpham, double alphaf, double a0, double a2, double a3,
                     const double *pin_km1, const double *pin_k, const double *sm, const double *um,
                     const double *vm, const double *am, const double *nku, double *reff, long n, cudaStream_t st)
{
    lin_reff_kernel<<<nb(n), kT, 0, st>>>(first, alpham, alphaf, a0, a2, a3, pin_km1, pin_k, sm, um, vm, am, nku,
                                           reff, n);
}
void launch_lin_update(const double *uc, double *um, double *vm, double *am, double *vc, double *ac, double *d,
                       double a0, double a2, double a3, double a6, double a7, long n, cudaStream_t st)
{
    lin_update_kernel<<<nb(n), kT, 0, st>>>(uc, um, vm, am, vc, ac, d, a0, a2, a3, a6, a7, n);
}
template <typename T>
void launch_nm_keff(T *band, long ld, const double *sm, double c0, double den, long n, cudaStream_t st)
{
    nm_keff_kernel<T><<<nb(n), kT, 0, st>>>(band, ld, sm, c0, den, n);
}
template void launch_nm_keff<float>(float *, long, const double *, double, double, long, cudaStream_t);
template void launch_nm_keff<double>(double *, long, const double *, double, double, long, cudaStream_t);
void launch_nm_update(double *dd, int neg, double *d_temp, const double *um, const double *vm, const double *am,
                      double *uc_i, double *vc_i, double *ac_i, double a0, double a2, double a3, double a6,
                      double a7, const int *eq_x, double *x_t, long n, cudaStream_t st)
{
    nm_update_kernel<<<nb(n), kT, 0, st>>>(dd, neg, d_temp, um, vm, am, uc_i, vc_i, ac_i, a0, a2, a3, a6, a7,
                                           eq_x, x_t, n);
}
void launch_nm_test(const double *dd, const double *dt, const double *f, const double *fp, const double *fip,
                    const double *qtot, const double *sm, const double *ac_i, double *dyn, double *partial,
                    MsalScalars *sc, int first, long n, cudaStream_t st)
{
    nm_test_dots_kernel<<<kRedBlocks, kT, 0, st>>>(dd, dt, f, fp, fip, qtot, sm, ac_i, dyn, partial, n);
    nm_test_kernel<<<1, 7 * 32, 0, st>>>(partial, sc, first);
}

}  // namespace cb
