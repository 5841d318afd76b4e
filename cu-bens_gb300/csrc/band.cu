// Band LDL^T of the tangent stiffness and its block-bidiagonal solve.
//
// This replaces skyfact/skysolve (solve.c:539-698). The factorisation keeps
// the reference's equation order (no pivoting, no reordering), so the pivots
// ssd and the indefiniteness flag det that the MSAL driver reads
// (main.c:2636-2642, 2765-2769) are the reference's quantities.
//
// Storage: lower band, column-major, L(i,j) at band[j*ld + (i-j)] for
// 0 <= i-j <= bw; after factoring, the diagonal slots hold D and the rest
// the unit-lower L. The matrix is padded to npad = nblk*s equations with
// identity rows, s >= bw a multiple of 32.
//
// Factor: right-looking over 32-column panels (diagonal LDL^T in shared
// memory, panel TRSM, trailing rank-32 update inside the band).
//
// Solve: with s >= bw, L is block lower-bidiagonal in s x s blocks. The
// factor step also forms Linv_i = L_ii^-1, P_i = Linv_i L_{i,i-1} and
// R_i = L_{i+1,i} Linv_i, so that
//     y_i = Linv_i b_i - P_i y_{i-1}            (forward)
//     x_i = Linv_i^T (y_i / D_i) - R_i^T x_{i+1} (backward)
// and one solve is 2*nblk dense GEMV steps instead of a scalar
// substitution over every column.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "internal.hpp"

namespace cb {

namespace {

constexpr int NB = 32;  // panel width

#define CB_CUDA(x)                                                                         \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + \
                                     " at " __FILE__ ":" + std::to_string(__LINE__));      \
    } while (0)

// -------------------------------------------------------------------------
// Factor kernels
// -------------------------------------------------------------------------

// Dense LDL^T of the 32x32 diagonal block at column p, in shared memory.
template <typename T>
__global__ void __launch_bounds__(256) diag_factor_kernel(T *band, long ld, long bw, long p, long n,
                                                          T *dinv, double *ssd, int *flags)
{
    __shared__ T a[NB][NB + 1];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
        int i = idx / NB, j = idx % NB;
        T v = 0;
        if (i >= j && i - j <= bw) v = band[(p + j) * ld + (i - j)];
        a[i][j] = v;
    }
    __syncthreads();
    for (int k = 0; k < NB; ++k) {
        T d = a[k][k];
        // l_ik = a_ik / d_k for i > k
        __syncthreads();
        if (tid > k && tid < NB) a[tid][k] = a[tid][k] / d;
        __syncthreads();
        // a_ij -= l_ik d_k l_jk, k < j <= i
        for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
            int i = idx / NB, j = idx % NB;
            if (j > k && i >= j) a[i][j] -= a[i][k] * d * a[j][k];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
        int i = idx / NB, j = idx % NB;
        if (i >= j && i - j <= bw) band[(p + j) * ld + (i - j)] = a[i][j];
    }
    if (tid < NB) {
        T d = a[tid][tid];
        dinv[p + tid] = T(1) / d;
        long g = p + tid;
        if (g < n) {
            ssd[g] = (double)d;
            if (!(d > T(0))) atomicOr(&flags[0], 1);
            if (d == T(0)) atomicOr(&flags[1], 1);
        }
    }
}

// Panel TRSM: rows r in [p+32, p+32+m), L_rc = w_c / d_c with
// w_c = A_rc - sum_{k<c} w_k L_ck; the products W = L D are kept for the
// trailing update (wbuf, column-major in the panel column).
template <typename T>
__global__ void __launch_bounds__(64) panel_trsm_kernel(T *band, long ld, long bw, long p, long m,
                                                        const T *dinv, T *wbuf)
{
    __shared__ T l[NB][NB + 1];
    __shared__ T di[NB];
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
        int i = idx / NB, j = idx % NB;
        l[i][j] = (i > j && i - j <= bw) ? band[(p + j) * ld + (i - j)] : T(0);
    }
    if (threadIdx.x < NB) di[threadIdx.x] = dinv[p + threadIdx.x];
    __syncthreads();
    long rr = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (rr >= m) return;
    long r = p + NB + rr;
    T w[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        long off = r - (p + c);
        T v = off <= bw ? band[(p + c) * ld + off] : T(0);
#pragma unroll
        for (int k = 0; k < c; ++k) v -= w[k] * l[c][k];
        w[c] = v;
    }
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        long off = r - (p + c);
        if (off <= bw) band[(p + c) * ld + off] = w[c] * di[c];
        wbuf[c * m + rr] = w[c];
    }
}

// Trailing update: A_rj -= sum_k W_rk L_jk over the panel, for the lower
// triangle of rows/cols [p+32, p+32+m) (always inside the band since m <= bw).
template <typename T, int TS>
__global__ void __launch_bounds__(256) trailing_kernel(T *band, long ld, long p, long m, const T *wbuf,
                                                       const T *dinv)
{
    int ti = blockIdx.y, tj = blockIdx.x;
    if (tj > ti) return;
    __shared__ T wr[NB][TS + 1];  // W rows of the tile (k, r)
    __shared__ T lc[NB][TS + 1];  // L rows of the tile columns (k, j)
    const long base = p + NB;
    const long r0 = (long)ti * TS, j0 = (long)tj * TS;
    for (int idx = threadIdx.x; idx < NB * TS; idx += blockDim.x) {
        int k = idx / TS, t = idx % TS;
        long rr = r0 + t, jj = j0 + t;
        wr[k][t] = rr < m ? wbuf[k * m + rr] : T(0);
        // L_{j,p+k} = W_jk / d_k
        lc[k][t] = jj < m ? wbuf[k * m + jj] * dinv[p + k] : T(0);
    }
    __syncthreads();
    constexpr int PER = TS * TS / 256 > 0 ? TS * TS / 256 : 1;
    for (int q = 0; q < PER; ++q) {
        int idx = threadIdx.x + q * 256;
        if (idx >= TS * TS) break;
        int ri = idx / TS, ji = idx % TS;
        long rr = r0 + ri, jj = j0 + ji;
        if (rr >= m || jj >= m || jj > rr) continue;
        T acc = 0;
#pragma unroll 8
        for (int k = 0; k < NB; ++k) acc += wr[k][ri] * lc[k][ji];
        long col = base + jj;
        band[col * ld + (rr - jj)] -= acc;
    }
}

// -------------------------------------------------------------------------
// Block-bidiagonal inverse form
// -------------------------------------------------------------------------

// Value of the unit-lower factor L at global (R, C), R >= C.
template <typename T>
__device__ __forceinline__ T lval(const T *band, long ld, long bw, long R, long C)
{
    if (R == C) return T(1);
    long off = R - C;
    return (off > 0 && off <= bw) ? band[C * ld + off] : T(0);
}

// Linv_i columns [c0, c0+W) by column-oriented forward substitution on a
// shared-memory copy of those columns. Linv is stored row-major (r*s + c).
template <typename T, int W>
__global__ void __launch_bounds__(256) block_inverse_kernel(const T *band, long ld, long bw, long s,
                                                            T *linv)
{
    extern __shared__ unsigned char smem_raw[];
    T *X = reinterpret_cast<T *>(smem_raw);  // [s][W]
    const long i = blockIdx.y;
    const long c0 = (long)blockIdx.x * W;
    const long gbase = i * s;
    for (long idx = threadIdx.x; idx < s * W; idx += blockDim.x) {
        long r = idx / W;
        int w = idx % W;
        X[idx] = (r == c0 + w) ? T(1) : T(0);
    }
    __syncthreads();
    for (long k = c0; k < s; ++k) {
        // X[r][w] -= L[r][k] X[k][w] for r in (k, min(s, k+bw)]
        long rmax = min(s - 1, k + bw);
        long cnt = (rmax - k) * W;
        for (long idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
            long r = k + 1 + idx / W;
            int w = idx % W;
            T xk = X[k * W + w];
            if (xk != T(0)) X[r * W + w] -= band[(gbase + k) * ld + (r - k)] * xk;
        }
        __syncthreads();
    }
    for (long idx = threadIdx.x; idx < s * W; idx += blockDim.x) {
        long r = idx / W;
        int w = idx % W;
        linv[i * s * s + r * s + c0 + w] = X[idx];
    }
}

// Batched products of the solve, 32x32 output tiles, shared-memory k-tiles:
//   mode 0: P_i = Linv_i * L_{i,i-1}           (i >= 1), row-major
//   mode 1: R_i = L_{i+1,i} * Linv_i           (i <= nblk-2), stored transposed
template <typename T, int MODE>
__global__ void __launch_bounds__(256) block_gemm_kernel(const T *band, long ld, long bw, long s,
                                                         long nblk, const T *linv, T *out)
{
    constexpr int TS = 32;
    __shared__ T As[TS][TS + 1];
    __shared__ T Bs[TS][TS + 1];
    const long i = blockIdx.z + (MODE == 0 ? 1 : 0);
    if (MODE == 0 && i >= nblk) return;
    if (MODE == 1 && i > nblk - 2) return;
    const long r0 = (long)blockIdx.y * TS, c0 = (long)blockIdx.x * TS;
    const T *Li = linv + i * s * s;
    const int tx = threadIdx.x % TS, ty = threadIdx.x / TS;  // 32 x 8
    T acc[4] = {0, 0, 0, 0};
    // k-tile range with non-zero contributions
    long kt_begin = 0, kt_end = s / TS;
    if (MODE == 0) {
        // A = Linv_i (lower): k <= r; B = L_{i,i-1}[k][c] needs s + k - c <= bw
        kt_end = min(kt_end, r0 / TS + 1);
        long kmax = c0 + TS - 1 + bw - s;  // largest k with a non-zero B entry
        if (kmax < 0) kt_end = 0;
        else kt_end = min(kt_end, kmax / TS + 1);
    } else {
        // A = L_{i+1,i}[r][k] needs s + r - k <= bw -> k >= s + r - bw; B = Linv_i (lower): k >= c
        long kmin = max(c0, s + r0 - bw);
        kt_begin = max(0L, kmin / TS);
    }
    for (long kt = kt_begin; kt < kt_end; ++kt) {
        const long k0 = kt * TS;
        for (int q = 0; q < 4; ++q) {
            int rr = ty + 8 * q;
            long r = r0 + rr, k = k0 + tx;
            T a, b;
            if (MODE == 0) {
                a = Li[r * s + k];
                // B[k][c] = L(global (i*s + k), (i-1)*s + c), with k = k0+rr, c = c0+tx
                long R = i * s + k0 + rr, C = (i - 1) * s + c0 + tx;
                b = lval(band, ld, bw, R, C);
            } else {
                long R = (i + 1) * s + r, C = i * s + k;
                a = lval(band, ld, bw, R, C);
                b = Li[(k0 + rr) * s + c0 + tx];
            }
            As[rr][tx] = a;
            Bs[rr][tx] = b;
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < TS; ++k) {
            T bv = Bs[k][tx];
            for (int q = 0; q < 4; ++q) acc[q] += As[ty + 8 * q][k] * bv;
        }
        __syncthreads();
    }
    T *O = out + i * s * s;
    for (int q = 0; q < 4; ++q) {
        long r = r0 + ty + 8 * q, c = c0 + tx;
        if (MODE == 0) O[r * s + c] = acc[q];
        else O[c * s + r] = acc[q];
    }
}

// -------------------------------------------------------------------------
// Solve kernels
// -------------------------------------------------------------------------

// u_i = Linv_i b_i for every block (warp per row; b in FP64).
template <typename T>
__global__ void __launch_bounds__(256) fwd_diag_kernel(const T *linv, long s, long n, const double *b,
                                                       T *u)
{
    const long row = blockIdx.x * 8L + threadIdx.x / 32;  // global padded row
    const int lane = threadIdx.x % 32;
    const long i = row / s, r = row % s;
    const T *L = linv + i * s * s + r * s;
    T acc = 0;
    for (long k = lane; k <= r; k += 32) {
        long g = i * s + k;
        T bv = g < n ? (T)b[g] : T(0);
        acc += L[k] * bv;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) u[row] = acc;
}

// y_i = u_i - P_i y_{i-1} (in place on y; warp per row)
template <typename T>
__global__ void __launch_bounds__(256) fwd_step_kernel(const T *pmat, long s, long i, T *y)
{
    const long r = blockIdx.x * 8L + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    const T *P = pmat + i * s * s + r * s;
    const T *yp = y + (i - 1) * s;
    T acc = 0;
    for (long k = lane; k < s; k += 32) acc += P[k] * yp[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) y[i * s + r] -= acc;
}

// v_i = Linv_i^T (y_i * dinv_i) for every block; thread per output column.
template <typename T>
__global__ void __launch_bounds__(256) bwd_diag_kernel(const T *linv, long s, long npad, const T *y,
                                                       const T *dinv, T *v)
{
    const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (g >= npad) return;
    const long i = g / s, c = g % s;
    const T *L = linv + i * s * s;
    const T *yi = y + i * s;
    const T *di = dinv + i * s;
    T acc = 0;
    for (long k = c; k < s; ++k) acc += L[k * s + c] * (yi[k] * di[k]);
    v[g] = acc;
}

// x_i = v_i - R_i^T x_{i+1} (in place on v; Rt row-major = R^T)
template <typename T>
__global__ void __launch_bounds__(256) bwd_step_kernel(const T *rt, long s, long i, T *x)
{
    const long r = blockIdx.x * 8L + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    const T *Rr = rt + i * s * s + r * s;
    const T *xn = x + (i + 1) * s;
    T acc = 0;
    for (long k = lane; k < s; k += 32) acc += Rr[k] * xn[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) x[i * s + r] -= acc;
}

template <typename T>
__global__ void store_f64_kernel(const T *x, long n, double *out)
{
    long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (g < n) out[g] = (double)x[g];
}

template <typename T>
__global__ void pad_identity_kernel(T *band, long ld, long n, long npad)
{
    long j = n + blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (j < npad) band[j * ld] = T(1);
}

template <typename T>
int inverse_width(long s)
{
    const long budget = 200 * 1024;
    if (s * 32 * (long)sizeof(T) <= budget) return 32;
    if (s * 16 * (long)sizeof(T) <= budget) return 16;
    return 8;
}

template <typename T, int W>
void set_inverse_smem(long s)
{
    size_t smem = (size_t)s * W * sizeof(T);
    CB_CUDA(cudaFuncSetAttribute(block_inverse_kernel<T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
}

template <typename T, int W>
void launch_inverse(BandFactor &f, cudaStream_t st)
{
    size_t smem = (size_t)f.s * W * sizeof(T);
    dim3 grid((unsigned)(f.s / W), (unsigned)f.nblk);
    block_inverse_kernel<T, W><<<grid, 256, smem, st>>>((const T *)f.band, f.ld, f.bw, f.s, (T *)f.linv);
}

template <typename T>
void factor_impl(BandFactor &f, cudaStream_t st, long *launches)
{
    T *band = (T *)f.band;
    T *dinv = (T *)f.dinv;
    T *wbuf = (T *)f.work;  // NB * bw scratch (the solve vectors are not live during a factor)
    const long npad = f.nblk * f.s;
    if (npad > f.n) {
        pad_identity_kernel<T><<<(unsigned)((npad - f.n + 127) / 128), 128, 0, st>>>(band, f.ld, f.n, npad);
        ++*launches;
    }
    CB_CUDA(cudaMemsetAsync(f.flags, 0, 2 * sizeof(int), st));
    for (long p = 0; p < npad; p += NB) {
        diag_factor_kernel<T><<<1, 256, 0, st>>>(band, f.ld, f.bw, p, f.n, dinv, f.ssd, f.flags);
        long m = std::min(f.bw, npad - p - NB);
        *launches += 1;
        if (m <= 0) continue;
        panel_trsm_kernel<T><<<(unsigned)((m + 63) / 64), 64, 0, st>>>(band, f.ld, f.bw, p, m, dinv, wbuf);
        constexpr int TS = sizeof(T) == 8 ? 16 : 32;
        unsigned nt = (unsigned)((m + TS - 1) / TS);
        trailing_kernel<T, TS><<<dim3(nt, nt), 256, 0, st>>>(band, f.ld, p, m, wbuf, dinv);
        *launches += 2;
    }
    int w = f.inv_width;
    if (w == 32) launch_inverse<T, 32>(f, st);
    else if (w == 16) launch_inverse<T, 16>(f, st);
    else launch_inverse<T, 8>(f, st);
    dim3 g((unsigned)(f.s / 32), (unsigned)(f.s / 32), (unsigned)std::max(1L, f.nblk - 1));
    block_gemm_kernel<T, 0><<<g, 256, 0, st>>>(band, f.ld, f.bw, f.s, f.nblk, (const T *)f.linv, (T *)f.pmat);
    block_gemm_kernel<T, 1><<<g, 256, 0, st>>>(band, f.ld, f.bw, f.s, f.nblk, (const T *)f.linv, (T *)f.rmat);
    *launches += 3;
    CB_CUDA(cudaGetLastError());
}

template <typename T>
void solve_impl(BandFactor &f, const double *rhs, double *x, cudaStream_t st, long *launches)
{
    const long s = f.s, nb = f.nblk, npad = nb * s;
    T *y = (T *)f.work;
    T *v = y + npad;
    fwd_diag_kernel<T><<<(unsigned)(npad / 8), 256, 0, st>>>((const T *)f.linv, s, f.n, rhs, y);
    for (long i = 1; i < nb; ++i)
        fwd_step_kernel<T><<<(unsigned)(s / 8), 256, 0, st>>>((const T *)f.pmat, s, i, y);
    bwd_diag_kernel<T><<<(unsigned)((npad + 255) / 256), 256, 0, st>>>((const T *)f.linv, s, npad, y,
                                                                        (const T *)f.dinv, v);
    for (long i = nb - 2; i >= 0; --i)
        bwd_step_kernel<T><<<(unsigned)(s / 8), 256, 0, st>>>((const T *)f.rmat, s, i, v);
    store_f64_kernel<T><<<(unsigned)((f.n + 255) / 256), 256, 0, st>>>(v, f.n, x);
    *launches += 2 * nb + 2;
    CB_CUDA(cudaGetLastError());
}

// The solve's launch sequence with caller-provided work vectors (2*npad T).
template <typename T>
void solve_ws_impl(const BandFactor &f, const double *rhs, double *x, void *work, cudaStream_t st)
{
    const long s = f.s, nb = f.nblk, npad = nb * s;
    T *y = (T *)work;
    T *v = y + npad;
    fwd_diag_kernel<T><<<(unsigned)(npad / 8), 256, 0, st>>>((const T *)f.linv, s, f.n, rhs, y);
    for (long i = 1; i < nb; ++i)
        fwd_step_kernel<T><<<(unsigned)(s / 8), 256, 0, st>>>((const T *)f.pmat, s, i, y);
    bwd_diag_kernel<T><<<(unsigned)((npad + 255) / 256), 256, 0, st>>>((const T *)f.linv, s, npad, y,
                                                                        (const T *)f.dinv, v);
    for (long i = nb - 2; i >= 0; --i)
        bwd_step_kernel<T><<<(unsigned)(s / 8), 256, 0, st>>>((const T *)f.rmat, s, i, v);
    store_f64_kernel<T><<<(unsigned)((f.n + 255) / 256), 256, 0, st>>>(v, f.n, x);
}

template <typename T>
void profile_impl(BandFactor &f, int which, cudaStream_t st)
{
    const long s = f.s;
    if (which == 0) {
        long i = f.nblk > 1 ? 1 : 0;
        if (i == 0) return;
        fwd_step_kernel<T><<<(unsigned)(s / 8), 256, 0, st>>>((const T *)f.pmat, s, i, (T *)f.work);
    } else if (which == 4) {
        long m = std::min(f.bw, f.nblk * f.s - NB);
        if (m <= 0) return;
        constexpr int TS = sizeof(T) == 8 ? 16 : 32;
        unsigned nt = (unsigned)((m + TS - 1) / TS);
        trailing_kernel<T, TS><<<dim3(nt, nt), 256, 0, st>>>((T *)f.band, f.ld, 0, m, (const T *)f.work,
                                                              (const T *)f.dinv);
    }
}

}  // namespace

void band_solve_with_work(const BandFactor &f, const double *rhs, double *x, void *work, cudaStream_t st)
{
    if (f.fp32) solve_ws_impl<float>(f, rhs, x, work, st);
    else solve_ws_impl<double>(f, rhs, x, work, st);
    CB_CUDA(cudaGetLastError());
}

void band_profile_launch(BandFactor &f, int which, cudaStream_t st)
{
    if (f.fp32) profile_impl<float>(f, which, st);
    else profile_impl<double>(f, which, st);
    CB_CUDA(cudaGetLastError());
}

void band_alloc(BandFactor &f, long n, long bw, bool fp32)
{
    f.n = n;
    f.bw = std::max(1L, bw);
    f.fp32 = fp32;
    f.ld = ((f.bw + 1 + 7) / 8) * 8;
    f.s = std::max(32L, ((f.bw + 31) / 32) * 32);
    f.nblk = (n + f.s - 1) / f.s;
    const long npad = f.nblk * f.s;
    const size_t es = fp32 ? 4 : 8;
    CB_CUDA(cudaMalloc(&f.band, es * (size_t)f.ld * npad));
    CB_CUDA(cudaMalloc(&f.dinv, es * (size_t)npad));
    CB_CUDA(cudaMalloc(&f.linv, es * (size_t)f.nblk * f.s * f.s));
    CB_CUDA(cudaMalloc(&f.pmat, es * (size_t)f.nblk * f.s * f.s));
    CB_CUDA(cudaMalloc(&f.rmat, es * (size_t)f.nblk * f.s * f.s));
    size_t work = std::max((size_t)2 * npad, (size_t)NB * f.bw + NB);
    CB_CUDA(cudaMalloc(&f.work, es * work));
    CB_CUDA(cudaMalloc(&f.ssd, sizeof(double) * (size_t)n));
    CB_CUDA(cudaMalloc(&f.flags, 2 * sizeof(int)));
    CB_CUDA(cudaMemset(f.pmat, 0, es * (size_t)f.nblk * f.s * f.s));
    CB_CUDA(cudaMemset(f.rmat, 0, es * (size_t)f.nblk * f.s * f.s));
    f.inv_width = fp32 ? inverse_width<float>(f.s) : inverse_width<double>(f.s);
    if (fp32) {
        if (f.inv_width == 32) set_inverse_smem<float, 32>(f.s);
        else if (f.inv_width == 16) set_inverse_smem<float, 16>(f.s);
        else set_inverse_smem<float, 8>(f.s);
    } else {
        if (f.inv_width == 32) set_inverse_smem<double, 32>(f.s);
        else if (f.inv_width == 16) set_inverse_smem<double, 16>(f.s);
        else set_inverse_smem<double, 8>(f.s);
    }
}

void band_free(BandFactor &f)
{
    if (f.factor_graph) cudaGraphExecDestroy(f.factor_graph);
    for (auto &g : f.solve_graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (void *p : {f.band, f.dinv, f.linv, f.pmat, f.rmat, f.work, (void *)f.ssd, (void *)f.flags})
        if (p) cudaFree(p);
    f = BandFactor{};
}

void band_factor(BandFactor &f, cudaStream_t st, bool use_graph, long *launches)
{
    long dummy = 0;
    long *cnt = launches ? launches : &dummy;
    if (!use_graph) {
        if (f.fp32) factor_impl<float>(f, st, cnt);
        else factor_impl<double>(f, st, cnt);
        return;
    }
    if (!f.factor_graph) {
        long per = 0;
        cudaGraph_t g;
        CB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        if (f.fp32) factor_impl<float>(f, st, &per);
        else factor_impl<double>(f, st, &per);
        CB_CUDA(cudaStreamEndCapture(st, &g));
        CB_CUDA(cudaGraphInstantiate(&f.factor_graph, g, 0));
        cudaGraphDestroy(g);
        f.factor_launches = per;
    }
    CB_CUDA(cudaGraphLaunch(f.factor_graph, st));
    *cnt += f.factor_launches;
}

void band_solve(BandFactor &f, const double *rhs, double *x, cudaStream_t st, bool use_graph, long *launches)
{
    long dummy = 0;
    long *cnt = launches ? launches : &dummy;
    if (!use_graph) {
        if (f.fp32) solve_impl<float>(f, rhs, x, st, cnt);
        else solve_impl<double>(f, rhs, x, st, cnt);
        return;
    }
    BandFactor::SolveGraph *slot = nullptr;
    for (auto &g : f.solve_graphs)
        if (g.exec && g.in == rhs && g.out == x) slot = &g;
    if (!slot) {
        slot = &f.solve_graphs[0];
        for (auto &g : f.solve_graphs)
            if (!g.exec) {
                slot = &g;
                break;
            }
        if (slot->exec) cudaGraphExecDestroy(slot->exec);
        long per = 0;
        cudaGraph_t g;
        CB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        if (f.fp32) solve_impl<float>(f, rhs, x, st, &per);
        else solve_impl<double>(f, rhs, x, st, &per);
        CB_CUDA(cudaStreamEndCapture(st, &g));
        CB_CUDA(cudaGraphInstantiate(&slot->exec, g, 0));
        cudaGraphDestroy(g);
        slot->in = rhs;
        slot->out = x;
        slot->launches = per;
    }
    CB_CUDA(cudaGraphLaunch(slot->exec, st));
    *cnt += slot->launches;
}

}  // namespace cb
