// Band LDL^T of the tangent stiffness and its block-bidiagonal solve.
//
// This replaces skyfact/skysolve (solve.c:539-698). The factorisation keeps
// the reference's equation order (no pivoting, no reordering), so the pivots
// ssd and the indefiniteness flag det that the MSAL driver reads
// (main.c:2636-2642, 2765-2769) are the reference's quantities.
//
// Storage: lower band, column-major, L(i,j) at band[j*ld + (i-j)] for
// 0 <= i-j <= bw; after factoring, the diagonal slots hold D and the rest the
// unit-lower L. The matrix is padded to npad = nblk*s equations with identity
// rows; s (a multiple of 32, at least w = bw rounded up to 32) is the block
// size of the solve.
//
// Factor: right-looking over 32-column panels, two launches per panel (the
// 32x32 diagonal LDL^T in shared memory fused with the panel TRSM; then the
// rank-32 update of the trailing band), replayed as a CUDA graph.
//
// Solve: with s >= bw, L is block lower-bidiagonal in s x s blocks and the
// coupling block L_{i,i-1} has non-zeros only in its last w columns (L_{i+1,i}
// only in its first w rows). The factor step forms
//     Linv_i = L_ii^-1                      (s x s, tiled triangular inverse)
//     Pn_i   = Linv_i L_{i,i-1}[:, s-w:s]   (s x w)
//     Rn_i   = (L_{i+1,i}[0:w, :] Linv_i)^T (s x w)
// so that one solve is
//     y_i = Linv_i b_i - Pn_i y_{i-1}[s-w:s]            (forward)
//     x_i = Linv_i^T (y_i / D_i) - Rn_i x_{i+1}[0:w]    (backward)
// run by one persistent cooperative kernel with 2*nblk + 2 grid barriers
// (Linv is also kept transposed so both block-diagonal products are
// coalesced row dots). A
// larger s lowers the number of sequential steps while the bytes per step
// (s*w) and per solve stay about the same.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "internal.hpp"

namespace cb {

namespace {

constexpr int NB = 32;  // panel width and tile size

#define CB_CUDA(x)                                                                         \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + \
                                     " at " __FILE__ ":" + std::to_string(__LINE__));      \
    } while (0)

// Value of the unit-lower factor L at global (R, C), R >= C.
template <typename T>
__device__ __forceinline__ T lval(const T *band, long ld, long bw, long R, long C)
{
    if (R == C) return T(1);
    long off = R - C;
    return (off > 0 && off <= bw) ? band[C * ld + off] : T(0);
}

// -------------------------------------------------------------------------
// Factor kernels
// -------------------------------------------------------------------------

// Panel p: every CTA (1024 threads, one per entry of the 32x32 diagonal
// block) redundantly
//   1. factors the diagonal block (LDL^T in shared memory, one elimination
//      step per column) and
//   2. inverts its unit-lower factor, Linv_pp = L_pp^-1 (one substitution
//      step per column),
// then takes up to kPanelRows of the panel rows r in [p+32, p+32+m), stages
// them in shared memory and solves them as a small GEMM with no dependency
// chain: W_r = A_r Linv_pp^T (= L_r D), L_rc = W_rc / d_c. W is kept for the
// trailing update (wbuf, column-major in the panel column). CTA 0 writes 1/d,
// the pivots, the flags and the factored diagonal block; the block goes to a
// staging buffer because the other CTAs still read the unfactored one from
// the band, and the trailing-update launch copies it into place.
constexpr int kPanelThreads = 1024;
constexpr int kPanelRows = 128;

template <typename T>
__global__ void __launch_bounds__(kPanelThreads) panel_kernel(T *band, long ld, long bw, long p, long m,
                                                              T *dinv, double *ssd, int *flags, T *wbuf,
                                                              long n, T *stage)
{
    __shared__ T a[NB][NB + 1];
    __shared__ T x[NB][NB + 1];
    __shared__ T ar[kPanelRows][NB + 1];
    __shared__ T di[NB];
    const int tid = threadIdx.x;
    const int i = tid % NB, j = tid / NB;  // this thread's entry (i, j)
    const long r_begin = (long)blockIdx.x * kPanelRows;
    const long nrows = m - r_begin < kPanelRows ? m - r_begin : kPanelRows;
    a[i][j] = (i >= j && i - j <= bw) ? band[(p + j) * ld + (i - j)] : T(0);
    x[i][j] = (i == j) ? T(1) : T(0);
    // stage this CTA's panel rows: ar[rr][k] = A(p+32+r_begin+rr, p+k)
    for (int idx = tid; idx < kPanelRows * NB; idx += kPanelThreads) {
        const int k = idx / kPanelRows, rr = idx % kPanelRows;
        const long off = NB + r_begin + rr - k;
        ar[rr][k] = (rr < nrows && off <= bw) ? band[(p + k) * ld + off] : T(0);
    }
    __syncthreads();
    for (int k = 0; k < NB; ++k) {
        const T d = a[k][k];
        const bool live = i >= j && j >= k;
        const T lik = (live && i > k) ? a[i][k] / d : T(0);
        const T ljk = (live && j > k) ? a[j][k] / d : T(0);
        __syncthreads();
        if (live && j > k) a[i][j] -= lik * d * ljk;
        if (j == k && i > k) a[i][k] = lik;
        __syncthreads();
    }
    for (int k = 0; k < NB; ++k) {
        if (i > k && j <= k) x[i][j] -= a[i][k] * x[k][j];
        __syncthreads();
    }
    if (tid < NB) di[tid] = T(1) / a[tid][tid];
    if (blockIdx.x == 0) {
        stage[j * NB + i] = a[i][j];
        if (tid < NB) {
            const T dl = a[tid][tid];
            dinv[p + tid] = T(1) / dl;
            long g = p + tid;
            if (g < n) {
                ssd[g] = (double)dl;
                if (!(dl > T(0))) atomicOr(&flags[0], 1);
                if (dl == T(0)) atomicOr(&flags[1], 1);
            }
        }
    }
    __syncthreads();
    for (int idx = tid; idx < kPanelRows * NB; idx += kPanelThreads) {
        const int c = idx / kPanelRows, rr = idx % kPanelRows;
        if (rr >= nrows) continue;
        T acc = 0;
#pragma unroll 8
        for (int k = 0; k <= c; ++k) acc += ar[rr][k] * x[c][k];
        const long row = r_begin + rr;
        wbuf[c * m + row] = acc;
        const long off = NB + row - c;
        if (off <= bw) band[(p + c) * ld + off] = acc * di[c];
    }
}

// Trailing update: A_rj -= sum_k W_rk L_jk over the panel, for the lower
// triangle of rows/cols [p+32, p+32+m) (always inside the band since m <= bw);
// CTA (0,0) also stores panel p's factored diagonal block from the stage.
template <typename T, int TS>
__global__ void __launch_bounds__(256) trailing_kernel(T *band, long ld, long bw, long p, long m, const T *wbuf,
                                                       const T *dinv, const T *stage)
{
    int ti = blockIdx.y, tj = blockIdx.x;
    if (tj > ti) return;
    if (ti == 0 && tj == 0) {
        // the factored 32x32 diagonal block of panel p, staged by panel_kernel
        for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
            int j = idx / NB, i = idx % NB;
            if (i >= j && i - j <= bw) band[(p + j) * ld + (i - j)] = stage[idx];
        }
    }
    __shared__ T wr[NB][TS + 1];
    __shared__ T lc[NB][TS + 1];
    const long base = p + NB;
    const long r0 = (long)ti * TS, j0 = (long)tj * TS;
    for (int idx = threadIdx.x; idx < NB * TS; idx += blockDim.x) {
        int k = idx / TS, t = idx % TS;
        long rr = r0 + t, jj = j0 + t;
        wr[k][t] = rr < m ? wbuf[k * m + rr] : T(0);
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

template <typename T>
__global__ void pad_identity_kernel(T *band, long ld, long n, long npad)
{
    long j = n + blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (j < npad) band[j * ld] = T(1);
}

// -------------------------------------------------------------------------
// Tiled inverse of the unit-lower diagonal blocks (Linv row-major, s x s)
// -------------------------------------------------------------------------

// Diagonal 32x32 tiles: lane c forms column c of the tile's inverse.
template <typename T>
__global__ void __launch_bounds__(32) inv_diag_kernel(const T *band, long ld, long bw, long s, T *linv)
{
    __shared__ T L[NB][NB + 1];
    __shared__ T X[NB][NB + 1];
    const long i = blockIdx.y, I = blockIdx.x;
    const long g0 = i * s + I * NB;
    const int c = threadIdx.x;
    for (int r = 0; r < NB; ++r) L[r][c] = (r > c) ? lval(band, ld, bw, g0 + r, g0 + c) : T(0);
    for (int r = 0; r < NB; ++r) X[r][c] = T(0);
    X[c][c] = T(1);
    __syncwarp();
    for (int r = c + 1; r < NB; ++r) {
        T acc = 0;
        for (int k = c; k < r; ++k) acc += L[r][k] * X[k][c];
        X[r][c] = -acc;
    }
    __syncwarp();
    T *out = linv + i * s * s + (I * NB) * s + I * NB;
    for (int r = 0; r < NB; ++r) out[r * s + c] = X[r][c];
}

// Row tile I of Linv: X_IJ = -T_II * sum_K L_IK X_KJ for J < I, K in
// [max(J, I-kb), I); T_II is the inverse diagonal tile written above.
template <typename T>
__global__ void __launch_bounds__(256) inv_row_kernel(const T *band, long ld, long bw, long s, long I,
                                                      long kb, T *linv)
{
    __shared__ T As[NB][NB + 1];
    __shared__ T Bs[NB][NB + 1];
    const long J = blockIdx.x, i = blockIdx.y;
    if (J >= I) return;
    T *Li = linv + i * s * s;
    const int tx = threadIdx.x % NB, ty = threadIdx.x / NB;  // 32 x 8
    T acc[4] = {0, 0, 0, 0};
    const long k_begin = J > I - kb ? J : I - kb;
    for (long K = k_begin; K < I; ++K) {
        for (int q = 0; q < 4; ++q) {
            int rr = ty + 8 * q;
            As[rr][tx] = lval(band, ld, bw, i * s + I * NB + rr, i * s + K * NB + tx);
            Bs[rr][tx] = Li[(K * NB + rr) * s + J * NB + tx];
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < NB; ++k) {
            T b = Bs[k][tx];
            for (int q = 0; q < 4; ++q) acc[q] += As[ty + 8 * q][k] * b;
        }
        __syncthreads();
    }
    for (int q = 0; q < 4; ++q) {
        int rr = ty + 8 * q;
        As[rr][tx] = Li[(I * NB + rr) * s + I * NB + tx];
        Bs[rr][tx] = acc[q];
    }
    __syncthreads();
    for (int q = 0; q < 4; ++q) {
        int rr = ty + 8 * q;
        T v = 0;
        for (int k = 0; k <= rr; ++k) v += As[rr][k] * Bs[k][tx];
        Li[(I * NB + rr) * s + J * NB + tx] = -v;
    }
}

// linvt_i = Linv_i^T (row-major), 32x32 tiles through shared memory.
template <typename T>
__global__ void __launch_bounds__(256) transpose_kernel(const T *linv, long s, T *linvt)
{
    __shared__ T t[NB][NB + 1];
    const long i = blockIdx.z, r0 = (long)blockIdx.y * NB, c0 = (long)blockIdx.x * NB;
    if (c0 > r0) return;  // upper tiles of Linv are zero and stay zero in linvt's lower part
    const T *src = linv + i * s * s;
    T *dst = linvt + i * s * s;
    const int tx = threadIdx.x % NB, ty = threadIdx.x / NB;
    for (int q = 0; q < 4; ++q) t[ty + 8 * q][tx] = src[(r0 + ty + 8 * q) * s + c0 + tx];
    __syncthreads();
    for (int q = 0; q < 4; ++q) dst[(c0 + ty + 8 * q) * s + r0 + tx] = t[tx][ty + 8 * q];
}

// Pn_i (s x w) = Linv_i * L_{i,i-1}[:, s-w:s], i >= 1; k in [0, min(r, j + bw - w)].
template <typename T>
__global__ void __launch_bounds__(256) pn_kernel(const T *band, long ld, long bw, long s, long w,
                                                 const T *linv, T *pn)
{
    __shared__ T As[NB][NB + 1];
    __shared__ T Bs[NB][NB + 1];
    const long i = blockIdx.z + 1;
    const long r0 = (long)blockIdx.y * NB, j0 = (long)blockIdx.x * NB;
    const T *Li = linv + i * s * s;
    const int tx = threadIdx.x % NB, ty = threadIdx.x / NB;
    T acc[4] = {0, 0, 0, 0};
    const long kmax_a = r0 + NB - 1, kmax_b = j0 + NB - 1 + bw - w;
    const long kmax = kmax_a < kmax_b ? kmax_a : kmax_b;
    for (long k0 = 0; k0 <= kmax; k0 += NB) {
        for (int q = 0; q < 4; ++q) {
            int rr = ty + 8 * q;
            As[rr][tx] = Li[(r0 + rr) * s + k0 + tx];
            Bs[rr][tx] = lval(band, ld, bw, i * s + k0 + rr, (i - 1) * s + s - w + j0 + tx);
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < NB; ++k) {
            T b = Bs[k][tx];
            for (int q = 0; q < 4; ++q) acc[q] += As[ty + 8 * q][k] * b;
        }
        __syncthreads();
    }
    T *O = pn + i * s * w;
    for (int q = 0; q < 4; ++q) O[(r0 + ty + 8 * q) * w + j0 + tx] = acc[q];
}

// Rn_i (s x w): Rn[c][j] = sum_k L((i+1)s + j, i s + k) Linv_i[k][c], i <= nblk-2;
// k in [max(c, s + j - bw), s).
template <typename T>
__global__ void __launch_bounds__(256) rn_kernel(const T *band, long ld, long bw, long s, long w,
                                                 const T *linv, T *rn)
{
    __shared__ T As[NB][NB + 1];  // Linv tile: As[k][c]
    __shared__ T Bs[NB][NB + 1];  // L tile transposed: Bs[k][j]
    const long i = blockIdx.z;
    const long c0 = (long)blockIdx.y * NB, j0 = (long)blockIdx.x * NB;
    const T *Li = linv + i * s * s;
    const int tx = threadIdx.x % NB, ty = threadIdx.x / NB;
    T acc[4] = {0, 0, 0, 0};  // rows c = c0 + ty + 8q, column j = j0 + tx
    long kmin = s + j0 - bw;
    if (kmin < c0) kmin = c0;
    long kstart = kmin > 0 ? (kmin / NB) * NB : 0;
    for (long k0 = kstart; k0 < s; k0 += NB) {
        for (int q = 0; q < 4; ++q) {
            int kk = ty + 8 * q;
            As[kk][tx] = Li[(k0 + kk) * s + c0 + tx];
            Bs[kk][tx] = lval(band, ld, bw, (i + 1) * s + j0 + tx, i * s + k0 + kk);
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < NB; ++k) {
            T b = Bs[k][tx];
            for (int q = 0; q < 4; ++q) acc[q] += As[k][ty + 8 * q] * b;
        }
        __syncthreads();
    }
    T *O = rn + i * s * w;
    for (int q = 0; q < 4; ++q) O[(c0 + ty + 8 * q) * w + j0 + tx] = acc[q];
}

// -------------------------------------------------------------------------
// Persistent solve
// -------------------------------------------------------------------------

// Grid barrier for a cooperative launch. The wait is bounded: after 2^24
// polls (well over a second) the CTA records a timeout in bar->err and goes
// on, so a fault cannot hang the GPU; the host turns the flag into
// CB_ERR_TIMEOUT.
__device__ __forceinline__ void grid_barrier(GridBarrier *bar, unsigned nblocks)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &bar->gen;
        unsigned gen = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(&bar->count, 1u) + 1u;
        if (arrived == nblocks) {
            bar->count = 0;
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            unsigned long long polls = 0;
            while (*vgen == gen) {
                if (++polls > (1ull << 24)) {
                    atomicExch(&bar->err, 1);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

template <typename T>
struct SolveArgs {
    const T *linv, *linvt, *pn, *rn, *dinv;
    long s, w, nblk, n;
    const double *rhs;
    double *out;
    T *y, *v, *z;
    GridBarrier *bar;
};

template <typename T>
__device__ __forceinline__ T warp_reduce(T v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Dot product of a warp's row with a vector: lanes stride the row, eight
// independent loads in flight per lane, then a shuffle reduction.
template <typename T>
__device__ __forceinline__ T warp_row_dot(const T *__restrict__ row, const T *__restrict__ vec, long len,
                                          int lane)
{
    T acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    long j = lane;
    for (; j + 7 * 32 < len; j += 8 * 32) {
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] += row[j + u * 32] * vec[j + u * 32];
    }
    for (; j < len; j += 32) acc[0] += row[j] * vec[j];
    T s = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
    return warp_reduce(s);
}

template <typename T>
__global__ void __launch_bounds__(256) solve_kernel(SolveArgs<T> a)
{
    const long s = a.s, w = a.w, nb = a.nblk, npad = nb * s;
    const int lane = threadIdx.x % 32;
    const long gwarp = blockIdx.x * 8L + threadIdx.x / 32;
    const long nwarps = gridDim.x * 8L;
    const long gthr = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const long nthr = gridDim.x * (long)blockDim.x;
    // A: y = blockdiag(Linv) b (b converted to T into w first)
    for (long g = gthr; g < npad; g += nthr) a.z[g] = g < a.n ? (T)a.rhs[g] : T(0);
    grid_barrier(a.bar, gridDim.x);
    for (long row = gwarp; row < npad; row += nwarps) {
        const long i = row / s, r = row % s;
        T acc = warp_row_dot(a.linv + i * s * s + r * s, a.z + i * s, r + 1, lane);
        if (lane == 0) a.y[row] = acc;
    }
    grid_barrier(a.bar, gridDim.x);
    // B: y_i -= Pn_i y_{i-1}[s-w:s]
    for (long i = 1; i < nb; ++i) {
        const T *yp = a.y + i * s - w;
        for (long r = gwarp; r < s; r += nwarps) {
            T acc = warp_row_dot(a.pn + i * s * w + r * w, yp, w, lane);
            if (lane == 0) a.y[i * s + r] -= acc;
        }
        grid_barrier(a.bar, gridDim.x);
    }
    // C: v = blockdiag(Linv^T) (y / D), warp per row of the stored transpose
    for (long g = gthr; g < npad; g += nthr) a.z[g] = a.y[g] * a.dinv[g];
    grid_barrier(a.bar, gridDim.x);
    for (long row = gwarp; row < npad; row += nwarps) {
        const long i = row / s, c = row % s;
        T acc = warp_row_dot(a.linvt + i * s * s + c * s + c, a.z + i * s + c, s - c, lane);
        if (lane == 0) a.v[row] = acc;
    }
    grid_barrier(a.bar, gridDim.x);
    // D: x_i -= Rn_i x_{i+1}[0:w]
    for (long i = nb - 2; i >= 0; --i) {
        const T *xn = a.v + (i + 1) * s;
        for (long c = gwarp; c < s; c += nwarps) {
            T acc = warp_row_dot(a.rn + i * s * w + c * w, xn, w, lane);
            if (lane == 0) a.v[i * s + c] -= acc;
        }
        grid_barrier(a.bar, gridDim.x);
    }
    for (long g = gthr; g < a.n; g += nthr) a.out[g] = (double)a.v[g];
}

// -------------------------------------------------------------------------
// Host sequences
// -------------------------------------------------------------------------

template <typename T>
void factor_impl(BandFactor &f, cudaStream_t st, long *launches)
{
    T *band = (T *)f.band;
    T *dinv = (T *)f.dinv;
    T *wbuf = (T *)f.work;  // 32 * bw panel scratch (no solve is live during a factor)
    const long npad = f.nblk * f.s;
    if (npad > f.n) {
        pad_identity_kernel<T><<<(unsigned)((npad - f.n + 127) / 128), 128, 0, st>>>(band, f.ld, f.n, npad);
        ++*launches;
    }
    CB_CUDA(cudaMemsetAsync(f.flags, 0, 2 * sizeof(int), st));
    for (long p = 0; p < npad; p += NB) {
        long m = std::min(f.bw, npad - p - NB);
        if (m < 0) m = 0;
        unsigned nct = (unsigned)std::max(1L, (m + kPanelRows - 1) / kPanelRows);
        panel_kernel<T><<<nct, kPanelThreads, 0, st>>>(band, f.ld, f.bw, p, m, dinv, f.ssd, f.flags, wbuf, f.n,
                                                        (T *)f.stage);
        constexpr int TS = sizeof(T) == 8 ? 16 : 32;
        unsigned nt = (unsigned)std::max(1L, (m + TS - 1) / TS);
        trailing_kernel<T, TS><<<dim3(nt, nt), 256, 0, st>>>(band, f.ld, f.bw, p, m, wbuf, dinv, (const T *)f.stage);
        *launches += 2;
    }
    const long nt = f.s / NB;
    const long kb = (f.bw + NB - 1) / NB + 1;
    inv_diag_kernel<T><<<dim3((unsigned)nt, (unsigned)f.nblk), 32, 0, st>>>(band, f.ld, f.bw, f.s, (T *)f.linv);
    for (long I = 1; I < nt; ++I)
        inv_row_kernel<T><<<dim3((unsigned)I, (unsigned)f.nblk), 256, 0, st>>>(band, f.ld, f.bw, f.s, I, kb,
                                                                               (T *)f.linv);
    *launches += nt;
    transpose_kernel<T><<<dim3((unsigned)nt, (unsigned)nt, (unsigned)f.nblk), 256, 0, st>>>((const T *)f.linv, f.s,
                                                                                        (T *)f.linvt);
    *launches += 1;
    if (f.nblk > 1) {
        dim3 g((unsigned)(f.w / NB), (unsigned)(f.s / NB), (unsigned)(f.nblk - 1));
        pn_kernel<T><<<g, 256, 0, st>>>(band, f.ld, f.bw, f.s, f.w, (const T *)f.linv, (T *)f.pmat);
        rn_kernel<T><<<g, 256, 0, st>>>(band, f.ld, f.bw, f.s, f.w, (const T *)f.linv, (T *)f.rmat);
        *launches += 2;
    }
    CB_CUDA(cudaGetLastError());
}

template <typename T>
void solve_launch(const BandFactor &f, const double *rhs, double *x, void *work, GridBarrier *bar,
                  cudaStream_t st)
{
    const long npad = f.nblk * f.s;
    SolveArgs<T> a;
    a.linv = (const T *)f.linv;
    a.linvt = (const T *)f.linvt;
    a.pn = (const T *)f.pmat;
    a.rn = (const T *)f.rmat;
    a.dinv = (const T *)f.dinv;
    a.s = f.s;
    a.w = f.w;
    a.nblk = f.nblk;
    a.n = f.n;
    a.rhs = rhs;
    a.out = x;
    a.y = (T *)work;
    a.v = a.y + npad;
    a.z = a.v + npad;
    a.bar = bar;
    CB_CUDA(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), st));
    void *args[] = {&a};
    CB_CUDA(cudaLaunchCooperativeKernel((const void *)solve_kernel<T>, dim3((unsigned)f.solve_grid), dim3(256),
                                        args, 0, st));
}

template <typename T>
int max_cooperative_grid()
{
    int dev = 0, sms = 0, per = 0;
    CB_CUDA(cudaGetDevice(&dev));
    CB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, solve_kernel<T>, 256, 0));
    return std::max(1, sms * std::min(per, 4));
}

template <typename T>
void profile_impl(BandFactor &f, int which, cudaStream_t st)
{
    long m = std::min(f.bw, f.nblk * f.s - NB);
    if (m <= 0) return;
    if (which == 3) {  // one trailing update of panel 0 (modifies the factor)
        constexpr int TS = sizeof(T) == 8 ? 16 : 32;
        unsigned nt = (unsigned)((m + TS - 1) / TS);
        trailing_kernel<T, TS><<<dim3(nt, nt), 256, 0, st>>>((T *)f.band, f.ld, f.bw, 0, m, (const T *)f.work,
                                                              (const T *)f.dinv, (const T *)f.stage);
    } else if (which == 4) {  // one panel factor of panel 0 (modifies the factor)
        unsigned nct = (unsigned)std::max(1L, (m + kPanelRows - 1) / kPanelRows);
        panel_kernel<T><<<nct, kPanelThreads, 0, st>>>((T *)f.band, f.ld, f.bw, 0, m, (T *)f.dinv, f.ssd,
                                                        f.flags, (T *)f.work, f.n, (T *)f.stage);
    }
}

}  // namespace

size_t band_work_bytes(const BandFactor &f)
{
    return 256 + 3 * (size_t)f.nblk * f.s * (f.fp32 ? sizeof(float) : sizeof(double));
}

void band_solve_with_work(const BandFactor &f, const double *rhs, double *x, void *work, cudaStream_t st)
{
    // the grid-barrier counters sit in front of the work vectors
    GridBarrier *bar = (GridBarrier *)work;
    void *vecs = (unsigned char *)work + 256;
    if (f.fp32) solve_launch<float>(f, rhs, x, vecs, bar, st);
    else solve_launch<double>(f, rhs, x, vecs, bar, st);
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
    f.w = std::max(32L, ((f.bw + 31) / 32) * 32);
    const size_t es = fp32 ? 4 : 8;
    // Block size of the solve: FP32 uses up to 4 w (fewer sequential steps,
    // bounded by the inverse blocks' memory of n*s elements); FP64 keeps
    // s = w because the FP64 inversion work grows with s^2.
    long s = f.w;
    if (fp32) {
        const double budget = 4.0e9;
        long cap = (long)(budget / ((double)es * (double)std::max(1L, n)));
        s = std::max(f.w, std::min(4 * f.w, (cap / 32) * 32));
    }
    f.s = s;
    f.nblk = (n + f.s - 1) / f.s;
    const long npad = f.nblk * f.s;
    CB_CUDA(cudaMalloc(&f.band, es * (size_t)f.ld * npad));
    CB_CUDA(cudaMalloc(&f.dinv, es * (size_t)npad));
    CB_CUDA(cudaMalloc(&f.linv, es * (size_t)f.nblk * f.s * f.s));
    CB_CUDA(cudaMalloc(&f.linvt, es * (size_t)f.nblk * f.s * f.s));
    CB_CUDA(cudaMalloc(&f.pmat, es * (size_t)f.nblk * f.s * f.w));
    CB_CUDA(cudaMalloc(&f.rmat, es * (size_t)f.nblk * f.s * f.w));
    size_t work = std::max((size_t)3 * npad, (size_t)NB * f.bw + NB);
    CB_CUDA(cudaMalloc(&f.work, es * work));
    CB_CUDA(cudaMalloc(&f.ssd, sizeof(double) * (size_t)n));
    CB_CUDA(cudaMalloc(&f.flags, 2 * sizeof(int)));
    CB_CUDA(cudaMalloc(&f.bar, sizeof(GridBarrier)));
    CB_CUDA(cudaMalloc(&f.stage, es * NB * NB));
    CB_CUDA(cudaMemset(f.linv, 0, es * (size_t)f.nblk * f.s * f.s));
    CB_CUDA(cudaMemset(f.linvt, 0, es * (size_t)f.nblk * f.s * f.s));
    CB_CUDA(cudaMemset(f.pmat, 0, es * (size_t)f.nblk * f.s * f.w));
    CB_CUDA(cudaMemset(f.rmat, 0, es * (size_t)f.nblk * f.s * f.w));
    CB_CUDA(cudaMemset(f.bar, 0, sizeof(GridBarrier)));
    f.solve_grid = fp32 ? max_cooperative_grid<float>() : max_cooperative_grid<double>();
    f.bytes = es * ((size_t)f.ld * npad + npad + (size_t)f.nblk * f.s * (2 * f.s + 2 * f.w) + work);
}

void band_free(BandFactor &f)
{
    if (f.factor_graph) cudaGraphExecDestroy(f.factor_graph);
    for (void *p : {f.band, f.dinv, f.linv, f.linvt, f.pmat, f.rmat, f.work, f.stage, (void *)f.ssd,
                    (void *)f.flags, (void *)f.bar})
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

void band_solve(BandFactor &f, const double *rhs, double *x, cudaStream_t st, bool /*use_graph*/, long *launches)
{
    if (f.fp32) solve_launch<float>(f, rhs, x, f.work, f.bar, st);
    else solve_launch<double>(f, rhs, x, f.work, f.bar, st);
    CB_CUDA(cudaGetLastError());
    if (launches) *launches += 1;
}

}  // namespace cb
