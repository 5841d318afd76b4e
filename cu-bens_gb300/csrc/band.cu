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
// Factor: right-looking over 32-column panels in one persistent cooperative
// kernel with bounded grid barriers between panels (factor_f32_kernel,
// factor_f64_kernel); then the solve blocks below, replayed as a CUDA graph.
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
// run by one persistent cooperative kernel (solve_kernel). Only the w rows of
// each block that feed the next one form the serial recurrence; they run on
// a few CTAs with a barrier of their own, and the other rows follow in
// grid-wide passes. Linv is also kept transposed so both block-diagonal
// products are coalesced row dots. A larger s lowers the number of
// sequential steps while the bytes per step (s*w) and per solve stay about
// the same.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "grid_barrier.cuh"
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

// 1/d from a band that already holds an LDL^T factor (D on the diagonal).
template <typename T>
__global__ void dinv_from_diag_kernel(const T *band, long ld, T *dinv, long npad)
{
    long j = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (j < npad) dinv[j] = T(1) / band[j * ld];
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

// Column sweep of Linv: CTA (i, J) forms tile column J of block i's inverse,
//     X_JJ = T_JJ,   X_IJ = -T_II sum_K L_IK X_KJ   for I = J+1 .. nt-1,
// K in [max(J, I-kb), I), with T_II the inverse diagonal tiles written by
// inv_diag_kernel. The last kb tiles of the column stay in shared memory
// (a ring indexed by K mod kb), so the only global reads on the dependent
// chain are the L tiles and T_II, which do not depend on X and stream in by
// cp.async two chunks ahead of the multiply. Each finished tile goes to linv
// and, transposed through the ring, to linvt. One launch replaces the
// nt - 1 launches of inv_row_kernel plus the transpose.
constexpr int kInvChunk = 4;  // L tiles per cp.async group

__device__ __forceinline__ void cp_async_elem(float *dst, const float *src, bool valid)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}

__device__ __forceinline__ void cp_async_elem(double *dst, const double *src, bool valid)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 8 : 0)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ void lds4(const float *p, float (&v)[4])
{
    const float4 u = *reinterpret_cast<const float4 *>(p);
    v[0] = u.x, v[1] = u.y, v[2] = u.z, v[3] = u.w;
}

__device__ __forceinline__ void lds4(const double *p, double (&v)[4])
{
    const double2 u = *reinterpret_cast<const double2 *>(p);
    const double2 t = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = u.x, v[1] = u.y, v[2] = t.x, v[3] = t.y;
}

// Dynamic shared memory of inv_col_kernel: ring (kb tiles, padded rows),
// two chunks of L tiles (k-major), two T_II tiles, one staging tile.
template <typename T>
size_t inv_col_smem(long kb)
{
    return sizeof(T) * ((size_t)kb * NB * (NB + 1) + 2 * (size_t)kInvChunk * NB * NB + 2 * NB * NB + NB * (NB + 1));
}

template <typename T>
__global__ void __launch_bounds__(256) inv_col_kernel(const T *band, long ld, long bw, long s, long kb, T *linv,
                                                      T *linvt)
{
    extern __shared__ __align__(16) unsigned char inv_smem[];
    constexpr int P = NB + 1;
    T *ring = reinterpret_cast<T *>(inv_smem);  // ring[slot][r][c], row stride P
    T *Ls = ring + kb * NB * P;                 // Ls[buf][t][k][r]: L_IK(r, k)
    T *Ts = Ls + 2 * kInvChunk * NB * NB;       // Ts[I & 1][r][k]: T_II(r, k)
    T *Y = Ts + 2 * NB * NB;                    // Y[r][c], row stride P
    const long i = blockIdx.x, J = blockIdx.y;
    const long nt = s / NB, g0 = i * s;
    T *Li = linv + i * s * s;
    T *Lt = linvt + i * s * s;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    // X_JJ = T_JJ into the ring; its transpose into linvt
    {
        T *X0 = ring + (J % kb) * NB * P;
        for (int q = 0; q < 4; ++q) {
            const int r = w + 8 * q;
            X0[r * P + lane] = Li[(J * NB + r) * s + J * NB + lane];
        }
        __syncthreads();
        for (int q = 0; q < 4; ++q) {
            const int c = w + 8 * q;
            Lt[(J * NB + c) * s + J * NB + lane] = X0[lane * P + c];
        }
    }
    if (J == nt - 1) return;

    auto kfirst = [&](long I) { return I - kb > J ? I - kb : J; };
    // chunk c of step I: L_IK for K = kfirst(I) + c*kInvChunk + t (K < I);
    // the first chunk of a step also brings T_II
    auto issue = [&](long I, long c, int buf) {
        const long K0 = kfirst(I) + c * kInvChunk;
        const long R = g0 + I * NB + lane;
        for (int t = 0; t < kInvChunk; ++t) {
            const long K = K0 + t;
            if (K >= I) break;
            T *dst = Ls + ((long)buf * kInvChunk + t) * NB * NB;
            for (int q = 0; q < 4; ++q) {
                const int k = w + 8 * q;
                const long C = g0 + K * NB + k;
                const long off = R - C;  // >= 1 because K < I
                const bool ok = off <= bw;
                cp_async_elem(dst + k * NB + lane, ok ? band + C * ld + off : band, ok);
            }
        }
        if (c == 0) {
            T *dst = Ts + (I & 1) * NB * NB;
            for (int q = 0; q < 4; ++q) {
                const int r = w + 8 * q;
                cp_async_elem(dst + r * NB + lane, Li + (I * NB + r) * s + I * NB + lane, true);
            }
        }
    };

    long I = J + 1, c = 0;
    int buf = 0;
    issue(I, c, buf);
    cp_async_commit();
    T acc[4] = {0, 0, 0, 0};  // rows 4w .. 4w+3, column lane
    for (;;) {
        long In = I, cn = c + 1;
        if (kfirst(I) + cn * kInvChunk >= I) {
            In = I + 1;
            cn = 0;
        }
        const bool more = In < nt;
        if (more) issue(In, cn, buf ^ 1);
        cp_async_commit();
        cp_async_wait1();
        __syncthreads();
        const long K0 = kfirst(I) + c * kInvChunk;
        for (int t = 0; t < kInvChunk; ++t) {
            const long K = K0 + t;
            if (K >= I) break;
            const T *X = ring + (K % kb) * NB * P + lane;
            const T *A = Ls + ((long)buf * kInvChunk + t) * NB * NB + 4 * w;
#pragma unroll 8
            for (int k = 0; k < NB; ++k) {
                T a[4];
                lds4(A + k * NB, a);
                const T x = X[k * P];
                acc[0] += a[0] * x;
                acc[1] += a[1] * x;
                acc[2] += a[2] * x;
                acc[3] += a[3] * x;
            }
        }
        if (In != I) {
            // step I done: X_IJ = -T_II * acc
            for (int q = 0; q < 4; ++q) {
                Y[(4 * w + q) * P + lane] = acc[q];
                acc[q] = 0;
            }
            __syncthreads();
            const T *Tb = Ts + (I & 1) * NB * NB + 4 * w * NB;
            T v[4] = {0, 0, 0, 0};
            for (int k = 0; k < 4 * w + 4; ++k) {  // T_II(r, k) = 0 for k > r
                const T y = Y[k * P + lane];
                for (int q = 0; q < 4; ++q) v[q] += Tb[q * NB + k] * y;
            }
            T *Xn = ring + (I % kb) * NB * P;
            for (int q = 0; q < 4; ++q) Xn[(4 * w + q) * P + lane] = -v[q];
            __syncthreads();
            for (int q = 0; q < 4; ++q) {
                const int r = w + 8 * q;
                Li[(I * NB + r) * s + J * NB + lane] = Xn[r * P + lane];
            }
            for (int q = 0; q < 4; ++q) {
                const int cc = w + 8 * q;
                Lt[(J * NB + cc) * s + I * NB + lane] = Xn[lane * P + cc];
            }
        }
        __syncthreads();
        if (!more) break;
        I = In;
        c = cn;
        buf ^= 1;
    }
    cp_async_wait0();
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


// -------------------------------------------------------------------------
// Persistent factorisation: one cooperative launch for the whole band
// -------------------------------------------------------------------------

template <typename T>
struct FactorArgs {
    T *band;
    long ld, bw, npad, n;
    T *dinv;
    double *ssd;
    int *flags;
    T *wbuf;     // 32 * bw: W of the current panel (FP64) / staged L rows, two buffers (FP32)
    T *dstage;   // 2 * 32 * 32: staged factored diagonal blocks (FP32)
    T *look;     // 2 * (2 * 32 * 32 + 32): the next panel's factored diagonal block, Linv, 1/D (FP32)
    GridBarrier *bar;
    int dist;    // FP32: panel rows formed once per panel (wide bands) instead of per tile
    long long max_polls;  // bound of each grid-barrier wait (grid_barrier)
};

// Tile t of the lower triangle of an nt x nt tile grid: t = ti (ti + 1) / 2 + tj.
__device__ __forceinline__ void tile_of(long t, long &ti, long &tj)
{
    ti = (long)((sqrt(8.0 * (double)t + 1.0) - 1.0) / 2.0);
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    while (ti * (ti + 1) / 2 > t) --ti;
    tj = t - ti * (ti + 1) / 2;
}

// 1, 1/d and the pivots of panel p, from the factored block A (D on the diagonal).
template <typename T>
__device__ __forceinline__ void record_pivots(const FactorArgs<T> &a, long p, T dl, T rd, int i)
{
    a.dinv[p + i] = rd;
    const long g = p + i;
    if (g < a.n) {
        a.ssd[g] = (double)dl;
        if (!(dl > T(0))) atomicOr(&a.flags[0], 1);
        if (dl == T(0)) atomicOr(&a.flags[1], 1);
    }
}

__device__ __noinline__ void ldlt32_noinv(float (*A)[NB + 1], float *di);

// Inverse of the unit-lower L held below the diagonal of A (one warp, lane
// j forms column j: x_rr = -sum_{k<rr} L_rr,k x_k, summed in four chains of
// k mod 4), into Li (row-major).
__device__ __noinline__ void linv32_warp(const float (*A)[NB + 1], float (*Li)[NB + 1])
{
    const int lane = threadIdx.x % 32;
    float x[NB];
#pragma unroll
    for (int rr = 0; rr < NB; ++rr) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // four chains of k mod 4
#pragma unroll
        for (int k = 0; k < rr; ++k) acc[k & 3] += A[rr][k] * x[k];
        const float s = (acc[0] + acc[1]) + (acc[2] + acc[3]);
        x[rr] = rr == lane ? 1.0f : (rr < lane ? 0.0f : -s);
    }
#pragma unroll
    for (int j = 0; j < NB; ++j) Li[j][lane] = x[j];
}

// LDL^T and the inverse of L in two steps (no register spills in either)
__device__ __forceinline__ void ldlt32_split(float (*A)[NB + 1], float (*Li)[NB + 1], float *di)
{
    ldlt32_noinv(A, di);
    __syncwarp();
    linv32_warp(A, Li);
}

// FP32: one grid barrier per 32-column panel p (m = min(bw, npad - p - 32)).
//   1. the panel's factored diagonal block, the inverse of its unit-lower
//      factor and 1/D: factored by every CTA for the first panel (warp 0:
//      ldlt32_noinv, then linv32_warp), afterwards read from the look-ahead
//      buffer that CTA 0 filled in step 3 of the previous panel;
//   2. each CTA takes TS x TS tiles (ti, tj) of the trailing lower triangle,
//      forms the panel rows it needs from the band, W = A Linv^T (= L D) for
//      the tile's rows and L = W D^-1 for its columns, and applies
//      A_rj -= sum_k W_rk L_jk. The owner of a diagonal tile stages its L
//      rows: other CTAs still read the panel's A values from the band during
//      this phase;
//   3. CTA 0, whose tile (0,0) is the next panel's diagonal block (final once
//      CTA 0 has applied this panel to it), factors that block, records its
//      pivots, stages it and publishes it with its inverse;
//   -- grid barrier --
//   0. (next panel) all CTAs copy the staged L rows and block into the band.
template <int TS>
__global__ void __launch_bounds__(256) factor_f32_kernel(FactorArgs<float> a)
{
    unsigned ep = 0;  // grid barriers passed
    using T = float;
    __shared__ T A[NB][NB + 1];   // factored diagonal block: L below, D on the diagonal
    __shared__ T Li[NB][NB + 1];  // Linv of the unit-lower L_pp
    __shared__ T di[NB];
    __shared__ T Ar[TS][NB + 1];  // raw panel rows of the tile's row block, then W
    __shared__ T Ac[TS][NB + 1];  // raw panel rows of the tile's column block, then L
    __shared__ T Bo[TS][TS + 1];  // the first tile's band values before this panel's update
    __shared__ T Wd[NB][64];      // wide bands: W of a 64-row block (k-major)
    __shared__ T Ld[NB][64];      // wide bands: L of a 64-column block
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const long ld = a.ld, bw = a.bw;
    long mprev = 0;
    for (long p = 0; p <= a.npad; p += NB) {
        // the look-ahead block of this panel (step 3 of the previous one:
        // L, D and 1/D) comes into shared memory by cp.async, overlapping
        // the staged copy; CTA 0 still holds it in A and di
        const bool look = !a.dist && p > 0 && p < a.npad;
        if (look && blockIdx.x != 0) {
            const T *lk = a.look + (int)((p / NB) & 1) * (NB * NB + NB);
            for (int e = tid; e < NB * NB; e += 256) cp_async_elem(&A[e / NB][e % NB], lk + e, true);
            if (tid < NB) cp_async_elem(&di[tid], lk + NB * NB + tid, true);
        }
        cp_async_commit();
        long m = a.npad - p - NB;
        if (m > bw) m = bw;
        if (m < 0) m = 0;
        // the first trailing tile's inputs are final at the barrier (the
        // staged copy below writes only the previous panel's columns): its
        // raw panel rows and the band values it updates come in by cp.async
        // too, so the tile starts with its data on chip
        const long nt_first = (m + TS - 1) / TS;
        const bool first_pre = !a.dist && p < a.npad && blockIdx.x < nt_first * (nt_first + 1) / 2;
        if (first_pre) {
            long ti, tj;
            tile_of((long)blockIdx.x, ti, tj);
            const long r0 = ti * TS, j0 = tj * TS;
            for (int idx = tid; idx < NB * TS; idx += 256) {
                const int k = idx / TS, q = idx % TS;
                const long o1 = NB + r0 + q - k, o2 = NB + j0 + q - k;
                const bool v1 = r0 + q < m && o1 <= bw, v2 = j0 + q < m && o2 <= bw;
                cp_async_elem(&Ar[q][k], v1 ? a.band + (p + k) * ld + o1 : a.band, v1);
                cp_async_elem(&Ac[q][k], v2 ? a.band + (p + k) * ld + o2 : a.band, v2);
            }
            for (int idx = tid; idx < TS * TS; idx += 256) {
                const int ji = idx / TS, ri = idx % TS;
                const long rr = r0 + ri, jj = j0 + ji;
                const bool v = rr < m && jj < m && jj <= rr;
                cp_async_elem(&Bo[ri][ji], v ? a.band + (p + NB + jj) * ld + (rr - jj) : a.band, v);
            }
        }
        cp_async_commit();
        // ---- 0. staged output of the previous panel into the band (CTA 0,
        //         the look-ahead's owner, stays out when there are others) ----
        const unsigned c0 = gridDim.x > 1 ? 1u : 0u;  // (the tile's group)
        if (p > 0 && !a.dist && blockIdx.x >= c0) {
            const long pp = p - NB;
            const int buf = (int)((pp / NB) & 1);
            const T *ls = a.wbuf + (long)buf * NB * bw;
            const T *ds = a.dstage + buf * NB * NB;
            const long total = NB * NB + NB * mprev;
            for (long idx = (blockIdx.x - c0) * 256L + tid; idx < total; idx += (gridDim.x - c0) * 256L) {
                if (idx < NB * NB) {
                    const int j = (int)(idx / NB), i = (int)(idx % NB);
                    if (i >= j && i - j <= bw) a.band[(pp + j) * ld + (i - j)] = ds[idx];
                } else {
                    const long q = idx - NB * NB;
                    const int c = (int)(q / mprev);
                    const long r = q % mprev;
                    const long off = NB + r - c;
                    if (off <= bw) a.band[(pp + c) * ld + off] = ls[c * mprev + r];
                }
            }
        }
        if (p == a.npad) break;
        const int buf = (int)((p / NB) & 1);
        // ---- 1. diagonal block: LDL^T and Linv by warp 0 in registers; on
        //         the narrow path after the first panel CTA 0 has factored it
        //         ahead (step 3), and every CTA forms Linv from its L while
        //         the first tile's inputs are still on their way ----
        if (look) {
            cp_async_wait1();  // the look-ahead block
            __syncthreads();
            if (warp == 0) linv32_warp(A, Li);
            cp_async_wait0();  // the first tile's inputs
            __syncthreads();
        } else {
            cp_async_wait0();
            for (int e = tid; e < NB * NB; e += 256) {
                const int jj = e / NB, ii = e % NB;
                A[ii][jj] = (ii >= jj && ii - jj <= bw) ? a.band[(p + jj) * ld + (ii - jj)] : T(0);
            }
            __syncthreads();
            if (warp == 0) {
                ldlt32_split(A, Li, di);
                if (blockIdx.x == 0) record_pivots(a, p, A[lane][lane], di[lane], lane);
            }
            __syncthreads();
            if (blockIdx.x == 0 && !a.dist) {
                T *ds = a.dstage + buf * NB * NB;
                for (int idx = tid; idx < NB * NB; idx += 256) ds[idx] = A[idx % NB][idx / NB];
            }
        }
        if (a.dist) {
            // ---- 2'. wide band: panel rows once, one warp per row; W to wbuf,
            //          L into the band (no other CTA reads this panel's A) ----
            const long gwarp = blockIdx.x * 8L + warp, nwarps = gridDim.x * 8L;
            for (long r = gwarp; r < m; r += nwarps) {
                const long off = NB + r - lane;
                const T ar = off <= bw ? a.band[(p + lane) * ld + off] : T(0);
                T w = 0;
                for (int k = 0; k < NB; ++k) {
                    const T v = __shfl_sync(0xffffffffu, ar, k);
                    if (k <= lane) w += v * Li[lane][k];
                }
                a.wbuf[lane * m + r] = w;
                if (off <= bw) a.band[(p + lane) * ld + off] = w * di[lane];
            }
            if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
            if (blockIdx.x == 0)
                for (int idx = tid; idx < NB * NB; idx += 256) {
                    const int j = idx / NB, i = idx % NB;
                    if (i >= j && i - j <= bw) a.band[(p + j) * ld + (i - j)] = A[i][j];
                }
            // 64 x 64 tiles, a 4 x 4 register block per thread: rows
            // r0 + tx + 16 i (consecutive threads, consecutive rows of a
            // column), columns j0 + ty + 16 j
            constexpr int WT = 64;
            const int tx = tid % 16, ty = tid / 16;
            const long nt = (m + WT - 1) / WT;
            const long ntiles = nt * (nt + 1) / 2;
            for (long t = blockIdx.x; t < ntiles; t += gridDim.x) {
                long ti, tj;
                tile_of(t, ti, tj);
                const long r0 = ti * WT, j0 = tj * WT;
                for (int idx = tid; idx < NB * WT; idx += 256) {
                    const int k = idx / WT, q = idx % WT;
                    const long rr = r0 + q, jj = j0 + q;
                    Wd[k][q] = rr < m ? a.wbuf[k * m + rr] : T(0);
                    Ld[k][q] = jj < m ? a.wbuf[k * m + jj] * di[k] : T(0);
                }
                __syncthreads();
                T acc[4][4];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = 0;
#pragma unroll 8
                for (int k = 0; k < NB; ++k) {
                    T wv[4], lv[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        wv[i] = Wd[k][tx + 16 * i];
                        lv[i] = Ld[k][ty + 16 * i];
                    }
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] += wv[i] * lv[j];
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const long jj = j0 + ty + 16 * j;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const long rr = r0 + tx + 16 * i;
                        if (rr < m && jj < m && jj <= rr) a.band[(p + NB + jj) * ld + (rr - jj)] -= acc[i][j];
                    }
                }
                __syncthreads();
            }
            if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
            continue;
        }
        // ---- 2. trailing tiles ----
        T *ls = a.wbuf + (long)buf * NB * bw;
        const long nt = (m + TS - 1) / TS;
        const long ntiles = nt * (nt + 1) / 2;
        for (long t = blockIdx.x; t < ntiles; t += gridDim.x) {
            long ti, tj;
            tile_of(t, ti, tj);
            const long r0 = ti * TS, j0 = tj * TS;
            const bool pre = t == blockIdx.x && first_pre;  // inputs already on chip
            // raw panel rows: X[q][k] = A(p+32+r0+q, p+k)
            if (!pre)
                for (int idx = tid; idx < NB * TS; idx += 256) {
                    const int k = idx / TS, q = idx % TS;
                    const long o1 = NB + r0 + q - k, o2 = NB + j0 + q - k;
                    Ar[q][k] = (r0 + q < m && o1 <= bw) ? a.band[(p + k) * ld + o1] : T(0);
                    Ac[q][k] = (j0 + q < m && o2 <= bw) ? a.band[(p + k) * ld + o2] : T(0);
                }
            __syncthreads();
            // W = X Linv^T for the row block, L = W D^-1 for the column block:
            // thread (warp, lane) forms row lane, columns warp + 8u, in eight
            // independent chains (Linv's upper triangle holds zeros)
            static_assert(TS == NB, "32 x 32 trailing tiles");
            T wv[4] = {0, 0, 0, 0}, lv[4] = {0, 0, 0, 0};
            if (ti == tj) {  // a diagonal tile: its row and column blocks are the same rows
#pragma unroll 8
                for (int k = 0; k < NB; ++k) {
                    const T x1 = Ar[lane][k];
#pragma unroll
                    for (int u = 0; u < 4; ++u) wv[u] += x1 * Li[warp + 8 * u][k];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) lv[u] = wv[u];
            } else {
#pragma unroll 8
                for (int k = 0; k < NB; ++k) {
                    const T x1 = Ar[lane][k], x2 = Ac[lane][k];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const T li = Li[warp + 8 * u][k];
                        wv[u] += x1 * li;
                        lv[u] += x2 * li;
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int c = warp + 8 * u;
                lv[u] *= di[c];
                Ar[lane][c] = wv[u];
                Ac[lane][c] = lv[u];
                if (ti == tj && j0 + lane < m) ls[c * m + j0 + lane] = lv[u];
            }
            __syncthreads();
            // the update, row lane and columns warp + 8u of the tile; tile (0,0)
            // is the next panel's diagonal block: with m >= 32 it is complete
            // here, and CTA 0 keeps it in A for the look-ahead
            const bool keep = t == 0 && m >= NB;
            T acc[4] = {0, 0, 0, 0};
#pragma unroll 8
            for (int k = 0; k < NB; ++k) {
                const T x = Ar[lane][k];
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[u] += x * Ac[warp + 8 * u][k];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int ri = lane, ji = warp + 8 * u;
                const long rr = r0 + ri, jj = j0 + ji;
                if (keep && ji > ri) A[ri][ji] = T(0);
                if (rr >= m || jj >= m || jj > rr) continue;
                T *slot = a.band + (p + NB + jj) * ld + (rr - jj);
                const T nv = (pre ? Bo[ri][ji] : *slot) - acc[u];
                *slot = nv;
                if (keep) A[ri][ji] = nv;
            }
            __syncthreads();
        }
        // ---- 3. look-ahead (CTA 0, whose first tile (0,0) is the next panel's
        //         diagonal block, final now): factor it before the barrier,
        //         record its pivots, stage it, publish L, D and 1/D ----
        if (blockIdx.x == 0 && m > 0) {
            const long pn = p + NB;
            const int bn = (int)((pn / NB) & 1);
            __syncthreads();
            if (m < NB) {  // a band narrower than a panel: not all of the block was in tile (0,0)
                for (int e = tid; e < NB * NB; e += 256) {
                    const int jj = e / NB, ii = e % NB;
                    A[ii][jj] = (ii >= jj && ii - jj <= bw) ? a.band[(pn + jj) * ld + (ii - jj)] : T(0);
                }
                __syncthreads();
            }
            if (warp == 0) {
                ldlt32_noinv(A, di);
                record_pivots(a, pn, A[lane][lane], di[lane], lane);
            }
            __syncthreads();
            T *ds = a.dstage + bn * NB * NB;
            T *lk = a.look + bn * (NB * NB + NB);
            for (int idx = tid; idx < NB * NB; idx += 256) {
                ds[idx] = A[idx % NB][idx / NB];
                lk[idx] = A[idx / NB][idx % NB];
            }
            if (tid < NB) lk[NB * NB + tid] = di[tid];
        }
        mprev = m;
        if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    }
}

// LDL^T of a 32x32 block in shared memory by one warp in registers (lane i
// holds row i, l_jk by shuffle), without the inverse of L: the grid factor
// forms it next with linv32_warp, the cluster factor substitutes instead.
// On return A holds L below and D on the diagonal, di = 1/D.
__device__ __noinline__ void ldlt32_noinv(float (*A)[NB + 1], float *di)
{
    const int lane = threadIdx.x % 32;
    float r[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) r[j] = A[lane][j];
#pragma unroll
    for (int k = 0; k < NB; ++k) {
        // row j's unscaled column-k entry c_j = l_jk d_k gives the update
        // l_ik d_k l_jk = l_ik c_j, so the broadcasts of c_j need only the
        // previous step's update, not this step's reciprocal
        const float rk = r[k];
        // the hardware's approximate 1/d (rcp.approx.ftz, within an ulp or so):
        // it only scales this column's L entries, so the correctly rounded
        // reciprocal's extra steps stay off the panel's serial chain; D and
        // 1/D themselves are exact below
        float rd;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rd) : "f"(__shfl_sync(0xffffffffu, rk, k)));
        const float l = lane > k ? rk * rd : 0.0f;
        if (lane > k) r[k] = l;
#pragma unroll
        for (int j = k + 1; j < NB; ++j) {
            const float cj = __shfl_sync(0xffffffffu, rk, j);
            if (j <= lane) r[j] -= l * cj;
        }
    }
    float dl = 0;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
        A[lane][j] = j <= lane ? r[j] : 0.0f;
        if (j == lane) dl = r[j];
    }
    di[lane] = __frcp_rn(dl);
}

// FP32 narrow bands: one thread-block cluster of C CTAs holds the active
// window of the band in its distributed shared memory.
//   - CTA o owns the 32-column blocks B = o, o + C, o + 2C, ...; block B lives
//     in slot (B / C) % nslot of its owner (32 band columns, ld rows each,
//     the band's own layout) from its load until it is factored;
//   - panel b: its owner factors the diagonal block (ldlt32_noinv), forms
//     the panel rows W (W L^T = A, by substitution) and L = W D^-1 into its
//     slot, publishes W and 1/D in its shared memory, writes the finished
//     block back to the band and loads the owned block (nslot - 1) C ahead
//     into the slot it frees;
//   -- cluster barrier --
//   - every CTA applies A_ij -= sum_k W_ik W_jk / d_k to its own blocks in
//     the window (b, b + nwin], reading W through distributed shared memory.
// One hardware cluster barrier per panel and no grid-wide synchronisation;
// each band entry is read from and written to HBM once. The owner of block
// b+1 applies panel b to it before factoring it, in program order, so one
// barrier per panel is enough: a CTA rewrites its W only C panels later,
// after every CTA has passed C barriers.
struct ClusterArgs {
    FactorArgs<float> f;
    int nslot, nwin;
};

constexpr int kClusterThreads = 256;
constexpr int kWs = NB + 4;  // row stride of W rows in shared memory (16-byte aligned rows)

// dst[e] = src[e] for e in [e0, e1) (float4), eight loads in flight per
// thread before their stores (the source may be global or another CTA's
// shared memory)
__device__ __forceinline__ void copy4(float4 *dst, const float4 *src, long e0, long e1)
{
    const long step = blockDim.x;
    for (long base = e0 + threadIdx.x; base < e1; base += 8 * step) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const long e = base + u * step;
            if (e < e1) v[u] = src[e];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const long e = base + u * step;
            if (e < e1) dst[e] = v[u];
        }
    }
}

__device__ __forceinline__ void copy_block_in(const float *__restrict__ band, long ld, long B, float *slot)
{
    copy4(reinterpret_cast<float4 *>(slot), reinterpret_cast<const float4 *>(band + (size_t)B * NB * ld), 0,
          (long)NB * ld / 4);
}

__device__ __forceinline__ void copy_block_out(float *__restrict__ band, long ld, long B, const float *slot)
{
    float4 *dst = reinterpret_cast<float4 *>(band + (size_t)B * NB * ld);
    const float4 *src = reinterpret_cast<const float4 *>(slot);
    const long n4 = (long)NB * ld / 4;
    for (long e = threadIdx.x; e < n4; e += blockDim.x) dst[e] = src[e];
}

// Panel row r (band row 32(b+1) + r of block b's columns): W_r L^T = A_r by
// substitution with the unit-lower L of the diagonal block; W_r to wout,
// L_r = W_r D^-1 over A_r in the slot.
__device__ __noinline__ void panel_row(float *S, long ld, long bw, long r, const float (*L)[NB + 1],
                                       const float *di, float *wout)
{
    float w[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        const long off = NB + r - c;
        float x = off <= bw ? S[(size_t)c * ld + off] : 0.0f;
#pragma unroll
        for (int k = 0; k < c; ++k) x -= w[k] * L[c][k];
        w[c] = x;
    }
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        const long off = NB + r - c;
        wout[c] = w[c];
        if (off <= bw) S[(size_t)c * ld + off] = w[c] * di[c];
    }
}

// A_ij -= sum_k W_ik W_jk / d_k for the 32 columns j of a block (W rows of the
// columns at panel row c0..c0+31) and its rows c0..r1-1 (panel rows), from
// the W rows in Wl (local copy) and LjT[k][j] = W_jk / d_k. 128 rows per
// pass, a 4x4 register block per thread.
__device__ void update_block(float *S, long ld, long bw, const float *Wl, const float (*LjT)[kWs], long c0,
                             long r1)
{
    const int tr = threadIdx.x >> 3, tc = threadIdx.x & 7;
    for (long rb = c0; rb < r1; rb += 128) {
        float acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
        long rr[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            rr[i] = rb + 4 * tr + i;
            if (rr[i] >= r1) rr[i] = r1 - 1;  // clamped rows compute a copy, not stored
        }
#pragma unroll 8
        for (int k = 0; k < NB; ++k) {
            const float4 l = *reinterpret_cast<const float4 *>(&LjT[k][4 * tc]);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float w = Wl[rr[i] * kWs + k];
                acc[i][0] += w * l.x;
                acc[i][1] += w * l.y;
                acc[i][2] += w * l.z;
                acc[i][3] += w * l.w;
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const long r = rb + 4 * tr + i;
            if (r >= r1) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const long jj = 4 * tc + j;
                const long off = r - (c0 + jj);
                if (off >= 0 && off <= bw) S[(size_t)jj * ld + off] -= acc[i][j];
            }
        }
    }
}

__global__ void __launch_bounds__(kClusterThreads) factor_cluster_kernel(ClusterArgs ca)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const FactorArgs<float> &a = ca.f;
    const int C = (int)cl.num_blocks(), o = (int)cl.block_rank();
    const int nslot = ca.nslot;
    const long ld = a.ld, bw = a.bw, nb = a.npad / NB;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    extern __shared__ float4 dsm4[];
    float *slots = reinterpret_cast<float *>(dsm4);           // nslot x 32 x ld
    float *Wb = slots + (size_t)nslot * NB * ld;               // bw x kWs: this CTA's last panel rows W
    float *Wl = Wb + (size_t)bw * kWs;                         // bw x kWs: a local copy of the owner's W
    float *dib = Wl + (size_t)bw * kWs;                        // 32: 1/D of this CTA's last panel
    __shared__ float A[NB][NB + 1];
    __shared__ float di[NB];
    __shared__ __align__(16) float LjT[NB][kWs];  // L rows of the updated block's columns, k-major
    for (int k = 0; k < nslot - 1; ++k) {
        const long B = o + (long)k * C;
        if (B < nb) copy_block_in(a.band, ld, B, slots + (size_t)k * NB * ld);
    }
    __syncthreads();
    for (long b = 0; b < nb; ++b) {
        const int owner = (int)(b % C);
        long m = a.npad - NB * (b + 1);
        if (m > bw) m = bw;
        if (o == owner) {
            const long kk = b / C;
            float *S = slots + (size_t)(kk % nslot) * NB * ld;
            for (int e = tid; e < NB * NB; e += blockDim.x) {
                const int j = e / NB, i = e % NB;
                A[i][j] = (i >= j && i - j <= bw) ? S[(size_t)j * ld + (i - j)] : 0.0f;
            }
            __syncthreads();
            if (warp == 0) {
                ldlt32_noinv(A, di);
                record_pivots(a, b * NB, A[lane][lane], di[lane], lane);
            }
            __syncthreads();
            for (int e = tid; e < NB * NB; e += blockDim.x) {
                const int j = e / NB, i = e % NB;
                if (i >= j && i - j <= bw) S[(size_t)j * ld + (i - j)] = A[i][j];
            }
            for (long r = tid; r < m; r += blockDim.x) panel_row(S, ld, bw, r, A, di, Wb + r * kWs);
            if (tid < NB) dib[tid] = di[tid];
            __syncthreads();
        }
        cl.sync();
        const long first = b + 1 + (((long)o - (b + 1)) % C + C) % C;  // first owned block after b
        const bool work = first <= b + ca.nwin && first < nb && NB * (first - b - 1) < m;
        if (work) {
            // the owner's W rows from this block's first column on, one pass
            const long c0f = NB * (first - b - 1);
            const float4 *src = reinterpret_cast<const float4 *>(cl.map_shared_rank(Wb, owner));
            float4 *dst = reinterpret_cast<float4 *>(Wl);
            copy4(dst, src, c0f * (kWs / 4), m * (kWs / 4));
            const float *dio = cl.map_shared_rank(dib, owner);
            if (tid < NB) A[0][tid] = dio[tid];  // the owner's 1/D (A is free outside the owner's factor)
            __syncthreads();
            for (long B = first; B <= b + ca.nwin && B < nb; B += C) {
                const long c0 = NB * (B - b - 1);
                if (c0 >= m) break;
                float *S = slots + (size_t)((B / C) % nslot) * NB * ld;
                for (int e = tid; e < NB * NB; e += blockDim.x) {
                    const int jj = e / NB, k = e % NB;
                    LjT[k][jj] = c0 + jj < m ? Wl[(c0 + jj) * kWs + k] * A[0][k] : 0.0f;
                }
                __syncthreads();
                long r1 = c0 + NB + bw;
                if (r1 > m) r1 = m;
                update_block(S, ld, bw, Wl, LjT, c0, r1);
                __syncthreads();
            }
        }
        if (o == owner) {
            // the finished block to the band; the owned block nslot - 1 turns
            // ahead into the slot of the previous one (finished and written)
            const long kk = b / C;
            copy_block_out(a.band, ld, b, slots + (size_t)(kk % nslot) * NB * ld);
            const long Bn = b + (long)(nslot - 1) * C;
            if (Bn < nb) copy_block_in(a.band, ld, Bn, slots + (size_t)((kk + nslot - 1) % nslot) * NB * ld);
            __syncthreads();
        }
    }
    // no CTA leaves while another may still read its shared memory
    cl.sync();
}

// FP64 (the FP64 pipe is the bound): two grid barriers per panel.
//   1. every CTA factors the diagonal block with all 256 threads (one
//      elimination step per column, warp-uniform columns);
//   2. one warp per panel row r forms W_r by forward substitution with the
//      unit-lower L_pp (W_r L_pp^T = A_r), writes L_r = W_r D^-1 into the band
//      and W_r into wbuf;
//   -- grid barrier --
//   3. CTA 0 writes the diagonal block and pivots; the CTAs share the TS x TS
//      tiles of the trailing update from wbuf;
//   -- grid barrier --
template <int TS>
__global__ void __launch_bounds__(256) factor_f64_kernel(FactorArgs<double> a)
{
    unsigned ep = 0;  // grid barriers passed
    using T = double;
    __shared__ T A[NB][NB + 1];
    __shared__ T di[NB];
    __shared__ T Wr[TS][NB + 1];
    __shared__ T Lc[TS][NB + 1];
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const long ld = a.ld, bw = a.bw;
    const long gwarp = blockIdx.x * 8L + warp, nwarps = gridDim.x * 8L;
    for (long p = 0; p < a.npad; p += NB) {
        long m = a.npad - p - NB;
        if (m > bw) m = bw;
        if (m < 0) m = 0;
        // ---- 1. diagonal block, all threads; entry e: column e / 32 (warp-uniform), row e % 32 ----
        for (int e = tid; e < NB * NB; e += 256) {
            const int j = e / NB, i = e % NB;
            A[i][j] = (i >= j && i - j <= bw) ? a.band[(p + j) * ld + (i - j)] : T(0);
        }
        __syncthreads();
        for (int k = 0; k < NB; ++k) {
            const T d = A[k][k];
            if (warp == 0 && lane > k) A[lane][k] = A[lane][k] / d;
            __syncthreads();
            for (int e = tid; e < NB * NB; e += 256) {
                const int j = e / NB, i = e % NB;
                if (j > k && j <= i) A[i][j] -= (A[i][k] * d) * A[j][k];
            }
            __syncthreads();
        }
        if (tid < NB) di[tid] = T(1) / A[tid][tid];
        __syncthreads();
        // ---- 2. panel rows by substitution, one warp per row ----
        for (long r = gwarp; r < m; r += nwarps) {
            const long off = NB + r - lane;
            T w = off <= bw ? a.band[(p + lane) * ld + off] : T(0);
            for (int k = 0; k < NB; ++k) {
                const T wk = __shfl_sync(0xffffffffu, w, k);
                if (lane > k) w -= wk * A[lane][k];
            }
            a.wbuf[lane * m + r] = w;
            if (off <= bw) a.band[(p + lane) * ld + off] = w * di[lane];
        }
        if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
        // ---- 3. diagonal block out, trailing update ----
        if (blockIdx.x == 0) {
            for (int e = tid; e < NB * NB; e += 256) {
                const int j = e / NB, i = e % NB;
                if (i >= j && i - j <= bw) a.band[(p + j) * ld + (i - j)] = A[i][j];
            }
            if (tid < NB) record_pivots(a, p, A[tid][tid], di[tid], tid);
        }
        const long nt = (m + TS - 1) / TS;
        const long ntiles = nt * (nt + 1) / 2;
        for (long t = blockIdx.x; t < ntiles; t += gridDim.x) {
            long ti, tj;
            tile_of(t, ti, tj);
            const long r0 = ti * TS, j0 = tj * TS;
            for (int idx = tid; idx < NB * TS; idx += 256) {
                const int k = idx / TS, q = idx % TS;
                const long rr = r0 + q, jj = j0 + q;
                Wr[q][k] = rr < m ? a.wbuf[k * m + rr] : T(0);
                Lc[q][k] = jj < m ? a.wbuf[k * m + jj] * di[k] : T(0);
            }
            __syncthreads();
            for (int idx = tid; idx < TS * TS; idx += 256) {
                const int ji = idx / TS, ri = idx % TS;
                const long rr = r0 + ri, jj = j0 + ji;
                if (rr >= m || jj >= m || jj > rr) continue;
                T acc = 0;
#pragma unroll 8
                for (int k = 0; k < NB; ++k) acc += Wr[ri][k] * Lc[ji][k];
                a.band[(p + NB + jj) * ld + (rr - jj)] -= acc;
            }
            __syncthreads();
        }
        if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    }
}

// Direct substitution with the band factor, for a factorisation that serves
// one solve (no block inverses): L y = b right-looking over 32-row panels
// (the panel's unit-lower block solved by warp 0 of every CTA, then the
// rows below updated), z = D^-1 y, then L^T x = z right-looking from the
// last panel (the block solved, then the bw rows above updated). One grid
// barrier per panel each way.
template <typename T>
struct DirectArgs {
    const T *band, *dinv;
    long ld, bw, npad, n;
    const double *rhs;
    double *out;
    T *y;
    GridBarrier *bar;
    long long max_polls;
};

template <typename T>
__global__ void __launch_bounds__(256) solve_direct_kernel(DirectArgs<T> a)
{
    unsigned ep = 0;  // grid barriers passed
    __shared__ T yp[NB];
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const long ld = a.ld, bw = a.bw, npad = a.npad;
    const long gthr = blockIdx.x * 256L + tid, nthr = gridDim.x * 256L;
    for (long g = gthr; g < npad; g += nthr) a.y[g] = g < a.n ? (T)a.rhs[g] : T(0);
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    // forward: y_p = L_pp^-1 y_p; y_r -= L(r, p..p+31) y_p for the rows below
    for (long p = 0; p < npad; p += NB) {
        long m = npad - p - NB;
        if (m > bw) m = bw;
        if (m < 0) m = 0;
        if (warp == 0) {
            T l[NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) l[k] = (k < lane && lane - k <= bw) ? a.band[(p + k) * ld + (lane - k)] : T(0);
            T v = a.y[p + lane];
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                const T vk = __shfl_sync(0xffffffffu, v, k);
                if (lane > k) v -= l[k] * vk;
            }
            yp[lane] = v;
        }
        __syncthreads();
        if (blockIdx.x == 0 && tid < NB) a.y[p + tid] = yp[tid];
        for (long r = gthr; r < m; r += nthr) {
            T acc = 0;
#pragma unroll 8
            for (int k = 0; k < NB; ++k) {
                const long off = NB + r - k;
                if (off <= bw) acc += a.band[(p + k) * ld + off] * yp[k];
            }
            a.y[p + NB + r] -= acc;
        }
        if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    }
    for (long g = gthr; g < npad; g += nthr) a.y[g] *= a.dinv[g];
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    // backward: x_p = L_pp^-T z_p; z_j -= sum_i L(p+i, j) x_i for j in [p-bw, p)
    for (long p = npad - NB; p >= 0; p -= NB) {
        if (warp == 0) {
            // lane k holds z_k; column k of the block: L(p+i, p+k), i > k
            T l[NB];
#pragma unroll
            for (int i = 0; i < NB; ++i) l[i] = (i > lane && i - lane <= bw) ? a.band[(p + lane) * ld + (i - lane)] : T(0);
            T v = a.y[p + lane];
#pragma unroll
            for (int i = NB - 1; i >= 0; --i) {
                const T xi = __shfl_sync(0xffffffffu, v, i);
                if (lane < i) v -= l[i] * xi;
            }
            yp[lane] = v;
        }
        __syncthreads();
        if (blockIdx.x == 0 && tid < NB) a.y[p + tid] = yp[tid];
        const long jlo = p - bw > 0 ? p - bw : 0;
        for (long j = jlo + gthr; j < p; j += nthr) {
            T acc = 0;
            const long base = p - j;  // band offset of L(p, j)
#pragma unroll 8
            for (int i = 0; i < NB; ++i)
                if (base + i <= bw) acc += a.band[j * ld + base + i] * yp[i];
            a.y[j] -= acc;
        }
        if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    }
    for (long g = gthr; g < a.n; g += nthr) a.out[g] = (double)a.y[g];
}

template <typename T>
struct SolveArgs {
    const T *linv, *linvt, *pn, *rn, *dinv;
    long s, w, nblk, n;
    const double *rhs;
    double *out;
    T *y, *v, *z;
    GridBarrier *bar;
    long long max_polls;
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

// The chain rows of the block-bidiagonal solve: a warp holds its row of the
// next step in registers (the first 32 * row_regs<T>() entries), loaded before
// the barrier that ends the current step, so a step waits on the vector only.
template <typename T>
constexpr int row_regs()
{
    return sizeof(T) == 4 ? 16 : 8;
}

template <typename T>
__device__ __forceinline__ void row_to_regs(T (&pre)[row_regs<T>()], const T *__restrict__ row, long len, int lane)
{
#pragma unroll
    for (int u = 0; u < row_regs<T>(); ++u) {
        const long j = lane + 32L * u;
        pre[u] = j < len ? row[j] : T(0);
    }
}

template <typename T>
__device__ __forceinline__ T regs_row_dot(const T (&pre)[row_regs<T>()], const T *__restrict__ row,
                                          const T *__restrict__ vec, long len, int lane)
{
    T acc[4] = {0, 0, 0, 0};
#pragma unroll
    for (int u = 0; u < row_regs<T>(); ++u) {
        const long j = lane + 32L * u;
        if (j < len) acc[u & 3] += pre[u] * vec[j];
    }
    for (long j = lane + 32L * row_regs<T>(); j < len; j += 32) acc[0] += row[j] * vec[j];
    return warp_reduce((acc[0] + acc[1]) + (acc[2] + acc[3]));
}

// Block-bidiagonal solve in one cooperative launch:
//   A  y_i = Linv_i b_i                                 (all rows)
//   B  y_i[s-w:s] -= Pn_i[s-w:s] y_{i-1}[s-w:s]         (chain, i = 1 .. nb-1)
//      y_i[0:s-w] -= Pn_i[0:s-w] y_{i-1}[s-w:s], z = y / D
//   C  v_i = Linv_i^T z_i                               (all rows)
//   D  v_i[0:w]   -= Rn_i[0:w] v_{i+1}[0:w]             (chain, i = nb-2 .. 0)
//      v_i[w:s]   -= Rn_i[w:s] v_{i+1}[0:w], x = v
// Only the w chain rows of each step depend on the previous step. They run
// on the first ceil(w/7) CTAs, warps 0-6 one row each, with a barrier of
// their own (bar[1]) led by warp 7, which has no loads in flight for its
// fence to wait on; a warp's next row and all its steps' own values are in
// registers before the step starts. The remaining rows of every block
// follow in one grid-wide pass.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) solve_kernel(SolveArgs<T> a)
{
    unsigned ep = 0, ep_chain = 0;  // grid and chain barriers passed
    constexpr int kChainWarps = 7;
    constexpr unsigned kLeader = 32 * kChainWarps;  // lane 0 of warp 7
    const long s = a.s, w = a.w, nb = a.nblk, npad = nb * s;
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    const long gwarp = blockIdx.x * 8L + warp;
    const long nwarps = gridDim.x * 8L;
    const long gthr = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const long nthr = gridDim.x * (long)blockDim.x;
    const unsigned nchain = (unsigned)min((w + kChainWarps - 1) / kChainWarps, (long)gridDim.x);
    const bool in_chain = blockIdx.x < nchain;
    const long cw = (long)kChainWarps * nchain;              // chain warps
    const long crow = warp < kChainWarps ? blockIdx.x * (long)kChainWarps + warp : w;  // chain row, w: none
    const bool regs = cw >= w;                               // one chain row per warp
    const bool own_regs = regs && nb - 1 <= 32;              // a lane per step for the warp's own values
    GridBarrier *cbar = a.bar + 1;
    auto chain_failed = [&]() {
        if (threadIdx.x == kLeader) atomicExch(&a.bar->err, 1);  // releases the CTAs waiting on bar[0]
    };
    T pre[row_regs<T>()];
    T own = 0;

    // A: y = blockdiag(Linv) b (b converted to T into z first)
    for (long g = gthr; g < npad; g += nthr) a.z[g] = g < a.n ? (T)a.rhs[g] : T(0);
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    for (long row = gwarp; row < npad; row += nwarps) {
        const long i = row / s, r = row % s;
        T acc = warp_row_dot(a.linv + i * s * s + r * s, a.z + i * s, r + 1, lane);
        if (lane == 0) a.y[row] = acc;
    }
    if (in_chain && regs && crow < w && nb > 1) row_to_regs(pre, a.pn + s * w + (s - w + crow) * w, w, lane);
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    // B, chain rows
    if (in_chain) {
        if (own_regs && crow < w && lane + 1 < nb) own = a.y[(lane + 1) * s + s - w + crow];
        for (long i = 1; i < nb; ++i) {
            const T *yp = a.y + i * s - w;
            if (regs) {
                const T oi = own_regs ? __shfl_sync(0xffffffffu, own, (int)(i - 1)) : T(0);
                if (crow < w) {
                    const T *row = a.pn + i * s * w + (s - w + crow) * w;
                    const T acc = regs_row_dot(pre, row, yp, w, lane);
                    if (lane == 0) {
                        T *dst = a.y + i * s + s - w + crow;
                        *dst = own_regs ? oi - acc : *dst - acc;
                    }
                    if (i + 1 < nb) row_to_regs(pre, row + s * w, w, lane);
                }
            } else if (warp < kChainWarps) {
                for (long r = crow; r < w; r += cw) {
                    const T acc = warp_row_dot(a.pn + i * s * w + (s - w + r) * w, yp, w, lane);
                    if (lane == 0) a.y[i * s + s - w + r] -= acc;
                }
            }
            if (!grid_barrier(cbar, nchain, ep_chain, a.max_polls, kLeader)) {
                chain_failed();
                return;
            }
        }
    }
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    // B, the other rows, and z = y / D
    for (long row = gwarp; row < npad; row += nwarps) {
        const long i = row / s, r = row % s;
        T acc = 0;
        if (i >= 1 && r < s - w) acc = warp_row_dot(a.pn + i * s * w + r * w, a.y + i * s - w, w, lane);
        if (lane == 0) a.z[row] = (a.y[row] - acc) * a.dinv[row];
    }
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    // C: v = blockdiag(Linv^T) z, warp per row of the stored transpose
    for (long row = gwarp; row < npad; row += nwarps) {
        const long i = row / s, c = row % s;
        T acc = warp_row_dot(a.linvt + i * s * s + c * s + c, a.z + i * s + c, s - c, lane);
        if (lane == 0) a.v[row] = acc;
    }
    if (in_chain && regs && crow < w && nb > 1) row_to_regs(pre, a.rn + (nb - 2) * s * w + crow * w, w, lane);
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    // D, chain rows
    if (in_chain) {
        if (own_regs && crow < w && lane + 1 < nb) own = a.v[lane * s + crow];
        for (long i = nb - 2; i >= 0; --i) {
            const T *xn = a.v + (i + 1) * s;
            if (regs) {
                const T oi = own_regs ? __shfl_sync(0xffffffffu, own, (int)i) : T(0);
                if (crow < w) {
                    const T *row = a.rn + i * s * w + crow * w;
                    const T acc = regs_row_dot(pre, row, xn, w, lane);
                    if (lane == 0) {
                        T *dst = a.v + i * s + crow;
                        *dst = own_regs ? oi - acc : *dst - acc;
                    }
                    if (i > 0) row_to_regs(pre, row - s * w, w, lane);
                }
            } else if (warp < kChainWarps) {
                for (long c = crow; c < w; c += cw) {
                    const T acc = warp_row_dot(a.rn + i * s * w + c * w, xn, w, lane);
                    if (lane == 0) a.v[i * s + c] -= acc;
                }
            }
            if (!grid_barrier(cbar, nchain, ep_chain, a.max_polls, kLeader)) {
                chain_failed();
                return;
            }
        }
    }
    if (!grid_barrier(a.bar, gridDim.x, ep, a.max_polls)) return;
    // D, the other rows, and x = v
    for (long row = gwarp; row < a.n; row += nwarps) {
        const long i = row / s, c = row % s;
        T acc = 0;
        if (i <= nb - 2 && c >= w) acc = warp_row_dot(a.rn + i * s * w + c * w, a.v + (i + 1) * s, w, lane);
        if (lane == 0) a.out[row] = (double)(a.v[row] - acc);
    }
}

// -------------------------------------------------------------------------
// Host sequences
// -------------------------------------------------------------------------

// The whole band LDL^T in one cooperative launch (plus the identity padding
// and the flag reset).
template <typename T>
void factor_band(BandFactor &f, cudaStream_t st, long *launches)
{
    constexpr int TS = sizeof(T) == 8 ? 16 : 32;
    T *band = (T *)f.band;
    const long npad = f.nblk * f.s;
    if (npad > f.n) {
        pad_identity_kernel<T><<<(unsigned)((npad - f.n + 127) / 128), 128, 0, st>>>(band, f.ld, f.n, npad);
        ++*launches;
    }
    CB_CUDA(cudaMemsetAsync(f.flags, 0, 2 * sizeof(int), st));
    CB_CUDA(cudaMemsetAsync(f.fbar, 0, sizeof(GridBarrier), st));
    const long nt = (f.bw + TS - 1) / TS;
    const long ntiles = nt * (nt + 1) / 2;
    const long need = std::max(ntiles, (f.bw + 7) / 8);
    const int grid = (int)std::max(1L, std::min((long)f.factor_grid, need));
    // FP32: form each panel's rows once (two barriers per panel) when the
    // trailing triangle has many more tiles than CTAs; otherwise per tile
    const int dist = (f.fp32 && ntiles > 2L * grid) ? 1 : 0;
    FactorArgs<T> a{band, f.ld, f.bw, npad, f.n, (T *)f.dinv, f.ssd, f.flags, (T *)f.work, (T *)f.stage,
                    (T *)f.look, f.fbar, dist, f.max_polls};
    if constexpr (sizeof(T) == 4) {
        if (f.cluster > 0) {
            ClusterArgs ca{a, f.cluster_slots, f.cluster_nwin};
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)f.cluster);
            cfg.blockDim = dim3(kClusterThreads);
            cfg.dynamicSmemBytes = f.cluster_smem;
            cfg.stream = st;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = (unsigned)f.cluster;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            CB_CUDA(cudaLaunchKernelEx(&cfg, factor_cluster_kernel, ca));
            ++*launches;
            return;
        }
    }
    void *args[] = {&a};
    const void *fn = f.fp32 ? (const void *)factor_f32_kernel<32> : (const void *)factor_f64_kernel<16>;
    CB_CUDA(cudaLaunchCooperativeKernel(fn, dim3((unsigned)grid), dim3(256), args, 0, st));
    ++*launches;
}

// The most dynamic shared memory inv_col_kernel<T> may take on this device
// (the attribute is set once, to the opt-in limit, for every handle).
template <typename T>
size_t inv_col_smem_max()
{
    static const size_t cap = [] {
        int dev = 0, optin = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaFuncSetAttribute(inv_col_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) !=
                cudaSuccess) {
            cudaGetLastError();
            return (size_t)0;
        }
        return (size_t)optin;
    }();
    return cap;
}

// Solve blocks from the factored band: Linv_i, its transpose, Pn_i, Rn_i.
template <typename T>
void form_solve_blocks(BandFactor &f, cudaStream_t st, long *launches)
{
    T *band = (T *)f.band;
    const long nt = f.s / NB;
    const long kb = (f.bw + NB - 1) / NB + 1;
    inv_diag_kernel<T><<<dim3((unsigned)nt, (unsigned)f.nblk), 32, 0, st>>>(band, f.ld, f.bw, f.s, (T *)f.linv);
    const size_t smem = inv_col_smem<T>(kb);
    if (smem <= inv_col_smem_max<T>()) {
        // CTAs ordered by column: the longest sweeps (J = 0) start first
        inv_col_kernel<T><<<dim3((unsigned)f.nblk, (unsigned)nt), 256, smem, st>>>(band, f.ld, f.bw, f.s, kb,
                                                                                  (T *)f.linv, (T *)f.linvt);
        *launches += 2;
    } else {
        // bands too wide for the column ring: one launch per tile row, then the transpose
        for (long I = 1; I < nt; ++I)
            inv_row_kernel<T><<<dim3((unsigned)I, (unsigned)f.nblk), 256, 0, st>>>(band, f.ld, f.bw, f.s, I, kb,
                                                                                   (T *)f.linv);
        transpose_kernel<T><<<dim3((unsigned)nt, (unsigned)nt, (unsigned)f.nblk), 256, 0, st>>>((const T *)f.linv,
                                                                                            f.s, (T *)f.linvt);
        *launches += nt + 1;
    }
    if (f.nblk > 1) {
        dim3 g((unsigned)(f.w / NB), (unsigned)(f.s / NB), (unsigned)(f.nblk - 1));
        pn_kernel<T><<<g, 256, 0, st>>>(band, f.ld, f.bw, f.s, f.w, (const T *)f.linv, (T *)f.pmat);
        rn_kernel<T><<<g, 256, 0, st>>>(band, f.ld, f.bw, f.s, f.w, (const T *)f.linv, (T *)f.rmat);
        *launches += 2;
    }
    CB_CUDA(cudaGetLastError());
}

template <typename T>
void solve_direct_launch(const BandFactor &f, const double *rhs, double *x, void *work, GridBarrier *bar,
                         cudaStream_t st)
{
    DirectArgs<T> a{(const T *)f.band, (const T *)f.dinv, f.ld, f.bw, f.nblk * f.s, f.n, rhs, x, (T *)work, bar,
                    f.max_polls};
    CB_CUDA(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), st));
    void *args[] = {&a};
    CB_CUDA(cudaLaunchCooperativeKernel((const void *)solve_direct_kernel<T>, dim3((unsigned)f.solve_grid),
                                        dim3(256), args, 0, st));
}

template <typename T>
void solve_launch(const BandFactor &f, const double *rhs, double *x, void *work, GridBarrier *bar,
                  cudaStream_t st)
{
    if (f.direct) {
        solve_direct_launch<T>(f, rhs, x, work, bar, st);
        return;
    }
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
    a.max_polls = f.max_polls;
    CB_CUDA(cudaMemsetAsync(bar, 0, 2 * sizeof(GridBarrier), st));  // grid and chain barriers
    void *args[] = {&a};
    CB_CUDA(cudaLaunchCooperativeKernel((const void *)solve_kernel<T>, dim3((unsigned)f.solve_grid), dim3(256),
                                        args, 0, st));
}

template <typename K>
int max_cooperative_grid(K kernel)
{
    int dev = 0, sms = 0, per = 0;
    CB_CUDA(cudaGetDevice(&dev));
    CB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, 0));
    return std::max(1, sms * std::min(per, 4));
}

// The cluster factor for FP32 bands whose active window fits the
// distributed shared memory of a cluster (16 CTAs, or 8 with more slots
// each): (nslot - 1) C >= nwin blocks of the window.
void choose_cluster(BandFactor &f)
{
    f.cluster = 0;
    if (!f.fp32 || !f.use_cluster) return;
    const int nwin = (int)((f.bw + NB - 1) / NB);
    int dev = 0, optin = 0;
    CB_CUDA(cudaGetDevice(&dev));
    CB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa{};
    CB_CUDA(cudaFuncGetAttributes(&fa, factor_cluster_kernel));
    for (int C : {16, 8}) {
        const int nslot = 1 + (nwin + C - 1) / C;
        const size_t dyn = sizeof(float) * ((size_t)nslot * NB * f.ld + 2 * (size_t)f.bw * kWs + NB);
        if (dyn + fa.sharedSizeBytes > (size_t)optin) continue;
        if (C > 8 && cudaFuncSetAttribute(factor_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                         cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        // one attribute for every handle: the most dynamic shared memory a CTA may have
        if (cudaFuncSetAttribute(factor_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa.sharedSizeBytes) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)C);
        cfg.blockDim = dim3(kClusterThreads);
        cfg.dynamicSmemBytes = dyn;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)C;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, factor_cluster_kernel, &cfg) != cudaSuccess || nclusters < 1) {
            cudaGetLastError();
            continue;
        }
        f.cluster = C;
        f.cluster_slots = nslot;
        f.cluster_nwin = nwin;
        f.cluster_smem = dyn;
        return;
    }
}

template <typename T>
void profile_impl(BandFactor &f, int which, cudaStream_t st)
{
    long dummy = 0;
    if (which == 3) factor_band<T>(f, st, &dummy);             // the persistent LDL^T alone
    else if (which == 4 && !f.direct) form_solve_blocks<T>(f, st, &dummy);  // Linv, Pn, Rn from the factor
}

// ---- FP64 effective stiffness beside an FP32 factor (iterative refinement) ----

// band32 = (float) band64 over the stored part of the band
__global__ void band_to_f32_kernel(const double *__restrict__ b64, float *__restrict__ b32, long total)
{
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q < total) b32[q] = (float)b64[q];
}

// w_j = K_jj x_j + sum_{i > j} K_ij x_i: one warp per column, coalesced
// along the column's band entries
__global__ void band_upper_dot_kernel(const double *__restrict__ band, long ld, long bw, long n,
                                      const double *__restrict__ x, double *__restrict__ w)
{
    const long j = (blockIdx.x * (long)blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    if (j >= n) return;
    double acc = 0;
    for (long off = lane; off <= bw && j + off < n; off += 32) acc += band[j * ld + off] * x[j + off];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) w[j] = acc;
}

// r_i = b_i - (w_i + sum_{j < i} K_ij x_j): one thread per row
__global__ void band_residual_kernel(const double *__restrict__ band, long ld, long bw, long n,
                                     const double *__restrict__ b, const double *__restrict__ x,
                                     const double *__restrict__ w, double *__restrict__ r)
{
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = w[i];
    const long lo = i - bw > 0 ? i - bw : 0;
    for (long j = lo; j < i; ++j) acc += band[j * ld + (i - j)] * x[j];
    r[i] = b[i] - acc;
}

}  // namespace

void band_share_gpu(BandFactor &f, bool shared)
{
    if (f.direct) return;
    f.solve_grid = shared ? (int)std::min<long>(f.solve_grid_full, std::max(32L, f.s / 8)) : f.solve_grid_full;
}

void band_copy_to_f32(const double *band64, BandFactor &f, cudaStream_t st)
{
    const long total = f.ld * f.nblk * f.s;
    band_to_f32_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(band64, (float *)f.band, total);
    CB_CUDA(cudaGetLastError());
}

void band_residual64(const double *band64, long ld, long bw, long n, const double *b, const double *x, double *r,
                     double *w, cudaStream_t st)
{
    band_upper_dot_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, st>>>(band64, ld, bw, n, x, w);
    band_residual_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(band64, ld, bw, n, b, x, w, r);
    CB_CUDA(cudaGetLastError());
}

void band_use_factored(BandFactor &f, cudaStream_t st)
{
    if (f.dw) throw std::runtime_error("a double-word band is factored by band_factor only");
    const long npad = f.nblk * f.s;
    const unsigned g = (unsigned)((npad + 255) / 256);
    long dummy = 0;
    if (f.fp32) {
        if (npad > f.n)
            pad_identity_kernel<float><<<(unsigned)((npad - f.n + 127) / 128), 128, 0, st>>>((float *)f.band, f.ld,
                                                                                            f.n, npad);
        dinv_from_diag_kernel<float><<<g, 256, 0, st>>>((const float *)f.band, f.ld, (float *)f.dinv, npad);
        if (!f.direct) form_solve_blocks<float>(f, st, &dummy);
    } else {
        if (npad > f.n)
            pad_identity_kernel<double><<<(unsigned)((npad - f.n + 127) / 128), 128, 0, st>>>((double *)f.band,
                                                                                             f.ld, f.n, npad);
        dinv_from_diag_kernel<double><<<g, 256, 0, st>>>((const double *)f.band, f.ld, (double *)f.dinv, npad);
        if (!f.direct) form_solve_blocks<double>(f, st, &dummy);
    }
    CB_CUDA(cudaGetLastError());
}

size_t band_work_bytes(const BandFactor &f)
{
    return 256 + 3 * (size_t)f.nblk * f.s * (f.fp32 ? sizeof(float) : sizeof(double));
}

void band_solve_with_work(const BandFactor &f, const double *rhs, double *x, void *work, cudaStream_t st)
{
    // the grid-barrier counters sit in front of the work vectors
    GridBarrier *bar = (GridBarrier *)work;
    void *vecs = (unsigned char *)work + 256;
    if (f.dw) band_dw_solve(f, rhs, x, vecs, bar, st);
    else if (f.fp32) solve_launch<float>(f, rhs, x, vecs, bar, st);
    else solve_launch<double>(f, rhs, x, vecs, bar, st);
    CB_CUDA(cudaGetLastError());
}

void band_profile_launch(BandFactor &f, int which, cudaStream_t st)
{
    long dummy = 0;
    if (f.dw) {
        if (which == 3) band_dw_factor(f, st, &dummy);
    } else if (f.fp32) profile_impl<float>(f, which, st);
    else profile_impl<double>(f, which, st);
    CB_CUDA(cudaGetLastError());
}

void band_alloc(BandFactor &f, long n, long bw, bool fp32, bool direct, bool use_cluster, long direct_block)
{
    f.n = n;
    f.bw = std::max(1L, bw);
    f.fp32 = fp32;
    f.direct = direct;
    f.use_cluster = use_cluster;
    f.ld = ((f.bw + 1 + 7) / 8) * 8;
    f.w = std::max(32L, ((f.bw + 31) / 32) * 32);
    const size_t es = fp32 ? 4 : 8;
    // Block size of the solve: FP32 uses up to 4 w (fewer sequential steps,
    // bounded by the inverse blocks' memory of n*s elements); FP64 keeps
    // s = w because the FP64 inversion work grows with s^2. The direct solve
    // needs no blocks: the matrix is padded to a multiple of 32 only.
    long s = f.w;
    if (direct) {
        s = direct_block > 0 ? direct_block : NB;
    } else if (fp32) {
        const double budget = 4.0e9;
        long cap = (long)(budget / ((double)es * (double)std::max(1L, n)));
        s = std::max(f.w, std::min(4 * f.w, (cap / 32) * 32));
    }
    f.s = s;
    f.nblk = (n + f.s - 1) / f.s;
    const long npad = f.nblk * f.s;
    const size_t blocks = direct ? 0 : (size_t)f.nblk * f.s;
    CB_CUDA(cudaMalloc(&f.band, es * (size_t)f.ld * npad));
    CB_CUDA(cudaMalloc(&f.dinv, es * (size_t)npad));
    if (!direct) {
        CB_CUDA(cudaMalloc(&f.linv, es * blocks * f.s));
        CB_CUDA(cudaMalloc(&f.linvt, es * blocks * f.s));
        CB_CUDA(cudaMalloc(&f.pmat, es * blocks * f.w));
        CB_CUDA(cudaMalloc(&f.rmat, es * blocks * f.w));
        CB_CUDA(cudaMemset(f.linv, 0, es * blocks * f.s));
        CB_CUDA(cudaMemset(f.linvt, 0, es * blocks * f.s));
        CB_CUDA(cudaMemset(f.pmat, 0, es * blocks * f.w));
        CB_CUDA(cudaMemset(f.rmat, 0, es * blocks * f.w));
    }
    size_t work = std::max((size_t)3 * npad, (size_t)2 * NB * f.bw + NB);
    CB_CUDA(cudaMalloc(&f.work, es * work));
    CB_CUDA(cudaMalloc(&f.ssd, sizeof(double) * (size_t)n));
    CB_CUDA(cudaMalloc(&f.flags, 2 * sizeof(int)));
    CB_CUDA(cudaMalloc(&f.bar, 2 * sizeof(GridBarrier)));  // the solve's grid and chain barriers
    CB_CUDA(cudaMalloc(&f.stage, es * 2 * NB * NB));
    CB_CUDA(cudaMalloc(&f.look, es * 2 * (NB * NB + NB)));  // two panels of L, D and 1/D
    CB_CUDA(cudaMemset(f.bar, 0, 2 * sizeof(GridBarrier)));
    CB_CUDA(cudaMalloc(&f.fbar, sizeof(GridBarrier)));
    CB_CUDA(cudaMemset(f.fbar, 0, sizeof(GridBarrier)));
    // The direct solve's grid is sized to the work of one panel step (at most
    // bw rows), which also keeps its grid barriers cheap; the block solve
    // takes every SM unless band_share_gpu narrows it.
    if (direct) {
        f.solve_grid = fp32 ? max_cooperative_grid(solve_direct_kernel<float>)
                            : max_cooperative_grid(solve_direct_kernel<double>);
        f.solve_grid = (int)std::min<long>(f.solve_grid, std::max(16L, f.bw / 64));
    } else {
        f.solve_grid = fp32 ? max_cooperative_grid(solve_kernel<float>) : max_cooperative_grid(solve_kernel<double>);
    }
    f.solve_grid_full = f.solve_grid;
    f.factor_grid = fp32 ? max_cooperative_grid(factor_f32_kernel<32>) : max_cooperative_grid(factor_f64_kernel<16>);
    if (fp32) choose_cluster(f);
    f.bytes = es * ((size_t)f.ld * npad + npad + blocks * (2 * f.s + 2 * f.w) + work);
}

void band_alloc_dw(BandFactor &f, long n, long bw, bool simt)
{
    band_alloc(f, n, bw, false, true, false, band_dw_block());
    f.dw = true;
    f.dw_simt = simt;
    band_dw_alloc(f);
}

void band_free(BandFactor &f)
{
    if (f.factor_graph) cudaGraphExecDestroy(f.factor_graph);
    for (void *p : {f.band, f.dinv, f.linv, f.linvt, f.pmat, f.rmat, f.work, f.stage, f.look, (void *)f.ssd,
                    (void *)f.flags, (void *)f.bar, (void *)f.fbar, f.slices, (void *)f.slice_exp})
        if (p) cudaFree(p);
    f = BandFactor{};
}

void band_factor(BandFactor &f, cudaStream_t st, bool use_graph, long *launches)
{
    long dummy = 0;
    long *cnt = launches ? launches : &dummy;
    if (f.dw) {
        band_dw_factor(f, st, cnt);
        return;
    }
    if (f.fp32) factor_band<float>(f, st, cnt);
    else factor_band<double>(f, st, cnt);
    if (f.direct) return;
    if (!use_graph) {
        if (f.fp32) form_solve_blocks<float>(f, st, cnt);
        else form_solve_blocks<double>(f, st, cnt);
        return;
    }
    if (!f.factor_graph) {
        long per = 0;
        cudaGraph_t g;
        CB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        if (f.fp32) form_solve_blocks<float>(f, st, &per);
        else form_solve_blocks<double>(f, st, &per);
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
    if (f.dw) band_dw_solve(f, rhs, x, f.work, f.bar, st);
    else if (f.fp32) solve_launch<float>(f, rhs, x, f.work, f.bar, st);
    else solve_launch<double>(f, rhs, x, f.work, f.bar, st);
    CB_CUDA(cudaGetLastError());
    if (launches) *launches += 1;
}

}  // namespace cb
