// Restarted flexible GMRES (FGMRES(m)) with a nodal block-Jacobi
// preconditioner over a CSR product, for the effective stiffness of the
// nonlinear Newmark iteration (solve.c:139-222 and 469-533 hand that system
// to skyfact/skysolve; here it is solved iteratively to a relative residual).
//
// Right preconditioning, Z kept (flexible): x = x0 + Z y. Orthogonalisation
// is classical Gram-Schmidt applied twice (CGS2): three passes over the
// basis per step, the second pass fused with the first update and the norm
// with the second. The Hessenberg column, its Givens rotations, the small
// triangular solve and the restart decision run in one-block kernels on a
// control block in device memory, so an Arnoldi step is a fixed sequence of
// launches that a CUDA graph replays; kernels read `done` first and return
// once the solve has ended. Every reduction has a fixed order (partials per
// block of rows, then one block), so a solve is bit-reproducible.
//
// Traffic per Arnoldi step at column j (n equations, nnz stored entries):
// SpMV 12 nnz + 24 n bytes, block-Jacobi about 8 bs n + 24 n, and the
// three Gram-Schmidt passes 8 n (4 j + 7) bytes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#include "internal.hpp"
#include "model.hpp"

namespace cb {

namespace {

constexpr int kKT = 256;

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- assembly ----

__global__ void kry_gather_kernel(const int *__restrict__ ptr, const int *__restrict__ src,
                                  const int64_t *__restrict__ dst, const int64_t *__restrict__ dst2,
                                  const double *__restrict__ in, double *__restrict__ val, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += in[src[k]];
    val[dst[i]] = s;
    if (dst2[i] >= 0) val[dst2[i]] = s;
}

__global__ void kry_shift_kernel(double *__restrict__ val, const int *__restrict__ diag,
                                 const double *__restrict__ sm, double c0, double den, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double add = c0 * sm[i] / den;
    val[diag[i]] = val[diag[i]] + add;
}

// ---- block-Jacobi ----

// One thread per block: gather the bs x bs diagonal block from the CSR rows
// and invert it by Gauss-Jordan elimination with partial pivoting. A
// singular block falls back to the inverse diagonal (1 where it is zero)
// and raises flag[0].
template <typename T>
__global__ void kry_bj_setup_kernel(const int *__restrict__ rowptr, const int *__restrict__ col,
                                    const double *__restrict__ val, const int *__restrict__ blk_start,
                                    const int *__restrict__ blk_off, T *__restrict__ binv, long nblk,
                                    int *__restrict__ flag)
{
    long b = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const int s0 = blk_start[b], bs = blk_start[b + 1] - s0;
    double A[8][8], X[8][8];
    for (int r = 0; r < bs; ++r)
        for (int c = 0; c < bs; ++c) {
            A[r][c] = 0;
            X[r][c] = r == c ? 1.0 : 0.0;
        }
    for (int r = 0; r < bs; ++r)
        for (int k = rowptr[s0 + r]; k < rowptr[s0 + r + 1]; ++k) {
            const int c = col[k] - s0;
            if (c >= 0 && c < bs) A[r][c] = val[k];
        }
    double dg[8];
    for (int r = 0; r < bs; ++r) dg[r] = A[r][r];
    bool ok = true;
    for (int c = 0; c < bs && ok; ++c) {
        int p = c;
        for (int r = c + 1; r < bs; ++r)
            if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
        if (!(fabs(A[p][c]) > 0)) {
            ok = false;
            break;
        }
        if (p != c)
            for (int k = 0; k < bs; ++k) {
                double t = A[p][k];
                A[p][k] = A[c][k];
                A[c][k] = t;
                t = X[p][k];
                X[p][k] = X[c][k];
                X[c][k] = t;
            }
        const double inv = 1.0 / A[c][c];
        for (int k = 0; k < bs; ++k) {
            A[c][k] *= inv;
            X[c][k] *= inv;
        }
        for (int r = 0; r < bs; ++r) {
            if (r == c) continue;
            const double f = A[r][c];
            if (f == 0) continue;
            for (int k = 0; k < bs; ++k) {
                A[r][k] -= f * A[c][k];
                X[r][k] -= f * X[c][k];
            }
        }
    }
    T *out = binv + blk_off[b];
    if (ok) {
        for (int r = 0; r < bs; ++r)
            for (int c = 0; c < bs; ++c) out[r * bs + c] = (T)X[r][c];
    } else {
        atomicExch(flag, 1);
        for (int r = 0; r < bs; ++r)
            for (int c = 0; c < bs; ++c) out[r * bs + c] = (T)(r == c ? (dg[r] != 0 ? 1.0 / dg[r] : 1.0) : 0.0);
    }
}

// v_j = w * scale; z_j = B^-1 v_j over the row's block (in Tb arithmetic)
template <typename Tb, typename T>
__global__ void kry_bj_apply_kernel(const KrylovCtl *__restrict__ ctl, const T *__restrict__ w, T *__restrict__ V,
                                    T *__restrict__ Z, const int *__restrict__ row_blk,
                                    const int *__restrict__ blk_start, const int *__restrict__ blk_off,
                                    const Tb *__restrict__ binv, long n)
{
    if (ctl->done) return;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = ctl->j;
    const T sc = (T)ctl->scale;
    V[(size_t)j * n + i] = w[i] * sc;
    const int b = row_blk[i];
    const int s0 = blk_start[b], bs = blk_start[b + 1] - s0;
    const Tb *B = binv + blk_off[b] + (i - s0) * bs;
    Tb z = 0;
    for (int c = 0; c < bs; ++c) z += B[c] * (Tb)(w[s0 + c] * sc);
    Z[(size_t)j * n + i] = (T)z;
}

// ---- products and Gram-Schmidt passes ----

// 8 lanes per row, fixed lane order. mode 0: y = A z_j (while the solve
// runs); mode 1: y = b - A x (when a cycle ends unconverged); mode 2: y = A x.
template <typename T>
__global__ void kry_spmv_kernel(const KrylovCtl *__restrict__ ctl, int mode, const int *__restrict__ rowptr,
                                const int *__restrict__ col, const T *__restrict__ val, const T *__restrict__ xin,
                                const T *__restrict__ bvec, T *__restrict__ y, long n)
{
    if (mode == 0 && ctl->done) return;
    if (mode == 1 && (ctl->done || !ctl->finish || ctl->conv)) return;
    const T *x = mode == 0 ? xin + (size_t)ctl->j * n : xin;
    const long row = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 3;
    const int lane = threadIdx.x & 7;
    T acc = 0;
    if (row < n)
        for (int k = rowptr[row] + lane; k < rowptr[row + 1]; k += 8) acc += val[k] * x[col[k]];
    acc += __shfl_xor_sync(0xffffffffu, acc, 4);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    if (row < n && lane == 0) y[row] = mode == 1 ? bvec[row] - acc : acc;
}

// ---- Gram-Schmidt passes. FP64 arithmetic is the scarce resource here, so
// the dots run one warp per basis vector with the lanes accumulating many
// rows each (few FP64 adds spent on reductions); the per-block sums are
// reduced across blocks by the last block to arrive (fixed order, so the
// sums do not depend on which block that is).

// Threads of the Gram-Schmidt blocks: 512 for FP64 (one block per SM; more
// warps in flight for the same FP64 reductions), 256 for FP32 (four blocks
// per SM).
constexpr int kGTMax = 512;
constexpr int kWarpsMax = kGTMax / 32;
template <typename T>
constexpr int gs_threads() { return sizeof(T) == 8 ? 512 : 256; }

// true in every thread of the last block of the grid to get here
__device__ bool last_block(unsigned *counter)
{
    __shared__ bool s_last;
    __threadfence();  // every thread's partial writes before the block's arrival
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last) __threadfence();
    return s_last;
}

// partial[k*nred + blk] = v_k . w over rows [r0, r1), k <= j (one warp per k)
template <typename T>
__device__ void block_dots(const T *__restrict__ V, const T *__restrict__ w, long n, int j, long r0, long r1,
                           T *__restrict__ partial, int nred)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    for (int k = warp; k <= j; k += nw) {
        const T *v = V + (size_t)k * n;
        T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        long i = r0 + lane;
        for (; i + 96 < r1; i += 128) {
            a0 += v[i] * w[i];
            a1 += v[i + 32] * w[i + 32];
            a2 += v[i + 64] * w[i + 64];
            a3 += v[i + 96] * w[i + 96];
        }
        for (; i < r1; i += 32) a0 += v[i] * w[i];
        const T acc = warp_sum((a0 + a1) + (a2 + a3));
        if (lane == 0) partial[(size_t)k * nred + blockIdx.x] = acc;
    }
}

// partial[blk] = |w|^2 over rows [r0, r1)
template <typename T>
__device__ void block_norm(const T *__restrict__ w, long r0, long r1, T *__restrict__ partial)
{
    __shared__ T red[kWarpsMax];
    T acc = 0;
    for (long i = r0 + threadIdx.x; i < r1; i += blockDim.x) acc += w[i] * w[i];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        T sum = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) sum += red[k];
        partial[blockIdx.x] = sum;
    }
}

// Sum of partial[0..nred) by one warp in a fixed order: each lane loads its
// strided values sixteen at a time (independent loads in flight), adds them
// in index order, then a butterfly across the lanes.
template <typename T>
__device__ __forceinline__ double warp_sum_partials(const T *__restrict__ pk, int nred)
{
    const int lane = threadIdx.x & 31;
    T acc = 0;
    for (int b0 = 0; b0 < nred; b0 += 32 * 16) {
        T v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int b = b0 + lane + 32 * u;
            v[u] = b < nred ? __ldcg(pk + b) : (T)0;
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) acc += v[u];
    }
    return (double)warp_sum(acc);
}

// last block: hp[k] = sum_b partial[k*nred + b] (one warp per k)
template <typename T>
__device__ void reduce_hp(KrylovCtl *ctl, const T *partial, int nred, int j, int pass)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int k = warp; k <= j; k += nw) {
        const double acc = warp_sum_partials(partial + (size_t)k * nred, nred);
        if (lane == 0) {
            ctl->hp[k] = acc;
            ctl->hcol[k] = pass == 0 ? acc : ctl->hcol[k] + acc;
        }
    }
}

// last block, warp 0: sum_b partial[b]
template <typename T>
__device__ double reduce_norm(const T *partial, int nred)
{
    return warp_sum_partials(partial, nred);
}

// w[i] -= sum_k hp[k] V_k[i] over rows [r0, r1)
template <typename T>
__device__ void block_update(const T *__restrict__ V, T *__restrict__ w, long n, int j, const T *hp, long r0,
                             long r1)
{
    for (long i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        T s = w[i];
#pragma unroll 8
        for (int k = 0; k <= j; ++k) s -= hp[k] * V[(size_t)k * n + i];
        w[i] = s;
    }
}

// Closes Arnoldi step j: h_{j+1,j} = |w|, rotations, residual estimate
// |g_{j+1}|; at the end of a cycle y = R^-1 g. One thread.
__device__ void close_step(KrylovCtl *ctl, double ww)
{
    const int j = ctl->j, m = ctl->m, ld = m + 1;
    const double hn = sqrt(ww);
    double *Hc = ctl->H + (size_t)j * ld;
    for (int i = 0; i <= j; ++i) Hc[i] = ctl->hcol[i];
    Hc[j + 1] = hn;
    for (int i = 0; i < j; ++i) {
        const double t = ctl->cs[i] * Hc[i] + ctl->sn[i] * Hc[i + 1];
        Hc[i + 1] = -ctl->sn[i] * Hc[i] + ctl->cs[i] * Hc[i + 1];
        Hc[i] = t;
    }
    const double a = Hc[j], b = Hc[j + 1];
    const double rr = hypot(a, b);
    const double c = rr > 0 ? a / rr : 1.0, s = rr > 0 ? b / rr : 0.0;
    ctl->cs[j] = c;
    ctl->sn[j] = s;
    Hc[j] = rr;
    Hc[j + 1] = 0;
    const double gj = ctl->g[j];
    ctl->g[j + 1] = -s * gj;
    ctl->g[j] = c * gj;
    ctl->iters += 1;
    const double res = fabs(ctl->g[j + 1]);
    ctl->resid = res;
    if (!isfinite(res) || !isfinite(hn) || !(rr > 0)) {
        // no usable column: end the solve with what the earlier cycles gave
        ctl->status = 2;
        ctl->done = 1;
        return;
    }
    const bool conv = res <= ctl->tol_abs || hn == 0;
    if (conv || j + 1 == m || ctl->iters >= ctl->maxit) {
        ctl->finish = 1;
        ctl->conv = conv ? 1 : 0;
        ctl->ncols = j + 1;
        for (int i = j; i >= 0; --i) {
            double t = ctl->g[i];
            for (int k = i + 1; k <= j; ++k) t -= ctl->H[(size_t)k * ld + i] * ctl->y[k];
            ctl->y[i] = t / ctl->H[(size_t)i * ld + i];
        }
    } else {
        ctl->scale = 1.0 / hn;
        ctl->j = j + 1;
    }
}

template <typename T>
struct GsArgs {
    KrylovCtl *ctl;
    const T *V;
    T *w;
    T *partial;
    long n;
    int rpr, nred;
};

// pass 1: h = V^T w (w = A z_j from the product)
template <typename T>
__global__ void kry_gs_dots_kernel(GsArgs<T> a)
{
    KrylovCtl *ctl = a.ctl;
    if (ctl->done) return;
    const int j = ctl->j;
    const long r0 = blockIdx.x * (long)a.rpr, r1 = min(a.n, r0 + a.rpr);
    block_dots(a.V, a.w, a.n, j, r0, r1, a.partial, a.nred);
    if (last_block(&ctl->arrive[0])) {
        reduce_hp(ctl, a.partial, a.nred, j, 0);
        if (threadIdx.x == 0) ctl->arrive[0] = 0;
    }
}

// w -= V h, then pass 2 (last == 0: h2 = V^T w) or the norm and the close of
// the step (last == 1)
template <typename T>
__global__ void kry_gs_update_kernel(GsArgs<T> a, int last)
{
    KrylovCtl *ctl = a.ctl;
    if (ctl->done) return;
    __shared__ T hp[kMaxRestart + 1];
    const int j = ctl->j;
    for (int k = threadIdx.x; k <= j; k += blockDim.x) hp[k] = (T)ctl->hp[k];
    __syncthreads();
    const long r0 = blockIdx.x * (long)a.rpr, r1 = min(a.n, r0 + a.rpr);
    block_update(a.V, a.w, a.n, j, hp, r0, r1);
    __syncthreads();
    if (!last) {
        block_dots(a.V, (const T *)a.w, a.n, j, r0, r1, a.partial, a.nred);
        if (last_block(&ctl->arrive[1])) {
            reduce_hp(ctl, a.partial, a.nred, j, 1);
            if (threadIdx.x == 0) ctl->arrive[1] = 0;
        }
        return;
    }
    block_norm((const T *)a.w, r0, r1, a.partial);
    if (last_block(&ctl->arrive[2])) {
        if (threadIdx.x < 32) {
            const double ww = reduce_norm(a.partial, a.nred);
            if (threadIdx.x == 0) {
                close_step(ctl, ww);
                ctl->arrive[2] = 0;
            }
        }
    }
}

// Start of a solve (mode 0; w = b): |b| and the first cycle. After a
// finished cycle (mode 1): done when the estimate converged, else restart
// from the true residual r = b - A x held in w.
template <typename T>
__global__ void kry_norm_start_kernel(GsArgs<T> a, int mode, int m, int maxit, double rtol)
{
    KrylovCtl *ctl = a.ctl;
    if (mode == 1) {
        if (ctl->done || !ctl->finish) return;
        if (ctl->conv) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                ctl->status = 0;
                ctl->done = 1;
            }
            return;
        }
    }
    const long r0 = blockIdx.x * (long)a.rpr, r1 = min(a.n, r0 + a.rpr);
    block_norm((const T *)a.w, r0, r1, a.partial);
    if (!last_block(&ctl->arrive[3])) return;
    if (threadIdx.x >= 32) return;
    const double bb = reduce_norm(a.partial, a.nred);
    if (threadIdx.x != 0) return;
    ctl->arrive[3] = 0;
    const double bn = sqrt(bb);
    if (mode == 0) {
        ctl->j = 0;
        ctl->finish = 0;
        ctl->conv = 0;
        ctl->iters = 0;
        ctl->restarts = 0;
        ctl->ncols = 0;
        ctl->m = m;
        ctl->maxit = maxit;
        ctl->rtol = rtol;
        ctl->bnorm = bn;
        ctl->beta = bn;
        ctl->resid = bn;
        ctl->tol_abs = rtol * bn;
        ctl->g[0] = bn;
        ctl->scale = bn > 0 ? 1.0 / bn : 0.0;
        ctl->status = isfinite(bn) ? 0 : 2;
        ctl->done = (bn == 0 || !isfinite(bn)) ? 1 : 0;
        return;
    }
    ctl->resid = bn;
    ctl->beta = bn;
    if (bn <= ctl->tol_abs) {
        ctl->status = 0;
        ctl->done = 1;
        return;
    }
    if (ctl->iters >= ctl->maxit || !isfinite(bn)) {
        ctl->status = isfinite(bn) ? 1 : 2;
        ctl->done = 1;
        return;
    }
    ctl->restarts += 1;
    ctl->j = 0;
    ctl->finish = 0;
    ctl->g[0] = bn;
    ctl->scale = 1.0 / bn;
}

// x += Z y at the end of a cycle
template <typename T>
__global__ void kry_xupdate_kernel(const KrylovCtl *__restrict__ ctl, const T *__restrict__ Z, T *__restrict__ x,
                                   long n)
{
    if (ctl->done || !ctl->finish) return;
    __shared__ T y[kMaxRestart];
    const int nc = ctl->ncols;
    for (int k = threadIdx.x; k < nc; k += blockDim.x) y[k] = (T)ctl->y[k];
    __syncthreads();
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    T s = x[i];
    for (int k = 0; k < nc; ++k) s += y[k] * Z[(size_t)k * n + i];
    x[i] = s;
}

// nested precision: v_j = w * scale (FP64) and its FP32 copy, the inner
// right-hand side
__global__ void kry_outer_pre_kernel(const KrylovCtl *__restrict__ ctl, const double *__restrict__ w,
                                     double *__restrict__ V, float *__restrict__ b32, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = w[i] * ctl->scale;
    V[(size_t)ctl->j * n + i] = v;
    b32[i] = (float)v;
}

// z_j = the inner FP32 solution
__global__ void kry_outer_post_kernel(const KrylovCtl *__restrict__ ctl, const float *__restrict__ x32,
                                      double *__restrict__ Z, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) Z[(size_t)ctl->j * n + i] = (double)x32[i];
}

__global__ void kry_to_f32_kernel(const double *__restrict__ a, float *__restrict__ b, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

inline unsigned nb(long n, int t = kKT) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------------------

void krylov_alloc(KrylovSolver &ks, const HostModel &h, int restart, int maxit, bool fp32, cudaStream_t st)
{
    const long n = h.neq;
    ks.n = n;
    ks.m = std::max(2, std::min(restart > 0 ? restart : 50, kMaxRestart));
    ks.maxit = maxit > 0 ? maxit : 2000;
    const bool fp32_precond = fp32;
    ks.fp32_precond = fp32;
    ks.nested = fp32;
    CsrPattern p;
    GatherMap g;
    std::vector<int64_t> dst2;
    build_csr_tangent(h, p, g, dst2);
    for (long i = 0; i < n; ++i)
        if (p.diag[i] < 0)
            throw cb_status_error(CB_ERR_NUMERIC, "equation " + std::to_string(i + 1) + " has no stiffness entry");
    ks.nnz = (long)p.col.size();
    std::vector<int> bstart;
    build_node_blocks(h, bstart);
    ks.nblk = (long)bstart.size() - 1;
    std::vector<int> off(ks.nblk + 1, 0), rblk(n);
    for (long b = 0; b < ks.nblk; ++b) {
        const int bs = bstart[b + 1] - bstart[b];
        off[b + 1] = off[b] + bs * bs;
        for (int q = bstart[b]; q < bstart[b + 1]; ++q) rblk[q] = (int)b;
    }
    ks.binv_n = off[ks.nblk];
    // Gram-Schmidt partition: one block per SM (at least 256 rows a block).
    // The FP64 pipe bounds these passes on GB300; every extra block adds
    // FP64 reduction work per basis vector.
    {
        int dev = 0, sms = 148;
        CB_CUDA(cudaGetDevice(&dev));
        CB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const long want = std::max<long>(1, std::min<long>(sms, (n + 255) / 256));
        ks.rows_per_red = (int)((n + want - 1) / want);
        ks.nred = (int)((n + ks.rows_per_red - 1) / ks.rows_per_red);
    }
    auto alloc = [&](size_t bytes) {
        void *q = nullptr;
        CB_CUDA(cudaMalloc(&q, std::max<size_t>(bytes, 16)));
        CB_CUDA(cudaMemsetAsync(q, 0, std::max<size_t>(bytes, 16), st));
        ks.bytes += std::max<size_t>(bytes, 16);
        return q;
    };
    ks.rowptr = (int *)alloc(sizeof(int) * (n + 1));
    ks.col = (int *)alloc(sizeof(int) * ks.nnz);
    ks.diag = (int *)alloc(sizeof(int) * n);
    ks.val = (double *)alloc(sizeof(double) * ks.nnz);
    ks.amap_n = (long)g.dst.size();
    ks.amap_ptr = (int *)alloc(sizeof(int) * g.ptr.size());
    ks.amap_src = (int *)alloc(sizeof(int) * g.src.size());
    ks.amap_dst = (int64_t *)alloc(sizeof(int64_t) * g.dst.size());
    ks.amap_dst2 = (int64_t *)alloc(sizeof(int64_t) * dst2.size());
    ks.blk_start = (int *)alloc(sizeof(int) * bstart.size());
    ks.blk_off = (int *)alloc(sizeof(int) * off.size());
    ks.row_blk = (int *)alloc(sizeof(int) * n);
    ks.binv = alloc((fp32_precond ? 4 : 8) * (size_t)ks.binv_n);
    ks.V = (double *)alloc(sizeof(double) * (size_t)(ks.m + 1) * n);
    ks.Z = (double *)alloc(sizeof(double) * (size_t)ks.m * n);
    ks.w = (double *)alloc(sizeof(double) * n);
    ks.b = (double *)alloc(sizeof(double) * n);
    ks.x = (double *)alloc(sizeof(double) * n);
    ks.partial = (double *)alloc(sizeof(double) * (size_t)(kMaxRestart + 1) * ks.nred + 16);
    ks.ctl = (KrylovCtl *)alloc(sizeof(KrylovCtl));
    CB_CUDA(cudaMallocHost(&ks.ctl_h, sizeof(KrylovCtl)));
    std::memset(ks.ctl_h, 0, sizeof(KrylovCtl));
    if (ks.nested) {
        ks.valf = (float *)alloc(sizeof(float) * ks.nnz);
        ks.V32 = (float *)alloc(sizeof(float) * (size_t)(ks.m32 + 1) * n);
        ks.Z32 = (float *)alloc(sizeof(float) * (size_t)ks.m32 * n);
        for (float **v : {&ks.w32, &ks.b32, &ks.x32}) *v = (float *)alloc(sizeof(float) * n);
        // FP32 passes: four blocks per SM, FP32 partial sums (the FP32 pipe is
        // not the limit there, the round trips are)
        int dev = 0, sms = 148;
        CB_CUDA(cudaGetDevice(&dev));
        CB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const long want = std::max<long>(1, std::min<long>(4L * sms, (n + 63) / 64));
        ks.rows_per_red32 = (int)((n + want - 1) / want);
        ks.nred32 = (int)((n + ks.rows_per_red32 - 1) / ks.rows_per_red32);
        ks.partial32 = (float *)alloc(sizeof(float) * (size_t)(kMaxRestart + 1) * ks.nred32 + 16);
        ks.ctl32 = (KrylovCtl *)alloc(sizeof(KrylovCtl));
        CB_CUDA(cudaMallocHost(&ks.ctl32_h, sizeof(KrylovCtl)));
        std::memset(ks.ctl32_h, 0, sizeof(KrylovCtl));
    }
    CB_CUDA(cudaMemcpyAsync(ks.rowptr, p.rowptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.col, p.col.data(), sizeof(int) * ks.nnz, cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.diag, p.diag.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.amap_ptr, g.ptr.data(), sizeof(int) * g.ptr.size(), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.amap_src, g.src.data(), sizeof(int) * g.src.size(), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.amap_dst, g.dst.data(), sizeof(int64_t) * g.dst.size(), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.amap_dst2, dst2.data(), sizeof(int64_t) * dst2.size(), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.blk_start, bstart.data(), sizeof(int) * bstart.size(), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.blk_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.row_blk, rblk.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaStreamSynchronize(st));
}

void krylov_free(KrylovSolver &ks)
{
    for (cudaGraphExec_t &g : ks.step_graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    if (ks.graph32) cudaGraphExecDestroy(ks.graph32);
    void *ptrs[] = {ks.rowptr, ks.col,      ks.diag,    ks.val,     ks.amap_ptr, ks.amap_src, ks.amap_dst,
                    ks.amap_dst2, ks.blk_start, ks.blk_off, ks.row_blk, ks.binv, ks.V,        ks.Z,
                    ks.w,      ks.b,        ks.x,       ks.partial, ks.ctl,      ks.valf,     ks.V32,
                    ks.Z32,    ks.w32,      ks.b32,     ks.x32,     ks.partial32, ks.ctl32};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (ks.ctl_h) cudaFreeHost(ks.ctl_h);
    if (ks.ctl32_h) cudaFreeHost(ks.ctl32_h);
    ks = KrylovSolver();
}

void krylov_assemble(KrylovSolver &ks, const double *kel, cudaStream_t st)
{
    if (ks.amap_n > 0)
        kry_gather_kernel<<<nb(ks.amap_n), kKT, 0, st>>>(ks.amap_ptr, ks.amap_src, ks.amap_dst, ks.amap_dst2, kel,
                                                          ks.val, ks.amap_n);
}

void krylov_shift_diag(KrylovSolver &ks, const double *sm, double c0, double den, cudaStream_t st)
{
    kry_shift_kernel<<<nb(ks.n), kKT, 0, st>>>(ks.val, ks.diag, sm, c0, den, ks.n);
}

void krylov_setup_block_jacobi(KrylovSolver &ks, cudaStream_t st)
{
    int *flag = (int *)(ks.partial + (size_t)(kMaxRestart + 1) * ks.nred);
    if (ks.fp32_precond)
        kry_bj_setup_kernel<float><<<nb(ks.nblk, 128), 128, 0, st>>>(ks.rowptr, ks.col, ks.val, ks.blk_start,
                                                                      ks.blk_off, (float *)ks.binv, ks.nblk, flag);
    else
        kry_bj_setup_kernel<double><<<nb(ks.nblk, 128), 128, 0, st>>>(ks.rowptr, ks.col, ks.val, ks.blk_start,
                                                                       ks.blk_off, (double *)ks.binv, ks.nblk, flag);
    if (ks.nested) kry_to_f32_kernel<<<nb(ks.nnz), kKT, 0, st>>>(ks.val, ks.valf, ks.nnz);
}

namespace {

// piv[s0 + r] = r-th pivot of the LDL^T (no pivoting) of joint block b's
// diagonal block of the matrix: the arc-length driver's substitute for the
// global factor's pivots (ssd) when it solves with FGMRES
__global__ void kry_block_pivots_kernel(const int *__restrict__ rowptr, const int *__restrict__ col,
                                        const double *__restrict__ val, const int *__restrict__ blk_start,
                                        double *__restrict__ piv, long nblk)
{
    const long b = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const int s0 = blk_start[b], bs = blk_start[b + 1] - s0;
    double A[8][8];
    for (int r = 0; r < bs; ++r)
        for (int c = 0; c < bs; ++c) A[r][c] = 0;
    for (int r = 0; r < bs; ++r)
        for (int k = rowptr[s0 + r]; k < rowptr[s0 + r + 1]; ++k) {
            const int c = col[k] - s0;
            if (c >= 0 && c < bs) A[r][c] = val[k];
        }
    for (int k = 0; k < bs; ++k) {
        const double d = A[k][k];
        piv[s0 + k] = d;
        if (d == 0.0) continue;
        for (int i = k + 1; i < bs; ++i) {
            const double l = A[i][k] / d;
            for (int j = k + 1; j <= i; ++j) A[i][j] -= l * A[j][k];
        }
    }
}

}  // namespace

void krylov_block_pivots(const KrylovSolver &ks, double *piv, cudaStream_t st)
{
    kry_block_pivots_kernel<<<nb(ks.nblk, 128), 128, 0, st>>>(ks.rowptr, ks.col, ks.val, ks.blk_start, piv, ks.nblk);
    CB_CUDA(cudaGetLastError());
}

void krylov_basis_pair(const KrylovSolver &ks, int k, double *b, double *t, cudaStream_t st)
{
    const double *z = ks.Z + (size_t)k * ks.n;
    CB_CUDA(cudaMemcpyAsync(t, z, sizeof(double) * ks.n, cudaMemcpyDeviceToDevice, st));
    krylov_spmv(ks, z, b, st);
}

void krylov_spmv(const KrylovSolver &ks, const double *x, double *y, cudaStream_t st)
{
    kry_spmv_kernel<double><<<nb(ks.n * 8), kKT, 0, st>>>(ks.ctl, 2, ks.rowptr, ks.col, ks.val, x, nullptr, y,
                                                          ks.n);
}

namespace {

// One precision level of the solver: its matrix values, basis and control.
template <typename T>
struct Core {
    long n;
    int m, maxit;
    double rtol;
    const T *val;
    T *V, *Z, *w, *b, *x;
    T *partial;
    int rpr, nred;  // Gram-Schmidt partition: rows per block, blocks
    KrylovCtl *ctl, *ctl_h;
    cudaGraphExec_t *graph;
};

Core<double> core64(KrylovSolver &ks, int gi)
{
    return Core<double>{ks.n, ks.m,       ks.maxit,     ks.rtol, ks.val,  ks.V,     ks.Z,
                        ks.w, ks.b,       ks.x,         ks.partial, ks.rows_per_red, ks.nred, ks.ctl,
                        ks.ctl_h, &ks.step_graph[gi]};
}

Core<float> core32(KrylovSolver &ks)
{
    return Core<float>{ks.n,   ks.m32,  ks.maxit32, ks.rtol32, ks.valf,          ks.V32,    ks.Z32,
                       ks.w32, ks.b32,  ks.x32,     ks.partial32, ks.rows_per_red32, ks.nred32, ks.ctl32,
                       ks.ctl32_h, &ks.graph32};
}

template <typename T>
GsArgs<T> gs_args(const KrylovSolver &, const Core<T> &c)
{
    return GsArgs<T>{c.ctl, c.V, c.w, c.partial, c.n, c.rpr, c.nred};
}

// The product, Gram-Schmidt, close and cycle-end launches of an Arnoldi
// step (7 launches; the last three act only when a cycle ends).
template <typename T>
void step_after_precond(const KrylovSolver &ks, const Core<T> &c, cudaStream_t st)
{
    const long n = c.n;
    kry_spmv_kernel<T><<<nb(n * 8), kKT, 0, st>>>(c.ctl, 0, ks.rowptr, ks.col, c.val, c.Z, nullptr, c.w, n);
    const GsArgs<T> ga = gs_args(ks, c);
    kry_gs_dots_kernel<T><<<c.nred, gs_threads<T>(), 0, st>>>(ga);
    kry_gs_update_kernel<T><<<c.nred, gs_threads<T>(), 0, st>>>(ga, 0);
    kry_gs_update_kernel<T><<<c.nred, gs_threads<T>(), 0, st>>>(ga, 1);
    kry_xupdate_kernel<T><<<nb(n), kKT, 0, st>>>(c.ctl, c.Z, c.x, n);
    kry_spmv_kernel<T><<<nb(n * 8), kKT, 0, st>>>(c.ctl, 1, ks.rowptr, ks.col, c.val, c.x, c.b, c.w, n);
    kry_norm_start_kernel<T><<<c.nred, gs_threads<T>(), 0, st>>>(ga, 1, 0, 0, 0.0);
}

// One Arnoldi step with the block-Jacobi (or learned, FP64) preconditioner.
template <typename T>
void arnoldi_step(KrylovSolver &ks, const Core<T> &c, KrylovPrecond pc, cudaStream_t st)
{
    const long n = c.n;
    if constexpr (sizeof(T) == 8) {
        if (pc == KrylovPrecond::learned) krylov_apply_learned(ks, st);
        else if (ks.fp32_precond)
            kry_bj_apply_kernel<float, double><<<nb(n), kKT, 0, st>>>(c.ctl, c.w, c.V, c.Z, ks.row_blk, ks.blk_start,
                                                                     ks.blk_off, (const float *)ks.binv, n);
        else
            kry_bj_apply_kernel<double, double><<<nb(n), kKT, 0, st>>>(
                c.ctl, c.w, c.V, c.Z, ks.row_blk, ks.blk_start, ks.blk_off, (const double *)ks.binv, n);
    } else {
        kry_bj_apply_kernel<float, float><<<nb(n), kKT, 0, st>>>(c.ctl, c.w, c.V, c.Z, ks.row_blk, ks.blk_start,
                                                                ks.blk_off, (const float *)ks.binv, n);
    }
    step_after_precond(ks, c, st);
}

constexpr int kStepLaunches = 8;

// x = 0, w = b (already in c.b), |b|: the start of a solve
template <typename T>
void start_solve(const KrylovSolver &ks, const Core<T> &c, cudaStream_t st)
{
    CB_CUDA(cudaMemcpyAsync(c.w, c.b, sizeof(T) * c.n, cudaMemcpyDeviceToDevice, st));
    CB_CUDA(cudaMemsetAsync(c.x, 0, sizeof(T) * c.n, st));
    kry_norm_start_kernel<T><<<c.nred, gs_threads<T>(), 0, st>>>(gs_args(ks, c), 0, c.m, c.maxit, c.rtol);
    CB_CUDA(cudaGetLastError());
}

void read_ctl(const KrylovCtl *dev, KrylovCtl *host, cudaStream_t st)
{
    CB_CUDA(cudaMemcpyAsync(host, dev, offsetof(KrylovCtl, hp), cudaMemcpyDeviceToHost, st));
    CB_CUDA(cudaStreamSynchronize(st));
}

// A whole solve of c.b at one precision, chunks of Arnoldi steps replayed
// (as a graph) until the control block reports the end.
template <typename T>
void core_solve(KrylovSolver &ks, Core<T> &c, bool use_graph, KrylovPrecond pc, long *launches, cudaStream_t st)
{
    start_solve(ks, c, st);
    if (launches) *launches += 1;
    if (use_graph && !*c.graph) {
        cudaGraph_t g;
        CB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < ks.chunk; ++k) arnoldi_step(ks, c, pc, st);
        CB_CUDA(cudaStreamEndCapture(st, &g));
        CB_CUDA(cudaGraphInstantiate(c.graph, g, 0));
        cudaGraphDestroy(g);
    }
    const long max_chunks = c.maxit / ks.chunk + 2;
    for (long chunks = 0;; ++chunks) {
        if (use_graph) {
            CB_CUDA(cudaGraphLaunch(*c.graph, st));
        } else {
            for (int k = 0; k < ks.chunk; ++k) arnoldi_step(ks, c, pc, st);
            CB_CUDA(cudaGetLastError());
        }
        if (launches) *launches += (long)kStepLaunches * ks.chunk;
        read_ctl(c.ctl, c.ctl_h, st);
        if (c.ctl_h->done) break;
        if (chunks > max_chunks) throw cb_status_error(CB_ERR_TIMEOUT, "the Krylov solve did not report an end");
    }
}

// Nested precision: each outer (FP64) Arnoldi step is preconditioned by an
// FP32 FGMRES solve with the FP32 matrix and block inverses.
void nested_solve(KrylovSolver &ks, bool use_graph, long *launches, cudaStream_t st)
{
    Core<double> c = core64(ks, 0);
    Core<float> in = core32(ks);
    const long n = ks.n;
    start_solve(ks, c, st);
    read_ctl(c.ctl, c.ctl_h, st);
    for (int steps = 0; !c.ctl_h->done; ++steps) {
        if (steps > c.maxit + 1) throw cb_status_error(CB_ERR_TIMEOUT, "the Krylov solve did not report an end");
        kry_outer_pre_kernel<<<nb(n), kKT, 0, st>>>(c.ctl, c.w, c.V, in.b, n);
        core_solve(ks, in, use_graph, KrylovPrecond::block_jacobi, launches, st);
        ks.inner_iterations += in.ctl_h->iters;
        kry_outer_post_kernel<<<nb(n), kKT, 0, st>>>(c.ctl, in.x, c.Z, n);
        step_after_precond(ks, c, st);
        CB_CUDA(cudaGetLastError());
        if (launches) *launches += 9;
        read_ctl(c.ctl, c.ctl_h, st);
    }
}

}  // namespace

int krylov_solve(KrylovSolver &ks, const double *b, double *x, cudaStream_t st, bool use_graph, KrylovPrecond pc,
                 long *launches)
{
    const long n = ks.n;
    CB_CUDA(cudaMemcpyAsync(ks.b, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    if (ks.nested && pc == KrylovPrecond::block_jacobi) {
        nested_solve(ks, use_graph, launches, st);
    } else {
        Core<double> c = core64(ks, pc == KrylovPrecond::learned ? 1 : 0);
        core_solve(ks, c, use_graph, pc, launches, st);
    }
    CB_CUDA(cudaMemcpyAsync(x, ks.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    const KrylovCtl &c = *ks.ctl_h;
    ks.solves++;
    ks.iterations_total += c.iters;
    ks.last_iters = c.iters;
    ks.last_resid = c.bnorm > 0 ? c.resid / c.bnorm : 0.0;
    if (c.status == 2) throw cb_status_error(CB_ERR_NUMERIC, "the Krylov solve broke down (non-finite value)");
    if (c.status == 1) ks.unconverged++;
    return c.iters;
}

}  // namespace cb
