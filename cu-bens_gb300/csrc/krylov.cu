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

__device__ __forceinline__ double warp_sum(double v)
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

// v_j = w * scale; z_j = B^-1 v_j over the row's block.
template <typename T>
__global__ void kry_bj_apply_kernel(const KrylovCtl *__restrict__ ctl, const double *__restrict__ w,
                                    double *__restrict__ V, double *__restrict__ Z, const int *__restrict__ row_blk,
                                    const int *__restrict__ blk_start, const int *__restrict__ blk_off,
                                    const T *__restrict__ binv, long n)
{
    if (ctl->done) return;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = ctl->j;
    const double sc = ctl->scale;
    V[(size_t)j * n + i] = w[i] * sc;
    const int b = row_blk[i];
    const int s0 = blk_start[b], bs = blk_start[b + 1] - s0;
    const T *B = binv + blk_off[b] + (i - s0) * bs;
    double z = 0;
    for (int c = 0; c < bs; ++c) z += (double)B[c] * (w[s0 + c] * sc);
    Z[(size_t)j * n + i] = z;
}

// ---- products and Gram-Schmidt passes ----

// 8 lanes per row, fixed lane order. mode 0: y = A z_j (while the solve
// runs); mode 1: y = b - A x (when a cycle ends unconverged); mode 2: y = A x.
__global__ void kry_spmv_kernel(const KrylovCtl *__restrict__ ctl, int mode, const int *__restrict__ rowptr,
                                const int *__restrict__ col, const double *__restrict__ val,
                                const double *__restrict__ xin, const double *__restrict__ bvec,
                                double *__restrict__ y, long n)
{
    if (mode == 0 && ctl->done) return;
    if (mode == 1 && (ctl->done || !ctl->finish || ctl->conv)) return;
    const double *x = mode == 0 ? xin + (size_t)ctl->j * n : xin;
    const long row = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 3;
    const int lane = threadIdx.x & 7;
    double acc = 0;
    if (row < n)
        for (int k = rowptr[row] + lane; k < rowptr[row + 1]; k += 8) acc += val[k] * x[col[k]];
    acc += __shfl_xor_sync(0xffffffffu, acc, 4);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    if (row < n && lane == 0) y[row] = mode == 1 ? bvec[row] - acc : acc;
}

// partial[k*nred + blk] = v_k . w over the block's rows, k <= j (one warp per k)
__device__ void chunk_dots(const KrylovCtl *ctl, const double *V, const double *w, double *partial, long n,
                           long r0, long r1, int nred)
{
    const int j = ctl->j;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int k = warp; k <= j; k += nw) {
        const double *v = V + (size_t)k * n;
        double acc = 0;
        for (long i = r0 + lane; i < r1; i += 32) acc += v[i] * w[i];
        acc = warp_sum(acc);
        if (lane == 0) partial[k * nred + blockIdx.x] = acc;
    }
}

__global__ void kry_dots_kernel(const KrylovCtl *__restrict__ ctl, const double *__restrict__ V,
                                const double *__restrict__ w, double *__restrict__ partial, long n, int rpr,
                                int nred)
{
    if (ctl->done) return;
    const long r0 = blockIdx.x * (long)rpr, r1 = min(n, r0 + rpr);
    chunk_dots(ctl, V, w, partial, n, r0, r1, nred);
}

// hp[k] = sum of the partials (one warp per k); pass 0 starts hcol, pass 1 adds
__global__ void kry_reduce_kernel(KrylovCtl *__restrict__ ctl, const double *__restrict__ partial, int nred,
                                  int pass)
{
    if (ctl->done) return;
    const int j = ctl->j;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int k = warp; k <= j; k += nw) {
        double acc = 0;
        for (int b = lane; b < nred; b += 32) acc += partial[k * nred + b];
        acc = warp_sum(acc);
        if (lane == 0) {
            ctl->hp[k] = acc;
            ctl->hcol[k] = pass == 0 ? acc : ctl->hcol[k] + acc;
        }
    }
}

// w -= sum_k hp[k] v_k over the block's rows, then (second) the pass-2 dots
// or (last) the partial |w|^2.
__global__ void kry_update_kernel(const KrylovCtl *__restrict__ ctl, const double *__restrict__ V,
                                  double *__restrict__ w, double *__restrict__ partial, long n, int rpr, int nred,
                                  int last)
{
    if (ctl->done) return;
    __shared__ double hp[kMaxRestart + 1];
    __shared__ double red[kKT / 32];
    const int j = ctl->j;
    for (int k = threadIdx.x; k <= j; k += blockDim.x) hp[k] = ctl->hp[k];
    __syncthreads();
    const long r0 = blockIdx.x * (long)rpr, r1 = min(n, r0 + rpr);
    double nrm = 0;
    for (long i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        double s = w[i];
        for (int k = 0; k <= j; ++k) s -= hp[k] * V[(size_t)k * n + i];
        w[i] = s;
        nrm += s * s;
    }
    if (!last) {
        __syncthreads();
        chunk_dots(ctl, V, w, partial, n, r0, r1, nred);
        return;
    }
    nrm = warp_sum(nrm);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nrm;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
        partial[blockIdx.x] = s;
    }
}

// partial[blk] = |w|^2 over the block's rows. mode 0: always (start of a
// solve); mode 1: when a cycle ends unconverged (the restart residual).
__global__ void kry_norm_kernel(const KrylovCtl *__restrict__ ctl, int mode, const double *__restrict__ w,
                                double *__restrict__ partial, long n, int rpr)
{
    if (mode == 1 && (ctl->done || !ctl->finish || ctl->conv)) return;
    __shared__ double red[kKT / 32];
    const long r0 = blockIdx.x * (long)rpr, r1 = min(n, r0 + rpr);
    double s = 0;
    for (long i = r0 + threadIdx.x; i < r1; i += blockDim.x) s += w[i] * w[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        partial[blockIdx.x] = t;
    }
}

__device__ double sum_partials(const double *partial, int nred)
{
    double acc = 0;
    for (int b = threadIdx.x; b < nred; b += 32) acc += partial[b];
    return warp_sum(acc);
}

// start of a solve (one warp): |b| from the partials, the first cycle
__global__ void kry_start_kernel(KrylovCtl *__restrict__ ctl, const double *__restrict__ partial, int nred,
                                 int m, int maxit, double rtol)
{
    const double bb = sum_partials(partial, nred);
    if (threadIdx.x != 0) return;
    const double bn = sqrt(bb);
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
}

// Closes Arnoldi step j (one warp): h_{j+1,j} = |w|, rotations, residual
// estimate |g_{j+1}|; at the end of a cycle y = R^-1 g.
__global__ void kry_close_kernel(KrylovCtl *__restrict__ ctl, const double *__restrict__ partial, int nred)
{
    if (ctl->done) return;
    const double ww = sum_partials(partial, nred);
    if (threadIdx.x != 0) return;
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

// x += Z y at the end of a cycle
__global__ void kry_xupdate_kernel(const KrylovCtl *__restrict__ ctl, const double *__restrict__ Z,
                                   double *__restrict__ x, long n)
{
    if (ctl->done || !ctl->finish) return;
    __shared__ double y[kMaxRestart];
    const int nc = ctl->ncols;
    for (int k = threadIdx.x; k < nc; k += blockDim.x) y[k] = ctl->y[k];
    __syncthreads();
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = x[i];
    for (int k = 0; k < nc; ++k) s += y[k] * Z[(size_t)k * n + i];
    x[i] = s;
}

// After a finished cycle: done when the estimate converged, else restart
// from the true residual r = b - A x (in w, its norm in the partials).
__global__ void kry_restart_kernel(KrylovCtl *__restrict__ ctl, const double *__restrict__ partial, int nred)
{
    if (ctl->done || !ctl->finish) return;
    const bool conv = ctl->conv != 0;
    const double rr = conv ? 0.0 : sum_partials(partial, nred);
    if (threadIdx.x != 0) return;
    if (conv) {
        ctl->status = 0;
        ctl->done = 1;
        return;
    }
    const double beta = sqrt(rr);
    ctl->resid = beta;
    ctl->beta = beta;
    if (beta <= ctl->tol_abs) {
        ctl->status = 0;
        ctl->done = 1;
        return;
    }
    if (ctl->iters >= ctl->maxit || !isfinite(beta)) {
        ctl->status = isfinite(beta) ? 1 : 2;
        ctl->done = 1;
        return;
    }
    ctl->restarts += 1;
    ctl->j = 0;
    ctl->finish = 0;
    ctl->g[0] = beta;
    ctl->scale = 1.0 / beta;
}

inline unsigned nb(long n, int t = kKT) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------------------

void krylov_alloc(KrylovSolver &ks, const HostModel &h, int restart, int maxit, bool fp32_precond,
                  cudaStream_t st)
{
    const long n = h.neq;
    ks.n = n;
    ks.m = std::max(2, std::min(restart > 0 ? restart : 50, kMaxRestart));
    ks.maxit = maxit > 0 ? maxit : 2000;
    ks.fp32_precond = fp32_precond;
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
    ks.rows_per_red = (int)((n + ks.nred - 1) / ks.nred);
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
    void *ptrs[] = {ks.rowptr, ks.col,      ks.diag,    ks.val,     ks.amap_ptr, ks.amap_src, ks.amap_dst,
                    ks.amap_dst2, ks.blk_start, ks.blk_off, ks.row_blk, ks.binv, ks.V,        ks.Z,
                    ks.w,      ks.b,        ks.x,       ks.partial, ks.ctl};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (ks.ctl_h) cudaFreeHost(ks.ctl_h);
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
}

void krylov_spmv(const KrylovSolver &ks, const double *x, double *y, cudaStream_t st)
{
    kry_spmv_kernel<<<nb(ks.n * 8), kKT, 0, st>>>(ks.ctl, 2, ks.rowptr, ks.col, ks.val, x, nullptr, y, ks.n);
}

void krylov_apply_learned(KrylovSolver &ks, cudaStream_t st)
{
    (void)st;
    if (!ks.mpnn) throw cb_status_error(CB_ERR_STATE, "no learned preconditioner attached");
}

namespace {

// One Arnoldi step (12 launches).
void arnoldi_step(KrylovSolver &ks, KrylovPrecond pc, cudaStream_t st)
{
    const long n = ks.n;
    if (pc == KrylovPrecond::learned) {
        krylov_apply_learned(ks, st);
    } else if (ks.fp32_precond) {
        kry_bj_apply_kernel<float><<<nb(n), kKT, 0, st>>>(ks.ctl, ks.w, ks.V, ks.Z, ks.row_blk, ks.blk_start,
                                                          ks.blk_off, (const float *)ks.binv, n);
    } else {
        kry_bj_apply_kernel<double><<<nb(n), kKT, 0, st>>>(ks.ctl, ks.w, ks.V, ks.Z, ks.row_blk, ks.blk_start,
                                                           ks.blk_off, (const double *)ks.binv, n);
    }
    kry_spmv_kernel<<<nb(n * 8), kKT, 0, st>>>(ks.ctl, 0, ks.rowptr, ks.col, ks.val, ks.Z, nullptr, ks.w, n);
    kry_dots_kernel<<<ks.nred, kKT, 0, st>>>(ks.ctl, ks.V, ks.w, ks.partial, n, ks.rows_per_red, ks.nred);
    kry_reduce_kernel<<<1, kKT, 0, st>>>(ks.ctl, ks.partial, ks.nred, 0);
    kry_update_kernel<<<ks.nred, kKT, 0, st>>>(ks.ctl, ks.V, ks.w, ks.partial, n, ks.rows_per_red, ks.nred, 0);
    kry_reduce_kernel<<<1, kKT, 0, st>>>(ks.ctl, ks.partial, ks.nred, 1);
    kry_update_kernel<<<ks.nred, kKT, 0, st>>>(ks.ctl, ks.V, ks.w, ks.partial, n, ks.rows_per_red, ks.nred, 1);
    kry_close_kernel<<<1, 32, 0, st>>>(ks.ctl, ks.partial, ks.nred);
    kry_xupdate_kernel<<<nb(n), kKT, 0, st>>>(ks.ctl, ks.Z, ks.x, n);
    kry_spmv_kernel<<<nb(n * 8), kKT, 0, st>>>(ks.ctl, 1, ks.rowptr, ks.col, ks.val, ks.x, ks.b, ks.w, n);
    kry_norm_kernel<<<ks.nred, kKT, 0, st>>>(ks.ctl, 1, ks.w, ks.partial, n, ks.rows_per_red);
    kry_restart_kernel<<<1, 32, 0, st>>>(ks.ctl, ks.partial, ks.nred);
}

constexpr int kStepLaunches = 12;

}  // namespace

int krylov_solve(KrylovSolver &ks, const double *b, double *x, cudaStream_t st, bool use_graph, KrylovPrecond pc,
                 long *launches)
{
    const long n = ks.n;
    CB_CUDA(cudaMemcpyAsync(ks.b, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    CB_CUDA(cudaMemcpyAsync(ks.w, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    CB_CUDA(cudaMemsetAsync(ks.x, 0, sizeof(double) * n, st));
    kry_norm_kernel<<<ks.nred, kKT, 0, st>>>(ks.ctl, 0, ks.w, ks.partial, n, ks.rows_per_red);
    kry_start_kernel<<<1, 32, 0, st>>>(ks.ctl, ks.partial, ks.nred, ks.m, ks.maxit, ks.rtol);
    CB_CUDA(cudaGetLastError());
    if (launches) *launches += 2;
    const int gi = pc == KrylovPrecond::learned ? 1 : 0;
    if (use_graph && !ks.step_graph[gi]) {
        cudaGraph_t g;
        CB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int c = 0; c < ks.chunk; ++c) arnoldi_step(ks, pc, st);
        CB_CUDA(cudaStreamEndCapture(st, &g));
        CB_CUDA(cudaGraphInstantiate(&ks.step_graph[gi], g, 0));
        cudaGraphDestroy(g);
    }
    const long max_chunks = ks.maxit / ks.chunk + 2;
    const size_t head = offsetof(KrylovCtl, hp);
    long chunks = 0;
    for (;;) {
        if (use_graph) {
            CB_CUDA(cudaGraphLaunch(ks.step_graph[gi], st));
        } else {
            for (int c = 0; c < ks.chunk; ++c) arnoldi_step(ks, pc, st);
            CB_CUDA(cudaGetLastError());
        }
        if (launches) *launches += (long)kStepLaunches * ks.chunk;
        ++chunks;
        CB_CUDA(cudaMemcpyAsync(ks.ctl_h, ks.ctl, head, cudaMemcpyDeviceToHost, st));
        CB_CUDA(cudaStreamSynchronize(st));
        if (ks.ctl_h->done) break;
        if (chunks > max_chunks)
            throw cb_status_error(CB_ERR_TIMEOUT, "the Krylov solve did not report an end");
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
