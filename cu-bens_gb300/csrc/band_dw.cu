// Band LDL^T and its solves in double-word ("double-float") arithmetic.
//
// The same factorisation as band.cu (skyfact's result in the reference's
// equation order, solve.c:539-653: pivots ssd and the indefiniteness flag
// det), for bands whose conditioning an FP32 factor cannot carry and whose
// size makes native FP64 slow on GB300: the 1.58M-equation DKT panel (band
// 3,083) takes 7.6e12 multiply-adds per factorisation. Every entry of the
// band is a pair of floats (dw.cuh, about 48 significant bits) and all
// arithmetic runs on the FP32 pipe.
//
// Factor: one persistent cooperative kernel, right-looking over 64-column
// panels, two bounded grid barriers per panel:
//   1. the panel's factored diagonal block (L below, D on the diagonal) and
//      1/D come from the look-ahead buffer (CTA 0 factored the block during
//      the previous panel; for the first panel every CTA factors it);
//   2. one warp per panel row r forms W_r (W_r L_pp^T = A_r, by
//      substitution, so W_r = L_r D) and L_r = W_r D^-1 into the band, and W
//      and L into a k-major buffer;
//   -- grid barrier --
//   3. the trailing lower triangle of the band window in 64 x 64 tiles,
//      A_ij -= sum_k W_ik L_jk; CTA 0 takes only tile (0,0), which is the
//      next panel's diagonal block, and factors that block right after its
//      update while the other CTAs work through the rest of the triangle;
//   -- grid barrier --
// Two kernels differ in step 3. factor_dw_tc_kernel (the default) forms the
// tile products on the tensor cores: step 2 splits every W and L row into
// bfloat16 slices whose mma.sync products accumulate exactly in FP32 (the
// comment above the kernel gives the bounds). factor_dw_kernel forms them
// on the FP32 pipe, each thread a 4 x 4 block of double-word accumulators.
// Then inv_block_kernel forms, for every 128-row block of the matrix, the
// inverse X_i of its unit-lower diagonal block: its ten lower 32 x 32 tiles,
// once row-major and once column-major.
//
// Solve: one cooperative kernel over 128-row blocks, forward and backward,
// one grid barrier per block each way. Every CTA forms the block's solution
// y_i = X_i t_i (or x_i = X_i^T u_i) from the block inverse in shared memory
// and applies it to 32 of the band's rows (columns) below (above) the
// block. Nothing a step reads besides the solution's 128 values depends on
// the solution: each CTA copies the next block's inverse into shared memory
// (cp.async) and each thread the next step's band values into registers
// before the barrier that ends a step.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>

#include "dw.cuh"
#include "grid_barrier.cuh"
#include "internal.hpp"

#define CB_CUDA_DW(x)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + \
                                     " at " __FILE__ ":" + std::to_string(__LINE__));      \
    } while (0)

namespace cb {

namespace {

constexpr int NB = 32;        // tile size of the block inverses
constexpr int PW = 64;        // panel width of the factor
constexpr int TW = 64;        // tile of the factor's trailing update (4 x 4 accumulators per thread)
constexpr int SB = 128;       // block size of the solve
constexpr int kTiles = (SB / NB) * (SB / NB + 1) / 2;  // lower 32 x 32 tiles of a block
constexpr int kThreads = 256;

__device__ __forceinline__ dw dw_zero() { return dw{0.0f, 0.0f}; }

__device__ __forceinline__ dw shfl_dw(dw v, int src)
{
    return dw{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

struct DwFactorArgs {
    dw *band;       // ld * npad, L(i, j) at band[j * ld + (i - j)]
    long ld, bw, npad, n;
    dw *dinv;       // npad: 1/D
    double *ssd;    // n pivots
    int *flags;     // [0] a pivot <= 0, [1] a zero pivot
    dw *wl;         // 2 * 64 * (bw + 1): W (row r of column k at k * ms + r, ms = m rounded up to
                    // even), then L at offset 64 * (bw + 1)
    dw *look;       // the next panel's factored block (64 x 64) and 1/D (64)
    GridBarrier *bar;
    long long max_polls;
    __nv_bfloat16 *wsl, *lsl;  // tensor-core factor: slices [NS][mrow][64] of W and of L
    int *ew, *el;               // ... row exponents [mrow]
    long mrow;                  // rows of a slice (bw + 1)
};

// shared memory of the factor: the diagonal block (and 1/D), W and L of a tile
constexpr int KH = PW / 2;  // depth of one stage of a tile's update (half the panel)
struct DwFactorSmem {
    dw A[PW][PW + 1];     // factored diagonal block of the panel: L below, D on the diagonal
    dw di[PW];            // 1/D
    dw Wt[2][KH][TW];     // W of a tile's rows for one stage, k-major, two buffers
    dw Lt[2][KH][TW];     // L of a tile's columns for one stage
};

__device__ __forceinline__ void cp_async16_zfill(void *smem, const void *gmem, bool valid)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 16 : 0;  // 0: the 16 bytes are zero-filled, nothing is read
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit_f() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_f() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Entry e of the lower triangle of a 64 x 64 block listed by columns
// (column j starts at j (129 - j) / 2): its row i and column j.
__device__ __forceinline__ void tri_entry(int e, int &i, int &j)
{
    constexpr int T2 = 2 * PW + 1;
    int c = (int)((T2 - sqrtf((float)(T2 * T2 - 8 * e))) * 0.5f);
    while (c > 0 && c * (T2 - c) / 2 > e) --c;
    while ((c + 1) * (T2 - (c + 1)) / 2 <= e) ++c;
    j = c;
    i = e - c * (T2 - c) / 2 + c;
}

// LDL^T of the 64 x 64 block in A (lower triangle) by all threads of the CTA,
// one CTA barrier per column: every thread forms 1/D_k itself from the final
// pivot and the update uses the unscaled column (W = L D). The entries of
// step k are the tail of the triangle's column list from column k + 1, dealt
// out evenly to the threads. The columns are scaled by 1/D at the end. On
// return L below the diagonal, D on it, di = 1/D.
__device__ void ldlt_block_dw(dw (*A)[PW + 1], dw *di)
{
    const int tid = threadIdx.x;
    constexpr int total = PW * (PW + 1) / 2;
    for (int k = 0; k < PW; ++k) {
        const dw dk = dw_recip(A[k][k]);
        for (int e = (k + 1) * (2 * PW - k) / 2 + tid; e < total; e += kThreads) {
            int i, j;
            tri_entry(e, i, j);
            A[i][j] = dw_sub(A[i][j], dw_mul(dw_mul(A[i][k], dk), A[j][k]));
        }
        if (tid == 0) di[k] = dk;
        __syncthreads();
    }
    for (int e = tid; e < total; e += kThreads) {
        int i, j;
        tri_entry(e, i, j);
        if (i > j) A[i][j] = dw_mul(A[i][j], di[j]);
    }
    __syncthreads();
}

// The factored block of panel p into the band, 1/D, the FP64 pivots and the flags.
__device__ void record_block(const DwFactorArgs &a, long p, const dw (*A)[PW + 1], const dw *di)
{
    const int tid = threadIdx.x;
    for (int e = tid; e < PW * PW; e += kThreads) {
        const int j = e / PW, i = e % PW;
        if (i >= j && i - j <= a.bw) a.band[(p + j) * a.ld + (i - j)] = A[i][j];
    }
    if (tid < PW) {
        a.dinv[p + tid] = di[tid];
        const long g = p + tid;
        if (g < a.n) {
            const double d = dw_to_double(A[tid][tid]);
            a.ssd[g] = d;
            if (!(d > 0.0)) atomicOr(&a.flags[0], 1);
            if (d == 0.0) atomicOr(&a.flags[1], 1);
        }
    }
}

__device__ void load_block(const DwFactorArgs &a, long p, dw (*A)[PW + 1])
{
    for (int e = threadIdx.x; e < PW * PW; e += kThreads) {
        const int j = e / PW, i = e % PW;
        A[i][j] = (i >= j && i - j <= a.bw) ? a.band[(p + j) * a.ld + (i - j)] : dw_zero();
    }
    __syncthreads();
}

// Row r of panel p (one warp; lane holds columns lane and lane + 32):
// W_r by substitution against the factored diagonal block (W_r L_pp^T =
// A_r), L_r = W_r D^-1 into the band. Returns W and L in w0, w1, l0, l1.
__device__ __forceinline__ void panel_row(const DwFactorArgs &a, const dw (*A)[PW + 1], const dw *di, long p,
                                          long r, int lane, dw &w0, dw &w1, dw &l0, dw &l1)
{
    const long ld = a.ld, bw = a.bw;
    const long off0 = PW + r - lane, off1 = off0 - 32;
    w0 = off0 <= bw ? a.band[(p + lane) * ld + off0] : dw_zero();
    w1 = off1 <= bw ? a.band[(p + 32 + lane) * ld + off1] : dw_zero();
    for (int k = 0; k < 32; ++k) {
        const dw wk = shfl_dw(w0, k);
        if (lane > k) w0 = dw_sub(w0, dw_mul(wk, A[lane][k]));
        w1 = dw_sub(w1, dw_mul(wk, A[32 + lane][k]));
    }
    for (int k = 0; k < 31; ++k) {
        const dw wk = shfl_dw(w1, k);
        if (lane > k) w1 = dw_sub(w1, dw_mul(wk, A[32 + lane][32 + k]));
    }
    l0 = dw_mul(w0, di[lane]);
    l1 = dw_mul(w1, di[32 + lane]);
    if (off0 <= bw) a.band[(p + lane) * ld + off0] = l0;
    if (off1 <= bw) a.band[(p + 32 + lane) * ld + off1] = l1;
}

// Two rows r and r2 of panel p at once (the second only when v2): the
// same arithmetic as panel_row with two independent dependency chains.
__device__ __forceinline__ void panel_row2(const DwFactorArgs &a, const dw (*A)[PW + 1], const dw *di, long p,
                                           long r, long r2, bool v2, int lane, dw *w, dw *l)
{
    const long ld = a.ld, bw = a.bw;
    const long o0 = PW + r - lane, o1 = o0 - 32, q0 = PW + r2 - lane, q1 = q0 - 32;
    dw w0 = o0 <= bw ? a.band[(p + lane) * ld + o0] : dw_zero();
    dw w1 = o1 <= bw ? a.band[(p + 32 + lane) * ld + o1] : dw_zero();
    dw x0 = v2 && q0 <= bw ? a.band[(p + lane) * ld + q0] : dw_zero();
    dw x1 = v2 && q1 <= bw ? a.band[(p + 32 + lane) * ld + q1] : dw_zero();
    for (int k = 0; k < 32; ++k) {
        const dw wk = shfl_dw(w0, k), xk = shfl_dw(x0, k);
        const dw akl = A[lane][k], ak2 = A[32 + lane][k];
        if (lane > k) {
            w0 = dw_sub(w0, dw_mul(wk, akl));
            x0 = dw_sub(x0, dw_mul(xk, akl));
        }
        w1 = dw_sub(w1, dw_mul(wk, ak2));
        x1 = dw_sub(x1, dw_mul(xk, ak2));
    }
    for (int k = 0; k < 31; ++k) {
        const dw wk = shfl_dw(w1, k), xk = shfl_dw(x1, k);
        const dw ak = A[32 + lane][32 + k];
        if (lane > k) {
            w1 = dw_sub(w1, dw_mul(wk, ak));
            x1 = dw_sub(x1, dw_mul(xk, ak));
        }
    }
    w[0] = w0;
    w[1] = w1;
    w[2] = x0;
    w[3] = x1;
    l[0] = dw_mul(w0, di[lane]);
    l[1] = dw_mul(w1, di[32 + lane]);
    l[2] = dw_mul(x0, di[lane]);
    l[3] = dw_mul(x1, di[32 + lane]);
    if (o0 <= bw) a.band[(p + lane) * ld + o0] = l[0];
    if (o1 <= bw) a.band[(p + 32 + lane) * ld + o1] = l[1];
    if (v2 && q0 <= bw) a.band[(p + lane) * ld + q0] = l[2];
    if (v2 && q1 <= bw) a.band[(p + 32 + lane) * ld + q1] = l[3];
}

__global__ void __launch_bounds__(kThreads, 1) factor_dw_kernel(DwFactorArgs a)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    DwFactorSmem &sm = *reinterpret_cast<DwFactorSmem *>(dyn);
    auto &A = sm.A;
    auto &di = sm.di;
    auto &Wt = sm.Wt;
    auto &Lt = sm.Lt;
    unsigned ep = 0;  // grid barriers passed
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const long ld = a.ld, bw = a.bw;
    const unsigned G = gridDim.x;
    for (long p = 0; p < a.npad; p += PW) {
        long m = a.npad - p - PW;
        if (m > bw) m = bw;
        if (m < 0) m = 0;
        // ---- 1. the factored diagonal block ----
        if (p == 0) {
            load_block(a, 0, A);
            ldlt_block_dw(A, di);
            if (blockIdx.x == 0) record_block(a, 0, A, di);
        } else {
            for (int e = tid; e < PW * PW; e += kThreads) A[e / PW][e % PW] = a.look[e];
            if (tid < PW) di[tid] = a.look[PW * PW + tid];
        }
        __syncthreads();
        // ---- 2. panel rows by substitution (one warp per row, lane: columns lane and lane + 32) ----
        // W and L of the panel, k-major with an even row stride (16-byte rows for cp.async)
        const long ms = (m + 1) & ~1L;
        dw *wbuf = a.wl, *lbuf = a.wl + (long)PW * (bw + 1);
        if (ms > m && blockIdx.x == 0 && tid < PW) {
            wbuf[tid * ms + m] = dw_zero();
            lbuf[tid * ms + m] = dw_zero();
        }
        for (long r = blockIdx.x * 8L + warp; r < m; r += G * 8L) {
            dw w0, w1, l0, l1;
            panel_row(a, A, di, p, r, lane, w0, w1, l0, l1);
            wbuf[lane * ms + r] = w0;
            wbuf[(32 + lane) * ms + r] = w1;
            lbuf[lane * ms + r] = l0;
            lbuf[(32 + lane) * ms + r] = l1;
        }
        if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
        // ---- 3. trailing triangle; CTA 0: tile (0,0), then the next block ----
        const long nt = (m + TW - 1) / TW;
        const long ntiles = nt * (nt + 1) / 2;
        const int tx = tid % 16, ty = tid / 16;
        // the tiles t = first, first + stride, ... (< last) in stages of half the
        // panel's depth; the next stage's W and L come in by cp.async while
        // the current one computes
        auto tiles = [&](long first, long stride, long last) {
            if (first >= last) return;
            const long nst = 2 * ((last - first + stride - 1) / stride);
            auto coords = [&](long t, long &r0, long &j0) {
                long ti = (long)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
                while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
                while (ti * (ti + 1) / 2 > t) --ti;
                r0 = ti * TW;
                j0 = (t - ti * (ti + 1) / 2) * TW;
            };
            auto fetch = [&](long st) {
                long r0, j0;
                coords(first + (st / 2) * stride, r0, j0);
                const int h = (int)(st & 1), b = (int)(st & 1);
                // 2 pairs per 16-byte chunk: KH x TW / 2 chunks per matrix
                for (int e = tid; e < KH * TW / 2; e += kThreads) {
                    const int k = e / (TW / 2), q = 2 * (e % (TW / 2));
                    const long kk = KH * h + k;
                    cp_async16_zfill(&Wt[b][k][q], wbuf + kk * ms + r0 + q, r0 + q < m);
                    cp_async16_zfill(&Lt[b][k][q], lbuf + kk * ms + j0 + q, j0 + q < m);
                }
                cp_async_commit_f();
            };
            dw_acc acc[4][4];
            long r0 = 0, j0 = 0;
            fetch(0);
            for (long st = 0; st < nst; ++st) {
                const int b = (int)(st & 1);
                if (st + 1 < nst) fetch(st + 1);
                if ((st & 1) == 0) {
                    // a new tile: rows r0 + tx + 16 i, columns j0 + ty + 16 j
                    coords(first + (st / 2) * stride, r0, j0);
#pragma unroll
                    for (int j = 0; j < 4; ++j)
#pragma unroll
                        for (int i = 0; i < 4; ++i) acc_zero(acc[i][j]);
                }
                if (st + 1 < nst) cp_async_wait_f<1>();
                else cp_async_wait_f<0>();
                __syncthreads();
#pragma unroll 2
                for (int k = 0; k < KH; ++k) {
                    dw w[4], l[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        w[i] = Wt[b][k][tx + 16 * i];
                        l[i] = Lt[b][k][ty + 16 * i];
                    }
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc_fma(acc[i][j], w[i], l[j]);
                }
                __syncthreads();  // the buffer is refilled by the stage after next
                if (st & 1) {
                    dw old[4][4];
#pragma unroll
                    for (int j = 0; j < 4; ++j)
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const long rr = r0 + tx + 16 * i, jj = j0 + ty + 16 * j;
                            old[i][j] = (rr < m && jj <= rr) ? a.band[(p + PW + jj) * ld + (rr - jj)] : dw_zero();
                        }
#pragma unroll
                    for (int j = 0; j < 4; ++j)
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const long rr = r0 + tx + 16 * i, jj = j0 + ty + 16 * j;
                            if (rr < m && jj <= rr)
                                a.band[(p + PW + jj) * ld + (rr - jj)] = dw_sub(old[i][j], acc_value(acc[i][j]));
                        }
                }
            }
            __syncthreads();  // the tiles' band values are written before the caller reads them
        };
        if (blockIdx.x == 0) {
            // tile (0,0) is the next panel's diagonal block (rows and columns
            // 0..63 of the window); band rows below the window, for a band
            // narrower than a panel, take no update from this panel
            tiles(0, 1, ntiles > 0 ? 1 : 0);
            if (p + PW < a.npad) {
                const long pn = p + PW;
                load_block(a, pn, A);
                ldlt_block_dw(A, di);
                record_block(a, pn, A, di);
                for (int e = tid; e < PW * PW; e += kThreads) a.look[e] = A[e / PW][e % PW];
                if (tid < PW) a.look[PW * PW + tid] = di[tid];
            }
            if (G == 1) tiles(1, 1, ntiles);
        } else {
            tiles(blockIdx.x, G - 1, ntiles);
        }
        if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
    }
}

// ---------------------------------------------------------------------------
// The same factor with the trailing update on the tensor cores.
//
// Every row of the panel's W (and of L) is split into NS bfloat16 slices of
// 8 bits. With 2^e the row's bound (|v| < 2^e for its 64 values),
// v = 2^(e-7) sum_s q_s 2^(-8s) with integers |q_s| <= 129; slice s holds
// q_s 2^(-8s), exact in bfloat16. The product of slices a and b is
// q_a q_b 2^(-8c), c = a + b, with |q_a q_b| < 2^15, so a 64-term sum of at
// most six such products per diagonal c stays below 2^24 units of 2^(-8c):
// mma.sync's FP32 accumulation of each of the diagonals 0, 1 and 2 is
// exact. The diagonals 3 .. NS-1 share one accumulator, whose rounding is
// below 2^-48 of the product of the two row bounds, and so are the
// diagonals dropped (c >= NS): the resolution of the double-word format
// itself. 21 slice products in all. Each output then adds its four
// accumulators in double-word arithmetic, scales the sum by the two row
// exponents and subtracts it from the band (the error-free splitting of
// Ozaki, Ogita, Oishi and Rump, Numer. Algorithms 59 (2012) 95-118, on
// 8-bit slices).
constexpr int NS = 6;         // slices per value: 7 + 5 x 8 = 47 bits
constexpr int NA = 4;         // accumulators: diagonals 0, 1, 2 and 3 .. NS-1
constexpr int SST = KH + 8;   // shared row stride of a stage's slices (bf16): conflict-free fragments

struct DwTcSmem {
    dw A[PW][PW + 1];
    dw di[PW];
    __nv_bfloat16 Ws[2][NS][TW][SST];  // W slices of a tile's rows, one stage (KH columns of the panel)
    __nv_bfloat16 Ls[2][NS][TW][SST];  // L slices of a tile's columns
};

__device__ __forceinline__ void mma16816(float *c, const unsigned *a, const unsigned *b)
{
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Slices of one panel row (one warp; lane holds columns lane and lane + 32)
// into out[s][r][0..63], its exponent e - 7 into ex[r].
__device__ void slice_row(dw v0, dw v1, __nv_bfloat16 *out, int *ex, long r, long mrow, int lane)
{
    float mx = fmaxf(fabsf(v0.hi), fabsf(v1.hi));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.0f) (void)frexpf(mx, &e);  // mx < 2^e, and so is every |v|
    const int sh = 7 - e;
    float h0 = ldexpf(v0.hi, sh), l0 = ldexpf(v0.lo, sh), h1 = ldexpf(v1.hi, sh), l1 = ldexpf(v1.lo, sh);
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const float q0 = rintf(h0), q1 = rintf(h1);
        __nv_bfloat16 *row = out + ((long)s * mrow + r) * PW;
        row[lane] = __float2bfloat16_rn(ldexpf(q0, -8 * s));
        row[32 + lane] = __float2bfloat16_rn(ldexpf(q1, -8 * s));
        // the remainder (h - q is exact: |h - q| <= 1/2 and q = rint(h)), times 2^8
        two_sum(__fsub_rn(h0, q0), l0, h0, l0);
        two_sum(__fsub_rn(h1, q1), l1, h1, l1);
        h0 *= 256.0f;
        l0 *= 256.0f;
        h1 *= 256.0f;
        l1 *= 256.0f;
    }
    if (lane == 0) ex[r] = e - 7;
}

__global__ void __launch_bounds__(kThreads, 1) factor_dw_tc_kernel(DwFactorArgs a)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    DwTcSmem &sm = *reinterpret_cast<DwTcSmem *>(dyn);
    auto &A = sm.A;
    auto &di = sm.di;
    unsigned ep = 0;  // grid barriers passed
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const int g = lane >> 2, q = lane & 3;     // mma fragment coordinates
    const int wr = warp >> 1, wc = warp & 1;   // the warp's 16 rows and 32 columns of a 64 x 64 tile
    const long ld = a.ld, bw = a.bw, mrow = a.mrow;
    const unsigned G = gridDim.x;
    for (long p = 0; p < a.npad; p += PW) {
        long m = a.npad - p - PW;
        if (m > bw) m = bw;
        if (m < 0) m = 0;
        // ---- 1. the factored diagonal block ----
        if (p == 0) {
            load_block(a, 0, A);
            ldlt_block_dw(A, di);
            if (blockIdx.x == 0) record_block(a, 0, A, di);
        } else {
            for (int e = tid; e < PW * PW; e += kThreads) A[e / PW][e % PW] = a.look[e];
            if (tid < PW) di[tid] = a.look[PW * PW + tid];
        }
        __syncthreads();
        // ---- 2. panel rows by substitution, then their slices ----
        // Column k of W is scaled by 2^-f_k and column k of L by 2^f_k, with
        // 2^f_k near sqrt|D_k|: W L^T is unchanged and both rows take the
        // magnitudes of the Cholesky-like factor L |D|^(1/2), whose row
        // entries stay within the square root of the row's diagonal. Pivots
        // that differ by orders of magnitude (the shells' drilling DOFs) then
        // do not widen a row's range, which the row exponent of the slices
        // would turn into lost bits.
        int f0 = 0, f1 = 0;
        {
            int e0 = 0, e1 = 0;
            const float d0 = fabsf(A[lane][lane].hi), d1 = fabsf(A[32 + lane][32 + lane].hi);
            if (d0 > 0.0f) (void)frexpf(d0, &e0);
            if (d1 > 0.0f) (void)frexpf(d1, &e1);
            f0 = e0 / 2;
            f1 = e1 / 2;
        }
        for (long r = blockIdx.x * 8L + warp; r < m; r += 2 * G * 8L) {
            const long r2 = r + G * 8L;
            const bool v2 = r2 < m;
            dw w[4], l[4];
            panel_row2(a, A, di, p, r, r2, v2, lane, w, l);
            for (int h = 0; h < (v2 ? 2 : 1); ++h) {
                const long rr = h ? r2 : r;
                slice_row(dw{ldexpf(w[2 * h].hi, -f0), ldexpf(w[2 * h].lo, -f0)},
                          dw{ldexpf(w[2 * h + 1].hi, -f1), ldexpf(w[2 * h + 1].lo, -f1)}, a.wsl, a.ew, rr, mrow, lane);
                slice_row(dw{ldexpf(l[2 * h].hi, f0), ldexpf(l[2 * h].lo, f0)},
                          dw{ldexpf(l[2 * h + 1].hi, f1), ldexpf(l[2 * h + 1].lo, f1)}, a.lsl, a.el, rr, mrow, lane);
            }
        }
        if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
        // ---- 3. trailing triangle on the tensor cores; CTA 0: tile (0,0), then the next block ----
        const long nt = (m + TW - 1) / TW;
        const long ntiles = nt * (nt + 1) / 2;
        auto tiles = [&](long first, long stride, long last) {
            if (first >= last) return;
            const long nst = 2 * ((last - first + stride - 1) / stride);
            auto coords = [&](long t, long &r0, long &j0) {
                long ti = (long)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
                while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
                while (ti * (ti + 1) / 2 > t) --ti;
                r0 = ti * TW;
                j0 = (t - ti * (ti + 1) / 2) * TW;
            };
            // stage st: half h = st & 1 of the panel's columns of tile st / 2;
            // 16-byte chunks of 8 slice values, rows past m zero-filled
            auto fetch = [&](long st) {
                long r0, j0;
                coords(first + (st / 2) * stride, r0, j0);
                const int h = (int)(st & 1), b = (int)(st & 1);
                constexpr int CH = KH / 8;
#pragma unroll 1
                for (int e = tid; e < NS * TW * CH; e += kThreads) {
                    const int sl = e / (TW * CH), rem = e % (TW * CH), row = rem / CH, c = rem % CH;
                    const long kk = KH * h + 8 * c;
                    const bool vw = r0 + row < m, vl = j0 + row < m;
                    const long rw = vw ? r0 + row : 0, rl = vl ? j0 + row : 0;
                    cp_async16_zfill(&sm.Ws[b][sl][row][8 * c], a.wsl + ((long)sl * mrow + rw) * PW + kk, vw);
                    cp_async16_zfill(&sm.Ls[b][sl][row][8 * c], a.lsl + ((long)sl * mrow + rl) * PW + kk, vl);
                }
                cp_async_commit_f();
            };
            float acc[NA][4][4];  // [diagonal 0, 1, 2, the rest][n-tile][fragment]
            long r0 = 0, j0 = 0;
            fetch(0);
            for (long st = 0; st < nst; ++st) {
                const int b = (int)(st & 1);
                if (st + 1 < nst) fetch(st + 1);
                if ((st & 1) == 0) {
                    coords(first + (st / 2) * stride, r0, j0);
#pragma unroll
                    for (int c = 0; c < NA; ++c)
#pragma unroll
                        for (int n = 0; n < 4; ++n)
#pragma unroll
                            for (int i = 0; i < 4; ++i) acc[c][n][i] = 0.0f;
                }
                if (st + 1 < nst) cp_async_wait_f<1>();
                else cp_async_wait_f<0>();
                __syncthreads();
#pragma unroll 1
                for (int ks = 0; ks < KH; ks += 16) {
                    // the warp's 16 rows: all slices' A fragments; then per
                    // column block and L slice one B fragment
                    unsigned af[NS][4];
#pragma unroll
                    for (int sa = 0; sa < NS; ++sa) {
                        const __nv_bfloat16 *ap = &sm.Ws[b][sa][16 * wr + g][ks + 2 * q];
                        af[sa][0] = *reinterpret_cast<const unsigned *>(ap);
                        af[sa][1] = *reinterpret_cast<const unsigned *>(ap + 8 * SST);
                        af[sa][2] = *reinterpret_cast<const unsigned *>(ap + 8);
                        af[sa][3] = *reinterpret_cast<const unsigned *>(ap + 8 * SST + 8);
                    }
                    // consecutive products go to the four column blocks' independent
                    // accumulators (the shared one of diagonals 3 .. 5 takes 15 of the
                    // 21 products of a block)
#pragma unroll
                    for (int sb = 0; sb < NS; ++sb) {
                        unsigned bfr[4][2];
#pragma unroll
                        for (int n = 0; n < 4; ++n) {
                            const __nv_bfloat16 *bp = &sm.Ls[b][sb][32 * wc + 8 * n + g][ks + 2 * q];
                            bfr[n][0] = *reinterpret_cast<const unsigned *>(bp);
                            bfr[n][1] = *reinterpret_cast<const unsigned *>(bp + 8);
                        }
#pragma unroll
                        for (int sa = 0; sa < NS - sb; ++sa)
#pragma unroll
                            for (int n = 0; n < 4; ++n) mma16816(acc[sa + sb < NA ? sa + sb : NA - 1][n], af[sa], bfr[n]);
                    }
                }
                __syncthreads();  // the buffer is refilled by the stage after next
                if (st & 1) {
                    // rows r0 + 16 wr + g (+8), columns j0 + 32 wc + 8 n + 2 q (+1):
                    // the exponents and the band values first (one round trip),
                    // then the updates
                    const long rb = r0 + 16 * wr + g, cb = j0 + 32 * wc + 2 * q;
                    int er[2], ec[8];
#pragma unroll
                    for (int h = 0; h < 2; ++h) er[h] = rb + 8 * h < m ? a.ew[rb + 8 * h] : 0;
#pragma unroll
                    for (int n = 0; n < 4; ++n)
#pragma unroll
                        for (int h = 0; h < 2; ++h) ec[2 * n + h] = cb + 8 * n + h < m ? a.el[cb + 8 * n + h] : 0;
#pragma unroll
                    for (int n0 = 0; n0 < 4; n0 += 2) {  // two column blocks per round trip
                        dw old[2][4];
#pragma unroll
                        for (int n = 0; n < 2; ++n)
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const long rr = rb + 8 * (i >> 1), jj = cb + 8 * (n0 + n) + (i & 1);
                                old[n][i] = (rr < m && jj <= rr) ? a.band[(p + PW + jj) * ld + (rr - jj)] : dw_zero();
                            }
#pragma unroll
                        for (int n = 0; n < 2; ++n)
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const long rr = rb + 8 * (i >> 1), jj = cb + 8 * (n0 + n) + (i & 1);
                                if (rr < m && jj <= rr) {
                                    dw v = dw{acc[NA - 1][n0 + n][i], 0.0f};
#pragma unroll
                                    for (int c = NA - 2; c >= 0; --c) v = dw_add(v, dw{acc[c][n0 + n][i], 0.0f});
                                    const int sc = er[i >> 1] + ec[2 * (n0 + n) + (i & 1)];
                                    v.hi = ldexpf(v.hi, sc);
                                    v.lo = ldexpf(v.lo, sc);
                                    a.band[(p + PW + jj) * ld + (rr - jj)] = dw_sub(old[n][i], v);
                                }
                            }
                    }
                }
            }
            __syncthreads();  // the tiles' band values are written before the caller reads them
        };
        if (blockIdx.x == 0) {
            tiles(0, 1, ntiles > 0 ? 1 : 0);
            if (p + PW < a.npad) {
                const long pn = p + PW;
                load_block(a, pn, A);
                ldlt_block_dw(A, di);
                record_block(a, pn, A, di);
                for (int e = tid; e < PW * PW; e += kThreads) a.look[e] = A[e / PW][e % PW];
                if (tid < PW) a.look[PW * PW + tid] = di[tid];
            }
            if (G == 1) tiles(1, 1, ntiles);
        } else {
            tiles(blockIdx.x, G - 1, ntiles);
        }
        if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
    }
}

// Lower tile (I, J), J <= I, of a block inverse: index I (I + 1) / 2 + J.
__host__ __device__ constexpr int tile_index(int I, int J) { return I * (I + 1) / 2 + J; }

// X_i = inverse of the unit-lower diagonal block i (rows and columns
// 128 i .. 128 i + 127) of the factored band, one CTA per block, by 32 x 32
// tiles: X_II = T_I (the inverse of tile L_II, by forward elimination on the
// identity), X_IJ = -T_I sum_{K=J}^{I-1} L_IK X_KJ. Tile (I, J) is written
// row-major to xr and column-major to xc (kTiles * 1024 pairs per block).
__global__ void __launch_bounds__(kThreads) inv_block_kernel(const dw *band, long ld, long bw, dw *xr, dw *xc)
{
    __shared__ dw T[NB][NB + 1];  // T_I
    __shared__ dw L[NB][NB + 1];  // a tile L_IK
    __shared__ dw X[NB][NB + 1];  // a tile X_KJ, then the tile sum S
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const long p0 = (long)blockIdx.x * SB;
    dw *Xr = xr + (long)blockIdx.x * kTiles * NB * NB, *Xc = xc + (long)blockIdx.x * kTiles * NB * NB;
    auto lval = [&](long r, long c) -> dw {  // L(p0 + r, p0 + c), r > c; 0 outside the band
        const long off = r - c;
        return off <= bw ? band[(p0 + c) * ld + off] : dw_zero();
    };
    auto store = [&](int I, int J, const dw v[2][2]) {
        dw *tr = Xr + tile_index(I, J) * NB * NB, *tc = Xc + tile_index(I, J) * NB * NB;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int r = tx + 16 * i, c = ty + 16 * j;
                tr[r * NB + c] = v[i][j];
                tc[c * NB + r] = v[i][j];
            }
    };
    for (int I = 0; I < SB / NB; ++I) {
        // T = L_II^-1: row k of T is final after step k
        for (int e = tid; e < NB * NB; e += kThreads) {
            const int i = e / NB, j = e % NB;
            T[i][j] = i == j ? dw{1.0f, 0.0f} : dw_zero();
            L[i][j] = i > j ? lval(NB * I + i, NB * I + j) : dw_zero();
        }
        __syncthreads();
        for (int k = 0; k < NB - 1; ++k) {
            for (int e = tid; e < NB * NB; e += kThreads) {
                const int j = e / NB, i = e % NB;
                if (i > k && j <= k) T[i][j] = dw_sub(T[i][j], dw_mul(L[i][k], T[k][j]));
            }
            __syncthreads();
        }
        {
            dw v[2][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) v[i][j] = T[tx + 16 * i][ty + 16 * j];
            store(I, I, v);
        }
        for (int J = 0; J < I; ++J) {
            dw_acc acc[2][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) acc_zero(acc[i][j]);
            for (int K = J; K < I; ++K) {
                __syncthreads();
                const dw *xk = Xr + tile_index(K, J) * NB * NB;
                for (int e = tid; e < NB * NB; e += kThreads) {
                    const int i = e / NB, j = e % NB;
                    L[i][j] = lval(NB * I + i, NB * K + j);
                    X[i][j] = xk[e];
                }
                __syncthreads();
#pragma unroll 4
                for (int k = 0; k < NB; ++k) {
                    const dw l0 = L[tx][k], l1 = L[tx + 16][k], x0 = X[k][ty], x1 = X[k][ty + 16];
                    acc_fma(acc[0][0], l0, x0);
                    acc_fma(acc[0][1], l0, x1);
                    acc_fma(acc[1][0], l1, x0);
                    acc_fma(acc[1][1], l1, x1);
                }
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) X[tx + 16 * i][ty + 16 * j] = acc_value(acc[i][j]);
            __syncthreads();
            dw v[2][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    dw_acc s;
                    acc_zero(s);
                    const int r = tx + 16 * i, c = ty + 16 * j;
                    for (int k = 0; k <= r; ++k) acc_fma(s, T[r][k], X[k][c]);
                    v[i][j] = dw_neg(acc_value(s));
                }
            store(I, J, v);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

struct DwSolveArgs {
    const dw *band, *dinv, *xr, *xc;
    long ld, bw, npad, n;
    const double *rhs;
    double *out;
    dw *t, *y;  // npad each: the right-hand side being reduced, the solution
    GridBarrier *bar;
    long long max_polls;
};

constexpr int kCols = SB / 8;  // columns (rows) of the block per warp in a step's update
constexpr int kBlockElems = kTiles * NB * NB;
// dynamic shared memory of the solve: two block inverses
constexpr size_t kSolveSmem = 2 * sizeof(dw) * kBlockElems;

// CTA b of the solve applies a block's solution to rows (columns) 32 b ..
// 32 b + 31 of the block's reach: thread (lane, warp) sums the 16 products
// of its row (column) with warp's 16 entries of the block.
__global__ void __launch_bounds__(kThreads, 1) solve_dw_kernel(DwSolveArgs a)
{
    extern __shared__ __align__(16) unsigned char dyn[];
    dw *xs = (dw *)dyn;                // [2][kBlockElems]
    __shared__ dw ts[SB], ys[SB];      // the block's right-hand side and solution
    __shared__ dw part[2][SB];         // halves of the block product
    __shared__ dw red[8][NB + 1];      // per-warp partial sums of the update
    unsigned ep = 0;
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    const long ld = a.ld, bw = a.bw, npad = a.npad;
    const long gthr = blockIdx.x * (long)kThreads + tid, nthr = gridDim.x * (long)kThreads;
    const unsigned G = gridDim.x;
    const long nb = npad / SB;
    const bool active = NB * (long)blockIdx.x < bw;  // this CTA's rows (columns) are in a block's reach
    auto fetch_inv = [&](const dw *src, long blk, int buf) {
        const char *g = (const char *)(src + blk * kBlockElems);
        char *sm = (char *)(xs + buf * kBlockElems);
        for (int e = tid; e < kBlockElems * (int)sizeof(dw) / 16; e += kThreads) cp_async16(sm + 16 * e, g + 16 * e);
        cp_async_commit();
    };
    dw v[kCols];  // this thread's band values for a step
    // forward: row r = p + 128 + 32 b + lane takes L(r, p + 16 warp + k), k < 16
    auto load_row = [&](long p) {
        const long r = p + SB + NB * (long)blockIdx.x + lane;
#pragma unroll
        for (int k = 0; k < kCols; ++k) {
            const long col = p + kCols * warp + k, off = r - col;
            v[k] = (active && r < npad && off <= bw) ? a.band[col * ld + off] : dw_zero();
        }
    };
    // backward: column c = p - 32 (b + 1) + lane takes L(p + 16 warp + i, c), i < 16
    auto load_col = [&](long p) {
        const long c = p - NB * ((long)blockIdx.x + 1) + lane;
#pragma unroll
        for (int i = 0; i < kCols; ++i) {
            const long off = p + kCols * warp + i - c;
            v[i] = (active && c >= 0 && off <= bw) ? a.band[c * ld + off] : dw_zero();
        }
    };
    // the products of this thread, summed over the warps into row (column) g
    auto apply = [&](long g, bool valid) {
        dw_acc acc;
        acc_zero(acc);
#pragma unroll
        for (int k = 0; k < kCols; ++k) acc_fma(acc, v[k], ys[kCols * warp + k]);
        red[warp][lane] = acc_value(acc);
        __syncthreads();
        if (warp == 0 && valid) {
            dw s = red[0][lane];
            for (int w = 1; w < 8; ++w) s = dw_add(s, red[w][lane]);
            a.t[g] = dw_sub(a.t[g], s);
        }
    };
    const int h = tid / SB, r = tid % SB;  // half of the block product, row (column) of the block
    for (long g = gthr; g < npad; g += nthr) a.t[g] = g < a.n ? dw_from_double(a.rhs[g]) : dw_zero();
    fetch_inv(a.xc, 0, 0);
    load_row(0);
    if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
    for (long i = 0; i < nb; ++i) {
        const long p = i * SB;
        const int buf = (int)(i & 1);
        if (tid < SB) ts[tid] = a.t[p + tid];
        cp_async_wait_all();
        __syncthreads();
        // y_i = X_i t_i: thread (h, r) sums k in [64 h, 64 h + 64), k <= r
        {
            const dw *xb = xs + buf * kBlockElems;
            dw_acc acc;
            acc_zero(acc);
            const int I = r / NB, rr = r % NB;
            for (int J = 2 * h; J < 2 * h + 2 && J <= I; ++J) {
                const dw *tile = xb + tile_index(I, J) * NB * NB + rr;  // column-major: (rr, kk) at kk * 32 + rr
                const int kend = J < I ? NB : rr + 1;
                for (int kk = 0; kk < kend; ++kk) acc_fma(acc, tile[kk * NB], ts[NB * J + kk]);
            }
            part[h][r] = acc_value(acc);
        }
        __syncthreads();
        if (tid < SB) {
            const dw yv = dw_add(part[0][tid], part[1][tid]);
            ys[tid] = yv;
            if (blockIdx.x == 0) a.y[p + tid] = yv;
        }
        __syncthreads();
        if (i + 1 < nb) fetch_inv(a.xc, i + 1, buf ^ 1);
        const long row = p + SB + NB * (long)blockIdx.x + lane;
        apply(row, active && row < npad);
        if (i + 1 < nb) load_row(p + SB);
        if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
    }
    // z = D^-1 y into t (the backward right-hand side)
    for (long g = gthr; g < npad; g += nthr) a.t[g] = dw_mul(a.y[g], a.dinv[g]);
    fetch_inv(a.xr, nb - 1, (int)((nb - 1) & 1));
    load_col(npad - SB);
    if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
    for (long i = nb - 1; i >= 0; --i) {
        const long p = i * SB;
        const int buf = (int)(i & 1);
        if (tid < SB) ts[tid] = a.t[p + tid];
        cp_async_wait_all();
        __syncthreads();
        // x_i = X_i^T u_i: thread (h, c = r) sums rows k in [64 h, 64 h + 64), k >= c
        {
            const dw *xb = xs + buf * kBlockElems;
            dw_acc acc;
            acc_zero(acc);
            const int J = r / NB, cc = r % NB;
            for (int I = 2 * h; I < 2 * h + 2; ++I) {
                if (I < J) continue;
                const dw *tile = xb + tile_index(I, J) * NB * NB + cc;  // row-major: (kk, cc) at kk * 32 + cc
                const int kbeg = I > J ? 0 : cc;
                for (int kk = kbeg; kk < NB; ++kk) acc_fma(acc, tile[kk * NB], ts[NB * I + kk]);
            }
            part[h][r] = acc_value(acc);
        }
        __syncthreads();
        if (tid < SB) {
            const dw xv = dw_add(part[0][tid], part[1][tid]);
            ys[tid] = xv;
            if (blockIdx.x == 0) a.y[p + tid] = xv;
        }
        __syncthreads();
        if (i > 0) fetch_inv(a.xr, i - 1, buf ^ 1);
        const long c = p - NB * ((long)blockIdx.x + 1) + lane;
        apply(c, active && c >= 0);
        if (i > 0) load_col(p - SB);
        if (!grid_barrier(a.bar, G, ep, a.max_polls)) return;
    }
    for (long g = gthr; g < a.n; g += nthr) a.out[g] = dw_to_double(a.y[g]);
}

// band[dst[i]] = the FP64 sum of slot i's contributions, split into a pair
__global__ void gather_band_dw_kernel(const int *__restrict__ ptr, const int *__restrict__ src,
                                      const int64_t *__restrict__ dst, const double *__restrict__ in,
                                      dw *__restrict__ band, long n)
{
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += in[src[k]];
    band[dst[i]] = dw_from_double(s);
}

__global__ void pad_identity_dw_kernel(dw *band, long ld, long n, long npad)
{
    const long g = n + blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (g < npad) band[g * ld] = dw{1.0f, 0.0f};
}

template <typename K>
int coop_grid(K kernel, int per_sm_cap, size_t dyn_smem = 0)
{
    int dev = 0, sms = 0, per = 0;
    CB_CUDA_DW(cudaGetDevice(&dev));
    CB_CUDA_DW(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CB_CUDA_DW(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, dyn_smem));
    return std::max(1, sms * std::min(per, per_sm_cap));
}

}  // namespace

long band_dw_block() { return SB; }

size_t band_dw_extra_bytes(long n, long bw)
{
    const long nblk = (n + SB - 1) / SB;
    (void)bw;
    return sizeof(dw) * 2 * (size_t)nblk * kBlockElems;
}

void band_dw_alloc(BandFactor &f)
{
    const long npad = f.nblk * f.s;
    if (f.s != SB) throw std::runtime_error("the double-word band is padded to 128-row blocks");
    const size_t inv = sizeof(dw) * (size_t)(npad / SB) * kBlockElems;
    CB_CUDA_DW(cudaMalloc(&f.linv, inv));
    CB_CUDA_DW(cudaMalloc(&f.linvt, inv));
    // the factor's W/L buffer (2 * 64 * bw) and look-ahead block (64 x 64 + 64)
    const size_t wl = std::max((size_t)3 * npad, (size_t)2 * PW * (f.bw + 1) + PW);
    CB_CUDA_DW(cudaFree(f.work));
    CB_CUDA_DW(cudaMalloc(&f.work, sizeof(dw) * wl));
    CB_CUDA_DW(cudaFree(f.look));
    CB_CUDA_DW(cudaMalloc(&f.look, sizeof(dw) * (PW * PW + PW)));
    if (f.dw_simt) {
        static const bool fsmem_ok = [] {
            return cudaFuncSetAttribute(factor_dw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sizeof(DwFactorSmem)) == cudaSuccess;
        }();
        if (!fsmem_ok) throw std::runtime_error("the double-word factor needs 97 KB of shared memory per CTA");
        f.factor_grid = coop_grid(factor_dw_kernel, 1, sizeof(DwFactorSmem));
    } else {
        static const bool tsmem_ok = [] {
            return cudaFuncSetAttribute(factor_dw_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sizeof(DwTcSmem)) == cudaSuccess;
        }();
        if (!tsmem_ok) throw std::runtime_error("the tensor-core double-word factor needs 157 KB of shared memory");
        f.factor_grid = coop_grid(factor_dw_tc_kernel, 1, sizeof(DwTcSmem));
        // W and L slices of one panel ([NS][bw + 1][64] bfloat16 each) and their row exponents
        const size_t mrow = (size_t)f.bw + 1;
        CB_CUDA_DW(cudaMalloc(&f.slices, sizeof(__nv_bfloat16) * 2 * NS * mrow * PW));
        CB_CUDA_DW(cudaMemset(f.slices, 0, sizeof(__nv_bfloat16) * 2 * NS * mrow * PW));
        CB_CUDA_DW(cudaMalloc(&f.slice_exp, sizeof(int) * 2 * mrow));
        CB_CUDA_DW(cudaMemset(f.slice_exp, 0, sizeof(int) * 2 * mrow));
        f.bytes += sizeof(__nv_bfloat16) * 2 * NS * mrow * PW + sizeof(int) * 2 * mrow;
    }
    static const bool smem_ok = [] {
        return cudaFuncSetAttribute(solve_dw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSolveSmem) == cudaSuccess;
    }();
    if (!smem_ok) throw std::runtime_error("the double-word solve needs 160 KB of shared memory per CTA");
    const int sgrid = coop_grid(solve_dw_kernel, 1, kSolveSmem);
    // the solve gives each 32 rows (columns) of a block's reach a CTA of its own
    const long need = (f.bw + NB - 1) / NB;
    if (need > sgrid) throw std::runtime_error("band too wide for the double-word solve's cooperative grid");
    f.solve_grid = (int)std::max(1L, need);
    f.solve_grid_full = f.solve_grid;
    f.bytes += band_dw_extra_bytes(f.n, f.bw);
}

void band_dw_gather(const int *ptr, const int *src, const int64_t *dst, const double *kel, BandFactor &f,
                    long nslots, cudaStream_t st)
{
    if (nslots > 0)
        gather_band_dw_kernel<<<(unsigned)((nslots + 255) / 256), 256, 0, st>>>(ptr, src, dst, kel, (dw *)f.band,
                                                                               nslots);
    CB_CUDA_DW(cudaGetLastError());
}

void band_dw_factor(BandFactor &f, cudaStream_t st, long *launches)
{
    const long npad = f.nblk * f.s;
    dw *band = (dw *)f.band;
    if (npad > f.n) {
        pad_identity_dw_kernel<<<(unsigned)((npad - f.n + 127) / 128), 128, 0, st>>>(band, f.ld, f.n, npad);
        ++*launches;
    }
    CB_CUDA_DW(cudaMemsetAsync(f.flags, 0, 2 * sizeof(int), st));
    CB_CUDA_DW(cudaMemsetAsync(f.fbar, 0, sizeof(GridBarrier), st));
    const long tiles = ((f.bw + TW - 1) / TW) * ((f.bw + TW - 1) / TW + 1) / 2;
    const int grid = (int)std::max(1L, std::min<long>(f.factor_grid, std::max(tiles + 1, (f.bw + 7) / 8)));
    const long mrow = f.bw + 1;
    __nv_bfloat16 *wsl = (__nv_bfloat16 *)f.slices;
    DwFactorArgs a{band,        f.ld,    f.bw,  npad,   f.n,         (dw *)f.dinv,
                   f.ssd,       f.flags, (dw *)f.work,  (dw *)f.look, f.fbar,    f.max_polls,
                   wsl,         wsl ? wsl + (size_t)NS * mrow * PW : nullptr,
                   f.slice_exp, f.slice_exp ? f.slice_exp + mrow : nullptr, mrow};
    void *args[] = {&a};
    if (f.dw_simt)
        CB_CUDA_DW(cudaLaunchCooperativeKernel((const void *)factor_dw_kernel, dim3((unsigned)grid),
                                               dim3(kThreads), args, sizeof(DwFactorSmem), st));
    else
        CB_CUDA_DW(cudaLaunchCooperativeKernel((const void *)factor_dw_tc_kernel, dim3((unsigned)grid),
                                               dim3(kThreads), args, sizeof(DwTcSmem), st));
    inv_block_kernel<<<(unsigned)(npad / SB), kThreads, 0, st>>>(band, f.ld, f.bw, (dw *)f.linv, (dw *)f.linvt);
    CB_CUDA_DW(cudaGetLastError());
    *launches += 2;
}

void band_dw_solve(const BandFactor &f, const double *rhs, double *x, void *work, GridBarrier *bar,
                   cudaStream_t st)
{
    const long npad = f.nblk * f.s;
    DwSolveArgs a{(const dw *)f.band, (const dw *)f.dinv, (const dw *)f.linv, (const dw *)f.linvt, f.ld, f.bw,
                  npad, f.n, rhs, x, (dw *)work, (dw *)work + npad, bar, f.max_polls};
    CB_CUDA_DW(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), st));
    void *args[] = {&a};
    CB_CUDA_DW(cudaLaunchCooperativeKernel((const void *)solve_dw_kernel, dim3((unsigned)f.solve_grid),
                                           dim3(kThreads), args, kSolveSmem, st));
}

}  // namespace cb
