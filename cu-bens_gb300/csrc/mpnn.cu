// Learned preconditioner: a mesh message-passing network on the joint graph,
// trained online on the GPU by its own forward, backward and Adam kernels,
// and applied inside FGMRES (which tolerates a preconditioner that changes
// from one application to the next).
//
// Network (float32 activations, node-major [joint][feature]):
//   x_i   = [r / rms(r), p / rms(p)] at the joint's six equations, p = B^-1 r
//           (block-Jacobi), 0 for a fixed DOF                            (12)
//   h     = relu(W0 x + b0)                                              (64)
//   3 x   [P;Q] = [A;B] h ; a_i = mean_{j ~ i} relu(P_i + Q_j + c)
//         h <- h + relu(U h + V a + d)
//   y     = Wd h + bd                                                     (6)
//   z     = p + rms(p) y at the joint's equations (z = p elsewhere)
// The parameters are one flat float32 vector: W0 b0 | A B c U V d (x3) | Wd bd.
// With y = 0 the preconditioner is block-Jacobi, and P(alpha r) = alpha P(r)
// for alpha > 0.
//
// Every reduction has a fixed order (node lists in ascending order, weight
// gradients as per-chunk partials summed in chunk order), so training is
// bit-reproducible. The edge messages are recomputed in the backward pass
// from the node arrays (P, Q, c), so nothing per edge is stored.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <stdexcept>
#include <vector>

#include "internal.hpp"
#include "model.hpp"

namespace cb {

namespace {

constexpr int kH = 64, kFin = 12, kFout = 6, kLayers = 3;
constexpr long kLayerParams = 4L * kH * kH + 2 * kH;
constexpr long kOffW0 = 0, kOffB0 = kH * kFin, kOffLayer0 = kOffB0 + kH;
constexpr long kOffWd = kOffLayer0 + kLayers * kLayerParams, kOffBd = kOffWd + kFout * kH;
constexpr long kParams = kOffBd + kFout;
// within a layer: A, B (stacked [A;B] 128x64), c, U, V, d
constexpr long kA = 0, kC = 2L * kH * kH, kU = kC + kH, kV = kU + kH * kH, kD = kV + kH * kH;
constexpr int kWChunk = 128;  // nodes per weight-gradient partial

constexpr int kT = 256;
inline unsigned nb(long n, int t = kT) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- inputs: r, p = B^-1 r, rms(r), rms(p) ----

// r_i = src_i * s (s = ctl->scale when ctl is given, else 1; r written to
// rout and, with ctl, to V_j), p = B^-1 r into pout and Zout (z = p before
// the network adds to the joints' equations), partial sums of r^2, p^2.
template <typename T>
__global__ void mp_prep_kernel(const KrylovCtl *__restrict__ ctl, const double *__restrict__ src,
                               double *__restrict__ rout, double *__restrict__ V, double *__restrict__ pout,
                               double *__restrict__ Zout, const int *__restrict__ row_blk,
                               const int *__restrict__ blk_start, const int *__restrict__ blk_off,
                               const T *__restrict__ binv, const double *__restrict__ pgiven,
                               double *__restrict__ part, long n)
{
    if (ctl && ctl->done) return;
    __shared__ double red[2][kT / 32];
    const double sc = ctl ? ctl->scale : 1.0;
    const size_t off = ctl ? (size_t)ctl->j * n : 0;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double rr = 0, pp = 0;
    if (i < n) {
        const double r = src[i] * sc;
        rout[i] = r;
        if (V) V[off + i] = r;
        double p = 0;
        if (pgiven) {
            p = pgiven[i];
        } else {
            const int b = row_blk[i];
            const int s0 = blk_start[b], bs = blk_start[b + 1] - s0;
            const T *B = binv + blk_off[b] + (i - s0) * bs;
            for (int c = 0; c < bs; ++c) p += (double)B[c] * (src[s0 + c] * sc);
        }
        pout[i] = p;
        Zout[off + i] = p;
        rr = r * r;
        pp = p * p;
    }
    rr = warp_sum_d(rr);
    pp = warp_sum_d(pp);
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = rr;
        red[1][threadIdx.x >> 5] = pp;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < kT / 32; ++w) {
            a += red[0][w];
            b += red[1][w];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// scal[0] = rms(r), scal[1] = rms(p) from the prep partials (one warp)
__global__ void mp_rms_kernel(const KrylovCtl *__restrict__ ctl, const double *__restrict__ part, int nparts,
                              double *__restrict__ scal, long n)
{
    if (ctl && ctl->done) return;
    double a = 0, b = 0;
    for (int k = threadIdx.x; k < nparts; k += 32) {
        a += part[2 * k];
        b += part[2 * k + 1];
    }
    a = warp_sum_d(a);
    b = warp_sum_d(b);
    if (threadIdx.x == 0) {
        scal[0] = sqrt(a / (double)n);
        scal[1] = sqrt(b / (double)n);
    }
}

__global__ void mp_features_kernel(const KrylovCtl *__restrict__ ctl, const int *__restrict__ node_eq,
                                   const double *__restrict__ r, const double *__restrict__ p,
                                   const double *__restrict__ scal, float *__restrict__ x, long nj)
{
    if (ctl && ctl->done) return;
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= nj * 6) return;
    const long i = t / 6;
    const int k = (int)(t % 6);
    const int q = node_eq[i * 6 + k];
    const double sr = scal[0], sp = scal[1];
    x[i * kFin + k] = (q >= 0 && sr > 0) ? (float)(r[q] / sr) : 0.f;
    x[i * kFin + 6 + k] = (q >= 0 && sp > 0) ? (float)(p[q] / sp) : 0.f;
}

// ---- dense layer: Y = act(sum_t X_t W_t^T + bias) + res (or Y += that) ----

struct DenseIn {
    const float *X;  // [n][K]
    int K;
    const float *W;  // W(o, k) = trans ? W[k*O + o] : W[o*K + k]
    int trans;
};

struct DenseArgs {
    DenseIn in[2];
    int nin;
    const float *bias;  // O entries or null
    const float *res;   // [n][O] added after the activation, or null
    float *Y;           // [n][O]
    float *Yres;        // with res: Y = act(...), Yres = Y + res (else Y = act(...) + res)
    int O;
    int relu;
    int accum;
    long n;
    const KrylovCtl *ctl;
};

// The dense products run on the tensor cores: BF16 operands (the float32
// activations and weights rounded to nearest), FP32 accumulation, with
// mma.sync.m16n8k16 (row-major A, column-major B).
__device__ __forceinline__ void mma_bf16(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned ld_pair(const __nv_bfloat16 *p) { return *(const unsigned *)p; }

constexpr int kTcNodes = 64;    // nodes per CTA of the dense kernel: 4 warps x 16 rows
constexpr int kTcThreads = 128;

// Y = act(sum_t X_t W_t^T + bias) (+ res) for 64 nodes per CTA: X and W in
// shared memory as BF16 (K padded to a multiple of 16, O to NT * 8), warp w
// computes rows 16 w .. 16 w + 15 and all NT column tiles.
template <int NT>
__global__ void __launch_bounds__(kTcThreads) mp_dense_tc_kernel(DenseArgs a, int Kp)
{
    if (a.ctl && a.ctl->done) return;
    extern __shared__ __align__(16) unsigned char dsm[];
    const int ldx = Kp + 8;  // row stride (bf16): 16-byte rows, conflict-free fragment loads
    __nv_bfloat16 *Xs = (__nv_bfloat16 *)dsm;           // [64][ldx]
    __nv_bfloat16 *Ws = Xs + kTcNodes * ldx;            // [NT*8][ldx]
    const int O = a.O, tid = threadIdx.x;
    const long n0 = blockIdx.x * (long)kTcNodes;
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
    int kb = 0;
    for (int t = 0; t < a.nin; ++t) {
        const DenseIn &in = a.in[t];
        for (int e = tid; e < kTcNodes * in.K; e += kTcThreads) {
            const int r = e / in.K, k = e % in.K;
            const long node = n0 + r;
            Xs[r * ldx + kb + k] = __float2bfloat16_rn(node < a.n ? in.X[node * in.K + k] : 0.f);
        }
        for (int e = tid; e < O * in.K; e += kTcThreads) {
            const int o = e / in.K, k = e % in.K;
            Ws[o * ldx + kb + k] = __float2bfloat16_rn(in.trans ? in.W[(size_t)k * O + o] : in.W[(size_t)o * in.K + k]);
        }
        kb += in.K;
    }
    for (int e = tid; e < kTcNodes * (Kp - kb); e += kTcThreads) Xs[(e / (Kp - kb)) * ldx + kb + e % (Kp - kb)] = zero;
    for (int e = tid; e < NT * 8 * Kp; e += kTcThreads) {
        const int o = e / Kp, k = e % Kp;
        if (o >= O || k >= kb) Ws[o * ldx + k] = zero;
    }
    __syncthreads();
    const int warp = tid / 32, lane = tid % 32, g = lane >> 2, q = lane & 3;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const __nv_bfloat16 *xr0 = Xs + (16 * warp + g) * ldx, *xr1 = xr0 + 8 * ldx;
    for (int k0 = 0; k0 < Kp; k0 += 16) {
        const unsigned a0 = ld_pair(xr0 + k0 + 2 * q), a1 = ld_pair(xr1 + k0 + 2 * q);
        const unsigned a2 = ld_pair(xr0 + k0 + 8 + 2 * q), a3 = ld_pair(xr1 + k0 + 8 + 2 * q);
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const __nv_bfloat16 *wr = Ws + (8 * j + g) * ldx + k0 + 2 * q;
            mma_bf16(acc[j], a0, a1, a2, a3, ld_pair(wr), ld_pair(wr + 8));
        }
    }
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const long node = n0 + 16 * warp + g + (e >= 2 ? 8 : 0);
            const int o = 8 * j + 2 * q + (e & 1);
            if (node >= a.n || o >= O) continue;
            float v = acc[j][e] + (a.bias ? a.bias[o] : 0.f);
            if (a.relu) v = fmaxf(v, 0.f);
            if (a.Yres) {
                a.Y[node * O + o] = v;
                a.Yres[node * O + o] = v + a.res[node * O + o];
                continue;
            }
            if (a.res) v += a.res[node * O + o];
            float *y = a.Y + node * O + o;
            *y = a.accum ? *y + v : v;
        }
}

size_t dense_smem(int Kp, int NT) { return sizeof(__nv_bfloat16) * (size_t)(kTcNodes + NT * 8) * (Kp + 8); }

void dense(const DenseArgs &a, cudaStream_t st)
{
    int Ktot = 0;
    for (int t = 0; t < a.nin; ++t) Ktot += a.in[t].K;
    const int Kp = (Ktot + 15) / 16 * 16;
    const unsigned grid = (unsigned)((a.n + kTcNodes - 1) / kTcNodes);
    if (a.O <= 64)
        mp_dense_tc_kernel<8><<<grid, kTcThreads, dense_smem(Kp, 8), st>>>(a, Kp);
    else
        mp_dense_tc_kernel<16><<<grid, kTcThreads, dense_smem(Kp, 16), st>>>(a, Kp);
}

// ---- edge aggregation: a_i = mean_j relu(P_i + Q_j + c) ----

__global__ void mp_edge_kernel(const KrylovCtl *__restrict__ ctl, const int *__restrict__ adj_ptr,
                               const int *__restrict__ adj, const float *__restrict__ PQ,
                               const float *__restrict__ c, float *__restrict__ out, long nj)
{
    if (ctl && ctl->done) return;
    const long i = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nj) return;
    const int e0 = adj_ptr[i], e1 = adj_ptr[i + 1];
    const float P0 = PQ[i * 128 + lane] + c[lane], P1 = PQ[i * 128 + 32 + lane] + c[32 + lane];
    float s0 = 0, s1 = 0;
    for (int e = e0; e < e1; ++e) {
        const int j = adj[e];
        s0 += fmaxf(P0 + PQ[(long)j * 128 + 64 + lane], 0.f);
        s1 += fmaxf(P1 + PQ[(long)j * 128 + 96 + lane], 0.f);
    }
    const float inv = e1 > e0 ? 1.f / (float)(e1 - e0) : 0.f;
    out[i * kH + lane] = s0 * inv;
    out[i * kH + 32 + lane] = s1 * inv;
}

// dP_i = da_i / deg_i * sum_j [P_i + Q_j + c > 0];
// dQ_i = sum_{j ~ i} da_j / deg_j * [P_j + Q_i + c > 0]
__global__ void mp_edge_bwd_kernel(const int *__restrict__ adj_ptr, const int *__restrict__ adj,
                                   const float *__restrict__ PQ, const float *__restrict__ c,
                                   const float *__restrict__ da, float *__restrict__ dPQ, long nj)
{
    const long i = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nj) return;
    const int e0 = adj_ptr[i], e1 = adj_ptr[i + 1];
    for (int h = 0; h < 2; ++h) {
        const int f = lane + 32 * h;
        const float Pi = PQ[i * 128 + f] + c[f], Qi = PQ[i * 128 + 64 + f];
        const float gi = e1 > e0 ? da[i * kH + f] / (float)(e1 - e0) : 0.f;
        float cnt = 0, dq = 0;
        for (int e = e0; e < e1; ++e) {
            const long j = adj[e];
            cnt += (Pi + PQ[j * 128 + 64 + f] > 0.f) ? 1.f : 0.f;
            const int dj = adj_ptr[j + 1] - adj_ptr[j];
            if (PQ[j * 128 + f] + c[f] + Qi > 0.f) dq += da[j * kH + f] / (float)dj;
        }
        dPQ[i * 128 + f] = gi * cnt;
        dPQ[i * 128 + 64 + f] = dq;
    }
}

// ---- decoder: z[eq] = p[eq] + rms(p) * (Wd h + bd) at the joints' equations ----

__global__ void mp_decode_kernel(const KrylovCtl *__restrict__ ctl, const int *__restrict__ node_eq,
                                 const float *__restrict__ h, const float *__restrict__ Wd,
                                 const float *__restrict__ bd, const double *__restrict__ p,
                                 const double *__restrict__ scal, double *__restrict__ Zout, long nj, long n)
{
    if (ctl && ctl->done) return;
    __shared__ float w[kFout * kH + kFout];
    for (int e = threadIdx.x; e < kFout * kH + kFout; e += blockDim.x)
        w[e] = e < kFout * kH ? Wd[e] : bd[e - kFout * kH];
    __syncthreads();
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= nj * kFout) return;
    const long i = t / kFout;
    const int k = (int)(t % kFout);
    const int q = node_eq[i * 6 + k];
    if (q < 0) return;
    float acc = w[kFout * kH + k];
    for (int f = 0; f < kH; ++f) acc = fmaf(w[k * kH + f], h[i * kH + f], acc);
    const size_t off = ctl ? (size_t)ctl->j * n : 0;
    Zout[off + q] = p[q] + scal[1] * (double)acc;
}

// ---- loss and its gradient at the output ----

// partial sums of |t|^2 and |z - t|^2 (block partials; scal[2], scal[3] by mp_loss_kernel)
__global__ void mp_loss_parts_kernel(const double *__restrict__ z, const double *__restrict__ t,
                                     double *__restrict__ part, long n)
{
    __shared__ double red[2][kT / 32];
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double tt = 0, ee = 0;
    if (i < n) {
        tt = t[i] * t[i];
        const double e = z[i] - t[i];
        ee = e * e;
    }
    tt = warp_sum_d(tt);
    ee = warp_sum_d(ee);
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = tt;
        red[1][threadIdx.x >> 5] = ee;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < kT / 32; ++w) {
            a += red[0][w];
            b += red[1][w];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

__global__ void mp_loss_kernel(const double *__restrict__ part, int nparts, double *__restrict__ scal)
{
    double a = 0, b = 0;
    for (int k = threadIdx.x; k < nparts; k += 32) {
        a += part[2 * k];
        b += part[2 * k + 1];
    }
    a = warp_sum_d(a);
    b = warp_sum_d(b);
    if (threadIdx.x == 0) {
        scal[2] = a;
        scal[3] = a > 0 ? b / a : 0.0;
    }
}

// dy[i][k] = rms(p) * 2 (z - t)[eq] / |t|^2
__global__ void mp_dy_kernel(const int *__restrict__ node_eq, const double *__restrict__ z,
                             const double *__restrict__ t, const double *__restrict__ scal, float *__restrict__ dy,
                             long nj)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= nj * kFout) return;
    const long i = e / kFout;
    const int k = (int)(e % kFout);
    const int q = node_eq[i * 6 + k];
    const double tt = scal[2];
    dy[i * kFout + k] = (q >= 0 && tt > 0) ? (float)(scal[1] * 2.0 * (z[q] - t[q]) / tt) : 0.f;
}

// dT = dh * [R > 0]
__global__ void mp_mask_kernel(const float *__restrict__ dh, const float *__restrict__ R, float *__restrict__ out,
                               long n)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e < n) out[e] = R[e] > 0.f ? dh[e] : 0.f;
}

// ---- weight gradients: dW[o][k] = sum_n dZ[n][o] X[n][k], db[o] = sum_n dZ[n][o] ----

// per chunk of kWChunk nodes: part[blk][o*(K+1) + k] (k == K: the bias sum),
// on the tensor cores: A = dZ^T (O x nodes), B = [X 1] (nodes x (K+1)), both
// as BF16 in shared memory, FP32 accumulation over the chunk's 128 nodes.
// Warp w takes row tiles w, w + 4, ... (RT of them) and all NT column tiles.
template <int RT, int NT>
__global__ void __launch_bounds__(kTcThreads) mp_wgrad_tc_kernel(const float *__restrict__ dZ, int O,
                                                                 const float *__restrict__ X, int K,
                                                                 float *__restrict__ part, long n)
{
    constexpr int kSub = 64;          // nodes staged at a time
    constexpr int kld = kSub + 8;     // row stride (bf16) over those nodes
    __shared__ __align__(16) __nv_bfloat16 As[4 * RT * 16][kld];  // [o][node]
    __shared__ __align__(16) __nv_bfloat16 Bs[NT * 8][kld];       // [k][node]
    const int tid = threadIdx.x;
    const long c0 = blockIdx.x * (long)kWChunk;
    const int KK = K + 1, tot = O * KK;
    const int warp = tid / 32, lane = tid % 32, g = lane >> 2, q = lane & 3;
    float acc[RT][NT][4];
#pragma unroll
    for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
    for (int s0 = 0; s0 < kWChunk; s0 += kSub) {
        for (int e = tid; e < 4 * RT * 16 * kSub; e += kTcThreads) {
            const int o = e / kSub, r = e % kSub;
            const long node = c0 + s0 + r;
            As[o][r] = __float2bfloat16_rn((o < O && node < n) ? dZ[node * O + o] : 0.f);
        }
        for (int e = tid; e < NT * 8 * kSub; e += kTcThreads) {
            const int k = e / kSub, r = e % kSub;
            const long node = c0 + s0 + r;
            const float v = node < n ? (k < K ? X[node * K + k] : (k == K ? 1.f : 0.f)) : 0.f;
            Bs[k][r] = __float2bfloat16_rn(v);
        }
        __syncthreads();
        for (int k0 = 0; k0 < kSub; k0 += 16) {
#pragma unroll
            for (int i = 0; i < RT; ++i) {
                const int row = 16 * (warp + 4 * i) + g;
                const unsigned a0 = ld_pair(&As[row][k0 + 2 * q]), a1 = ld_pair(&As[row + 8][k0 + 2 * q]);
                const unsigned a2 = ld_pair(&As[row][k0 + 8 + 2 * q]), a3 = ld_pair(&As[row + 8][k0 + 8 + 2 * q]);
#pragma unroll
                for (int j = 0; j < NT; ++j)
                    mma_bf16(acc[i][j], a0, a1, a2, a3, ld_pair(&Bs[8 * j + g][k0 + 2 * q]),
                             ld_pair(&Bs[8 * j + g][k0 + 8 + 2 * q]));
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int o = 16 * (warp + 4 * i) + g + (e >= 2 ? 8 : 0);
                const int k = 8 * j + 2 * q + (e & 1);
                if (o < O && k < KK) part[(size_t)blockIdx.x * tot + o * KK + k] = acc[i][j][e];
            }
}

// grad += sum over chunks (in chunk order); bias sums for the first nbias outputs
__global__ void mp_wgrad_reduce_kernel(const float *__restrict__ part, int nparts, int O, int K,
                                       float *__restrict__ gW, float *__restrict__ gb, int nbias)
{
    const int KK = K + 1, tot = O * KK;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= tot) return;
    float s = 0;
    for (int b = 0; b < nparts; ++b) s += part[(size_t)b * tot + idx];
    const int o = idx / KK, k = idx % KK;
    if (k < K) gW[o * K + k] += s;
    else if (gb && o < nbias) gb[o] += s;
}

__global__ void mp_adam_kernel(float *__restrict__ th, const float *__restrict__ g, float *__restrict__ m1,
                               float *__restrict__ m2, long n, float lr, float b1, float b2, float eps, float c1,
                               float c2)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float m = b1 * m1[i] + (1.f - b1) * gi;
    const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = m;
    m2[i] = v;
    th[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

}  // namespace

// ---------------------------------------------------------------------------

struct Mpnn {
    long nj = 0, neq = 0, nedge = 0;
    int *node_eq = nullptr, *adj_ptr = nullptr, *adj = nullptr;
    float *theta = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    float *x = nullptr, *h[kLayers + 1] = {}, *PQ[kLayers] = {}, *a[kLayers] = {}, *R[kLayers] = {};
    float *dh = nullptr, *dh2 = nullptr, *dT = nullptr, *da = nullptr, *dPQ = nullptr, *dy = nullptr;
    float *wpart = nullptr;
    double *rbuf = nullptr, *pbuf = nullptr, *zbuf = nullptr, *scal = nullptr, *part = nullptr;
    double *pair_b = nullptr, *pair_t = nullptr;
    int cap = 0, count = 0, next = 0;
    long adam_t = 0;
    float lr = 1e-3f;
    double last_loss = 0;
    size_t bytes = 0;
    std::vector<void *> allocs;
    template <typename T>
    T *alloc(size_t n, cudaStream_t st)
    {
        void *p = nullptr;
        const size_t b = std::max<size_t>(n, 1) * sizeof(T);
        CB_CUDA(cudaMalloc(&p, b));
        CB_CUDA(cudaMemsetAsync(p, 0, b, st));
        allocs.push_back(p);
        bytes += b;
        return (T *)p;
    }
};

long mpnn_param_count() { return kParams; }

namespace {

// Joint graph: equations of each joint's six DOFs and the joints that share
// an element with it (ascending, no repeats).
void build_joint_graph(const HostModel &h, std::vector<int> &node_eq, std::vector<int> &ptr, std::vector<int> &adj)
{
    const long NJ = h.nj;
    node_eq.assign(NJ * 6, -1);
    for (long i = 0; i < NJ; ++i)
        for (int d = 0; d < 6; ++d) node_eq[i * 6 + d] = (int)h.jcode[i * 7 + d] - 1;
    std::vector<std::vector<int>> nbr(NJ);
    auto link = [&](int a, int b) {
        if (a == b) return;
        nbr[a].push_back(b);
        nbr[b].push_back(a);
    };
    for (long e = 0; e < h.ne_tr; ++e) link(h.tr_conn[2 * e], h.tr_conn[2 * e + 1]);
    for (long e = 0; e < h.ne_fr; ++e) link(h.fr_conn[2 * e], h.fr_conn[2 * e + 1]);
    for (long e = 0; e < h.ne_sh; ++e)
        for (int a = 0; a < 3; ++a) link(h.sh_conn[3 * e + a], h.sh_conn[3 * e + (a + 1) % 3]);
    ptr.assign(NJ + 1, 0);
    adj.clear();
    for (long i = 0; i < NJ; ++i) {
        std::sort(nbr[i].begin(), nbr[i].end());
        nbr[i].erase(std::unique(nbr[i].begin(), nbr[i].end()), nbr[i].end());
        adj.insert(adj.end(), nbr[i].begin(), nbr[i].end());
        ptr[i + 1] = (int)adj.size();
    }
}

// He-scaled normal weights (seeded), zero biases, a decoder 100 times
// smaller: the network starts close to block-Jacobi.
std::vector<float> init_params(unsigned seed)
{
    std::mt19937_64 gen(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    std::vector<float> th(kParams, 0.f);
    auto fill = [&](long off, int out, int in, double gain) {
        const double s = std::sqrt(2.0 / in) * gain;
        for (long k = 0; k < (long)out * in; ++k) th[off + k] = (float)(nd(gen) * s);
    };
    fill(kOffW0, kH, kFin, 1.0);
    for (int l = 0; l < kLayers; ++l) {
        const long b = kOffLayer0 + l * kLayerParams;
        fill(b + kA, 2 * kH, kH, 0.5);
        fill(b + kU, kH, kH, 0.5);
        fill(b + kV, kH, kH, 0.5);
    }
    fill(kOffWd, kFout, kH, 0.01);
    return th;
}

// r = src (* ctl->scale), p = B^-1 r (or pgiven), z = p, then rms(r), rms(p)
void prep(Mpnn &mp, const KrylovSolver &ks, const KrylovCtl *ctl, const double *src, const double *pgiven,
          double *V, double *Zout, cudaStream_t st)
{
    const unsigned g = nb(ks.n);
    if (ks.fp32_precond)
        mp_prep_kernel<float><<<g, kT, 0, st>>>(ctl, src, mp.rbuf, V, mp.pbuf, Zout, ks.row_blk, ks.blk_start,
                                                ks.blk_off, (const float *)ks.binv, pgiven, mp.part, ks.n);
    else
        mp_prep_kernel<double><<<g, kT, 0, st>>>(ctl, src, mp.rbuf, V, mp.pbuf, Zout, ks.row_blk, ks.blk_start,
                                                 ks.blk_off, (const double *)ks.binv, pgiven, mp.part, ks.n);
    mp_rms_kernel<<<1, 32, 0, st>>>(ctl, mp.part, (int)g, mp.scal, ks.n);
}

// The network's forward pass from the inputs (r, p) in rbuf/pbuf (and the
// rms values in scal) to z (Zout, at V_j's column with ctl).
void forward(Mpnn &mp, const KrylovCtl *ctl, double *Zout, cudaStream_t st)
{
    const long nj = mp.nj;
    mp_features_kernel<<<nb(nj * 6), kT, 0, st>>>(ctl, mp.node_eq, mp.rbuf, mp.pbuf, mp.scal, mp.x, nj);
    {
        DenseArgs d{};
        d.in[0] = DenseIn{mp.x, kFin, mp.theta + kOffW0, 0};
        d.nin = 1;
        d.bias = mp.theta + kOffB0;
        d.Y = mp.h[0];
        d.O = kH;
        d.relu = 1;
        d.n = nj;
        d.ctl = ctl;
        dense(d, st);
    }
    for (int l = 0; l < kLayers; ++l) {
        const float *L = mp.theta + kOffLayer0 + l * kLayerParams;
        DenseArgs d{};
        d.in[0] = DenseIn{mp.h[l], kH, L + kA, 0};
        d.nin = 1;
        d.Y = mp.PQ[l];
        d.O = 2 * kH;
        d.n = nj;
        d.ctl = ctl;
        dense(d, st);
        mp_edge_kernel<<<nb(nj * 32), kT, 0, st>>>(ctl, mp.adj_ptr, mp.adj, mp.PQ[l], L + kC, mp.a[l], nj);
        DenseArgs u{};
        u.in[0] = DenseIn{mp.h[l], kH, L + kU, 0};
        u.in[1] = DenseIn{mp.a[l], kH, L + kV, 0};
        u.nin = 2;
        u.bias = L + kD;
        u.res = mp.h[l];
        u.Y = mp.R[l];
        u.Yres = mp.h[l + 1];
        u.O = kH;
        u.relu = 1;
        u.n = nj;
        u.ctl = ctl;
        dense(u, st);
    }
    mp_decode_kernel<<<nb(nj * kFout), kT, 0, st>>>(ctl, mp.node_eq, mp.h[kLayers], mp.theta + kOffWd,
                                                     mp.theta + kOffBd, mp.pbuf, mp.scal, Zout, nj, mp.neq);
}

void wgrad(Mpnn &mp, const float *dZ, int O, const float *X, int K, float *gW, float *gb, int nbias,
           cudaStream_t st)
{
    const int nparts = (int)((mp.nj + kWChunk - 1) / kWChunk);
    // O <= 64: one row tile per warp; O = 128: two. K + 1 <= 72 (nine column tiles) or <= 16
    if (K + 1 <= 16) mp_wgrad_tc_kernel<1, 2><<<nparts, kTcThreads, 0, st>>>(dZ, O, X, K, mp.wpart, mp.nj);
    else if (O <= 64) mp_wgrad_tc_kernel<1, 9><<<nparts, kTcThreads, 0, st>>>(dZ, O, X, K, mp.wpart, mp.nj);
    else mp_wgrad_tc_kernel<2, 9><<<nparts, kTcThreads, 0, st>>>(dZ, O, X, K, mp.wpart, mp.nj);
    mp_wgrad_reduce_kernel<<<nb((long)O * (K + 1)), kT, 0, st>>>(mp.wpart, nparts, O, K, gW, gb, nbias);
}

void mask(const float *dh, const float *R, float *out, long n, cudaStream_t st)
{
    mp_mask_kernel<<<nb(n), kT, 0, st>>>(dh, R, out, n);
}

// Loss |z - t|^2 / |t|^2 of the forward pass in zbuf and the parameter
// gradient into mp.grad (overwritten).
void backward(Mpnn &mp, const double *t, cudaStream_t st)
{
    const long nj = mp.nj, nf = nj * kH;
    const unsigned g = nb(mp.neq);
    mp_loss_parts_kernel<<<g, kT, 0, st>>>(mp.zbuf, t, mp.part, mp.neq);
    mp_loss_kernel<<<1, 32, 0, st>>>(mp.part, (int)g, mp.scal);
    mp_dy_kernel<<<nb(nj * kFout), kT, 0, st>>>(mp.node_eq, mp.zbuf, t, mp.scal, mp.dy, nj);
    CB_CUDA(cudaMemsetAsync(mp.grad, 0, sizeof(float) * kParams, st));
    float *th = mp.theta, *gr = mp.grad;
    // decoder
    wgrad(mp, mp.dy, kFout, mp.h[kLayers], kH, gr + kOffWd, gr + kOffBd, kFout, st);
    {
        DenseArgs d{};
        d.in[0] = DenseIn{mp.dy, kFout, th + kOffWd, 1};
        d.nin = 1;
        d.Y = mp.dh;
        d.O = kH;
        d.n = nj;
        dense(d, st);
    }
    for (int l = kLayers - 1; l >= 0; --l) {
        const float *L = th + kOffLayer0 + l * kLayerParams;
        float *G = gr + kOffLayer0 + l * kLayerParams;
        mask(mp.dh, mp.R[l], mp.dT, nf, st);
        wgrad(mp, mp.dT, kH, mp.h[l], kH, G + kU, G + kD, kH, st);
        wgrad(mp, mp.dT, kH, mp.a[l], kH, G + kV, nullptr, 0, st);
        DenseArgs d{};
        d.in[0] = DenseIn{mp.dT, kH, L + kV, 1};
        d.nin = 1;
        d.Y = mp.da;
        d.O = kH;
        d.n = nj;
        dense(d, st);  // da = dT V
        DenseArgs e{};
        e.in[0] = DenseIn{mp.dT, kH, L + kU, 1};
        e.nin = 1;
        e.res = mp.dh;
        e.Y = mp.dh2;
        e.O = kH;
        e.n = nj;
        dense(e, st);  // dh_in = dh + dT U
        mp_edge_bwd_kernel<<<nb(nj * 32), kT, 0, st>>>(mp.adj_ptr, mp.adj, mp.PQ[l], L + kC, mp.da, mp.dPQ, nj);
        wgrad(mp, mp.dPQ, 2 * kH, mp.h[l], kH, G + kA, G + kC, kH, st);
        DenseArgs f{};
        f.in[0] = DenseIn{mp.dPQ, 2 * kH, L + kA, 1};
        f.nin = 1;
        f.Y = mp.dh2;
        f.O = kH;
        f.accum = 1;
        f.n = nj;
        dense(f, st);  // dh_in += dPQ [A;B]
        std::swap(mp.dh, mp.dh2);
    }
    mask(mp.dh, mp.h[0], mp.dT, nf, st);
    wgrad(mp, mp.dT, kH, mp.x, kFin, gr + kOffW0, gr + kOffB0, kH, st);
}

void adam_step(Mpnn &mp, cudaStream_t st)
{
    mp.adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)mp.adam_t), c2 = 1.f - std::pow(b2, (float)mp.adam_t);
    mp_adam_kernel<<<nb(kParams), kT, 0, st>>>(mp.theta, mp.grad, mp.m1, mp.m2, kParams, mp.lr, b1, b2, 1e-8f, c1,
                                               c2);
}

}  // namespace

// ---------------------------------------------------------------------------

Mpnn *mpnn_create(const HostModel &h, unsigned seed, int capacity, cudaStream_t st)
{
    static const bool smem_ok = [] {
        return cudaFuncSetAttribute(mp_dense_tc_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)dense_smem(128, 8)) == cudaSuccess &&
               cudaFuncSetAttribute(mp_dense_tc_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)dense_smem(128, 16)) == cudaSuccess;
    }();
    if (!smem_ok) throw std::runtime_error("the network's dense kernel needs 52 KB of shared memory per CTA");
    Mpnn *mp = new Mpnn();
    std::vector<int> node_eq, ptr, adj;
    build_joint_graph(h, node_eq, ptr, adj);
    mp->nj = h.nj;
    mp->neq = h.neq;
    mp->nedge = (long)adj.size();
    const long nj = mp->nj;
    mp->node_eq = mp->alloc<int>(node_eq.size(), st);
    mp->adj_ptr = mp->alloc<int>(ptr.size(), st);
    mp->adj = mp->alloc<int>(adj.size(), st);
    CB_CUDA(cudaMemcpyAsync(mp->node_eq, node_eq.data(), sizeof(int) * node_eq.size(), cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemcpyAsync(mp->adj_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, st));
    if (!adj.empty())
        CB_CUDA(cudaMemcpyAsync(mp->adj, adj.data(), sizeof(int) * adj.size(), cudaMemcpyHostToDevice, st));
    for (float **v : {&mp->theta, &mp->grad, &mp->m1, &mp->m2}) *v = mp->alloc<float>(kParams, st);
    const std::vector<float> th = init_params(seed);
    CB_CUDA(cudaMemcpyAsync(mp->theta, th.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice, st));
    mp->x = mp->alloc<float>(nj * kFin, st);
    for (int l = 0; l <= kLayers; ++l) mp->h[l] = mp->alloc<float>(nj * kH, st);
    for (int l = 0; l < kLayers; ++l) {
        mp->PQ[l] = mp->alloc<float>(nj * 2 * kH, st);
        mp->a[l] = mp->alloc<float>(nj * kH, st);
        mp->R[l] = mp->alloc<float>(nj * kH, st);
    }
    for (float **v : {&mp->dh, &mp->dh2, &mp->dT, &mp->da}) *v = mp->alloc<float>(nj * kH, st);
    mp->dPQ = mp->alloc<float>(nj * 2 * kH, st);
    mp->dy = mp->alloc<float>(nj * kFout, st);
    mp->wpart = mp->alloc<float>((size_t)((nj + kWChunk - 1) / kWChunk) * 128 * 65, st);
    for (double **v : {&mp->rbuf, &mp->pbuf, &mp->zbuf}) *v = mp->alloc<double>(h.neq, st);
    mp->scal = mp->alloc<double>(8, st);
    mp->part = mp->alloc<double>(2 * (size_t)nb(h.neq) + 64, st);
    mp->cap = std::max(1, capacity);
    mp->pair_b = mp->alloc<double>((size_t)mp->cap * h.neq, st);
    mp->pair_t = mp->alloc<double>((size_t)mp->cap * h.neq, st);
    CB_CUDA(cudaStreamSynchronize(st));
    return mp;
}

void mpnn_destroy(Mpnn *mp)
{
    if (!mp) return;
    for (void *p : mp->allocs) cudaFree(p);
    delete mp;
}

size_t mpnn_bytes(const Mpnn *mp) { return mp ? mp->bytes : 0; }
long mpnn_adam_steps(const Mpnn *mp) { return mp ? mp->adam_t : 0; }
double mpnn_last_loss(const Mpnn *mp) { return mp ? mp->last_loss : 0.0; }
void mpnn_set_lr(Mpnn *mp, double lr) { mp->lr = (float)lr; }

void mpnn_set_params(Mpnn *mp, const float *theta, cudaStream_t st)
{
    CB_CUDA(cudaMemcpyAsync(mp->theta, theta, sizeof(float) * kParams, cudaMemcpyHostToDevice, st));
    CB_CUDA(cudaMemsetAsync(mp->m1, 0, sizeof(float) * kParams, st));
    CB_CUDA(cudaMemsetAsync(mp->m2, 0, sizeof(float) * kParams, st));
    mp->adam_t = 0;
}

void mpnn_get_params(const Mpnn *mp, float *theta, float *grad, cudaStream_t st)
{
    if (theta) CB_CUDA(cudaMemcpyAsync(theta, mp->theta, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st));
    if (grad) CB_CUDA(cudaMemcpyAsync(grad, mp->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st));
    CB_CUDA(cudaStreamSynchronize(st));
}

// The preconditioner inside the Arnoldi step: v_j = w * scale, z_j = P(v_j).
void mpnn_apply(Mpnn &mp, KrylovSolver &ks, cudaStream_t st)
{
    prep(mp, ks, ks.ctl, ks.w, nullptr, ks.V, ks.Z, st);
    forward(mp, ks.ctl, ks.Z, st);
}

// Forward (and with t, the loss and gradient) on device vectors r, t and an
// optional given p (else p = B^-1 r); z (device, optional) gets the output.
double mpnn_eval(Mpnn &mp, const KrylovSolver &ks, const double *r, const double *p, const double *t, double *z,
                 bool train, cudaStream_t st)
{
    prep(mp, ks, nullptr, r, p, nullptr, mp.zbuf, st);
    forward(mp, nullptr, mp.zbuf, st);
    if (z) CB_CUDA(cudaMemcpyAsync(z, mp.zbuf, sizeof(double) * mp.neq, cudaMemcpyDeviceToDevice, st));
    if (!t) return 0.0;
    backward(mp, t, st);
    if (train) adam_step(mp, st);
    double loss = 0;
    CB_CUDA(cudaMemcpyAsync(&loss, mp.scal + 3, sizeof(double), cudaMemcpyDeviceToHost, st));
    CB_CUDA(cudaStreamSynchronize(st));
    mp.last_loss = loss;
    return loss;
}

// Training pairs: a ring of (b, t = K^-1 b) in device memory.
void mpnn_push_pair(Mpnn &mp, const double *b, const double *t, cudaStream_t st)
{
    const size_t off = (size_t)mp.next * mp.neq;
    CB_CUDA(cudaMemcpyAsync(mp.pair_b + off, b, sizeof(double) * mp.neq, cudaMemcpyDeviceToDevice, st));
    CB_CUDA(cudaMemcpyAsync(mp.pair_t + off, t, sizeof(double) * mp.neq, cudaMemcpyDeviceToDevice, st));
    mp.next = (mp.next + 1) % mp.cap;
    mp.count = std::min(mp.count + 1, mp.cap);
}

void mpnn_slot(Mpnn &mp, double **b, double **t)
{
    const size_t off = (size_t)mp.next * mp.neq;
    *b = mp.pair_b + off;
    *t = mp.pair_t + off;
}

void mpnn_commit_pair(Mpnn &mp)
{
    mp.next = (mp.next + 1) % mp.cap;
    mp.count = std::min(mp.count + 1, mp.cap);
}

// `steps` Adam steps on stored pairs (one pair per step, newest first, then
// back through the ring); returns the last loss.
double mpnn_train(Mpnn &mp, const KrylovSolver &ks, int steps, cudaStream_t st)
{
    double loss = 0;
    for (int s = 0; s < steps && mp.count > 0; ++s) {
        const int k = ((mp.next - 1 - s) % mp.count + mp.count) % mp.count;
        const size_t off = (size_t)k * mp.neq;
        prep(mp, ks, nullptr, mp.pair_b + off, nullptr, nullptr, mp.zbuf, st);
        forward(mp, nullptr, mp.zbuf, st);
        backward(mp, mp.pair_t + off, st);
        adam_step(mp, st);
    }
    CB_CUDA(cudaMemcpyAsync(&loss, mp.scal + 3, sizeof(double), cudaMemcpyDeviceToHost, st));
    CB_CUDA(cudaStreamSynchronize(st));
    mp.last_loss = loss;
    return loss;
}

void krylov_apply_learned(KrylovSolver &ks, cudaStream_t st)
{
    if (!ks.mpnn) throw cb_status_error(CB_ERR_STATE, "no learned preconditioner attached");
    mpnn_apply(*(Mpnn *)ks.mpnn, ks, st);
}

}  // namespace cb
