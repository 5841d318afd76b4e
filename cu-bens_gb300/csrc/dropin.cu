// Drop-in layer: the hot-path entry points of prototypes.h with the
// reference's own signatures, computed on the GPU (declared in
// include/cubens_gb300_dropin.h). Built into libcubens_dropin.so.
//
// Each call uploads the host arrays it reads, runs the element, band-factor
// or vector kernels of libcubens_gb300, and writes back what the reference
// writes. Accumulating outputs (f_temp, ss, sm) are added to on the GPU, per
// destination in the reference's order (element types truss, frame, shell;
// elements ascending), starting from the caller's value, so the sums are
// formed as the reference forms them. Element arrays arrive in the
// reference's layout: per type concatenated, trusses first (see the offsets
// used below, e.g. shell.c:126-130, frame.c:246-247).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "cubens_gb300_dropin.h"
#include "dkt.cuh"
#include "frame.cuh"
#include "internal.hpp"

// The sizes and flags CU-BENs' main.c defines (main.c:323-328), bound weakly.
extern "C" {
extern long NJ __attribute__((weak));
extern long NE_TR __attribute__((weak));
extern long NE_FR __attribute__((weak));
extern long NE_SH __attribute__((weak));
extern long NEQ __attribute__((weak));
extern long NTSTPS __attribute__((weak));
extern long NBC __attribute__((weak));
extern int ANAFLAG __attribute__((weak));
extern int ALGFLAG __attribute__((weak));
extern int SLVFLAG __attribute__((weak));
extern double dt __attribute__((weak));
}

#define DI_CUDA(x)                                                                         \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess)                                                             \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + \
                                     " at " __FILE__ ":" + std::to_string(__LINE__));      \
    } while (0)

namespace {

using cb::DevFrame;
using cb::DevShell;
using cb::DevTruss;

// ---- sizes ----------------------------------------------------------------

struct Sizes {
    long nj, t, f, e, neq;
    int ana, alg, slv;
};

Sizes sizes()
{
    if (!&NJ || !&NE_TR || !&NE_FR || !&NE_SH || !&NEQ || !&ANAFLAG || !&ALGFLAG)
        throw std::runtime_error("the CU-BENs globals NJ, NE_TR, NE_FR, NE_SH, NEQ, ANAFLAG, ALGFLAG are "
                                 "not defined in this process");
    return Sizes{NJ, NE_TR, NE_FR, NE_SH, NEQ, ANAFLAG, ALGFLAG, &SLVFLAG ? SLVFLAG : 0};
}

void require_ana2(const Sizes &z, const char *fn)
{
    if (z.ana != 2) throw std::runtime_error(std::string(fn) + ": only ANAFLAG 2 is on the GPU path");
}

// ---- device context: one stream, grow-only scratch buffers, the factor ----

enum Slot {
    S_X, S_XIP, S_DD, S_EQX, S_CONN, S_EQ, S_PROP, S_AUX, S_XL, S_KEM, S_KEB, S_CIP, S_CI, S_AI, S_EFIP,
    S_EFI, S_LEN0, S_LENI, S_LENIP, S_DIR, S_N, S_FE, S_KEL, S_MAP_PTR, S_MAP_SRC, S_MAP_DST, S_VAL, S_OUT,
    S_OUT2, S_OUT3, S_OUT4, S_V1, S_V2, S_V3, S_V4, S_V5, S_V6, S_RED, S_SKY, S_SKYIDX, S_COUNT
};

struct Ctx {
    cudaStream_t st = nullptr;
    void *buf[S_COUNT] = {};
    size_t cap[S_COUNT] = {};
    cb::BandFactor bf;
    const double *factored_ss = nullptr;  // host skyline the device factor belongs to
    long factored_neq = -1;
};

std::mutex g_mu;
Ctx *g_ctx = nullptr;

Ctx &ctx()
{
    if (!g_ctx) {
        Ctx *c = new Ctx;
        DI_CUDA(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
        g_ctx = c;
    }
    return *g_ctx;
}

template <typename T>
T *dbuf(Slot s, size_t n)
{
    Ctx &c = ctx();
    size_t b = std::max<size_t>(1, n) * sizeof(T);
    if (c.cap[s] < b) {
        if (c.buf[s]) DI_CUDA(cudaFree(c.buf[s]));
        DI_CUDA(cudaMalloc(&c.buf[s], b));
        c.cap[s] = b;
    }
    return (T *)c.buf[s];
}

template <typename T>
T *upload(Slot s, const T *h, size_t n)
{
    T *d = dbuf<T>(s, n);
    if (n) DI_CUDA(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx().st));
    return d;
}

template <typename T>
T *upload(Slot s, const std::vector<T> &h)
{
    return upload(s, h.data(), h.size());
}

template <typename T>
void download(T *h, const T *d, size_t n)
{
    if (n) DI_CUDA(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx().st));
}

void sync() { DI_CUDA(cudaStreamSynchronize(ctx().st)); }

// SoA (k-major) from element-major AoS with a stride and offset.
std::vector<double> soa(const double *aos, long ne, int k, long offset = 0)
{
    std::vector<double> s((size_t)ne * k);
    for (long e = 0; e < ne; ++e)
        for (int j = 0; j < k; ++j) s[(size_t)j * ne + e] = aos[offset + (size_t)e * k + j];
    return s;
}

// Triads (rows x^, y^, z^) from the reference's c1/c2/c3 arrays at an offset.
std::vector<double> triads(const double *c1, const double *c2, const double *c3, long ne, long offset)
{
    std::vector<double> s((size_t)ne * 9);
    for (long e = 0; e < ne; ++e)
        for (int m = 0; m < 3; ++m) {
            s[(size_t)m * ne + e] = c1[offset + e * 3 + m];
            s[(size_t)(3 + m) * ne + e] = c2[offset + e * 3 + m];
            s[(size_t)(6 + m) * ne + e] = c3[offset + e * 3 + m];
        }
    return s;
}

// ---- kernels ----------------------------------------------------------------

constexpr int kT = 128;
inline unsigned nb(long n) { return (unsigned)std::max(1L, (n + kT - 1) / kT); }

// out[i] = base[i] + sum of in[src[k]], k in ptr[i]..ptr[i+1], added one at a
// time in list order; base and out may alias.
__global__ void gather_add_kernel(const int *__restrict__ ptr, const int *__restrict__ src,
                                  const double *__restrict__ in, const double *base, double *out, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = base[i];
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += in[src[k]];
    out[i] = s;
}

// updatc: joint coordinates (misc.c:83-93)
__global__ void upd_joints_kernel(const long *__restrict__ jcode, const double *__restrict__ dd, double *x,
                                  double *x_ip, long nj)
{
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= nj * 3) return;
    const long i = q / 3, j = q % 3;
    const long k = jcode[i * 7 + j];
    x_ip[q] = x[q];
    if (k != 0) x[q] += dd[k - 1];
}

// updatc: element geometry (misc.c:95-184) into the reference's arrays
__global__ void upd_elements_kernel(const double *__restrict__ x, const long *__restrict__ minc,
                                    const double *__restrict__ aux, const double *__restrict__ offset,
                                    const int *__restrict__ osflag, long T, long F, long E, double *defllen,
                                    double *deffarea, double *defslen, double *c1, double *c2, double *c3,
                                    double *xfr)
{
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= T + F + E) return;
    if (q < T) {
        const long j = minc[q * 2] - 1, k = minc[q * 2 + 1] - 1;
        double el[3] = {x[k * 3] - x[j * 3], x[k * 3 + 1] - x[j * 3 + 1], x[k * 3 + 2] - x[j * 3 + 2]};
        const double L = sqrt(el[0] * el[0] + el[1] * el[1] + el[2] * el[2]);
        defllen[q] = L;
        c1[q] = el[0] / L;
        c2[q] = el[1] / L;
        c3[q] = el[2] / L;
    } else if (q < T + F) {
        const long i = q - T;
        const long j = minc[2 * T + i * 2] - 1, k = minc[2 * T + i * 2 + 1] - 1;
        double pa[3], pb[3];
        for (int l = 0; l < 3; ++l) {
            const double oa = osflag[i] ? offset[i * 6 + l] : 0.0, ob = osflag[i] ? offset[i * 6 + 3 + l] : 0.0;
            pa[l] = x[j * 3 + l] + oa;
            pb[l] = x[k * 3 + l] + ob;
            xfr[i * 6 + l] = pa[l];
            xfr[i * 6 + 3 + l] = pb[l];
        }
        double c[9], L;
        cb::frame_geometry(pa, pb, aux + i * 3, c, &L);
        defllen[T + i] = L;
        for (int m = 0; m < 3; ++m) {
            c1[T + i * 3 + m] = c[m];
            c2[T + i * 3 + m] = c[3 + m];
            c3[T + i * 3 + m] = c[6 + m];
        }
    } else {
        const long i = q - T - F;
        const long base = 2 * T + 2 * F;
        const long a = minc[base + i * 3] - 1, b = minc[base + i * 3 + 1] - 1, cc = minc[base + i * 3 + 2] - 1;
        double c[9], area, slen[3];
        cb::shell_geometry(x + a * 3, x + b * 3, x + cc * 3, c, area, slen);
        deffarea[i] = area;
        for (int m = 0; m < 3; ++m) {
            defslen[i * 3 + m] = slen[m];
            c1[T + 3 * F + i * 3 + m] = c[m];
            c2[T + 3 * F + i * 3 + m] = c[3 + m];
            c3[T + 3 * F + i * 3 + m] = c[6 + m];
        }
    }
}

// Truss axial force from the updated geometry (forces_tr truss.c:326-375):
// N = EA (eps + eps^2/2) L/L0; -N c at end 1, +N c at end 2.
__global__ void truss_force_dropin_kernel(const double *__restrict__ ea, const double *__restrict__ len0,
                                          const double *__restrict__ len, const double *__restrict__ dir,
                                          double *__restrict__ ef, double *__restrict__ fe, long T)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= T) return;
    const double L = len[e], L0 = len0[e];
    const double eps = (L - L0) / L0;
    const double N = ea[e] * (eps + 0.5 * (eps * eps)) * L / L0;
    ef[2 * e] = N;
    ef[2 * e + 1] = -N;
    for (int d = 0; d < 3; ++d) {
        const double c = dir[d * T + e];
        fe[d * T + e] = -(N * c);
        fe[(3 + d) * T + e] = -((-N) * c);
    }
}

// Shell membrane and bending stiffness from the reference's initial geometry
// arrays (xlocal, farea, slength; stiffe_m_sh shell.c:487-531, stiffe_b_sh
// shell.c:533-658).
__global__ void shell_props_kernel(DevShell s, const double *__restrict__ farea, const double *__restrict__ slen,
                                   long E)
{
    long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double xl[3] = {s.xl[e], s.xl[E + e], s.xl[2 * E + e]};
    const double sl[3] = {slen[e * 3], slen[e * 3 + 1], slen[e * 3 + 2]};
    double kem[36], keb[81];
    const double em = s.prop[e], nu = s.prop[E + e], t = s.prop[2 * E + e];
    cb::shell_kem(em, nu, t, farea[e], xl, kem);
    cb::shell_keb(em, nu, t, farea[e], xl, sl, keb);
    for (int k = 0; k < 36; ++k) s.kem[k * E + e] = kem[k];
    for (int k = 0; k < 81; ++k) s.keb[k * E + e] = keb[k];
}

__global__ void dot_partial_kernel(const double *__restrict__ a, const double *__restrict__ b, double *part,
                                   long n)
{
    __shared__ double sm[256];
    double s = 0;
    for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += gridDim.x * 256L) s += a[i] * b[i];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// quad's per-root sums (arc.c:96-107) and the update of dt and dd
// (arc.c:111-124) for the selected root.
__global__ void quad_gamma_kernel(const double *__restrict__ dt, const double *__restrict__ dp,
                                  const double *__restrict__ ddr, const double *__restrict__ ddq, double r1,
                                  double r2, double *part, long n)
{
    __shared__ double s1[256], s2[256];
    double g1 = 0, g2 = 0;
    for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += gridDim.x * 256L) {
        const double a = dt[i] - dp[i];
        g1 += a * (dt[i] - dp[i] + ddr[i] + r1 * ddq[i]);
        g2 += a * (dt[i] - dp[i] + ddr[i] + r2 * ddq[i]);
    }
    s1[threadIdx.x] = g1;
    s2[threadIdx.x] = g2;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s1[0];
        part[2 * blockIdx.x + 1] = s2[0];
    }
}

__global__ void quad_apply_kernel(double *dt, const double *__restrict__ dp, const double *__restrict__ ddr,
                                  const double *__restrict__ ddq, double *dd, double root, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double di = dt[i] - dp[i] + ddr[i] + root * ddq[i];
    dt[i] = di + dp[i];
    dd[i] = ddr[i] + root * ddq[i];
}

// the five sums of test (misc.c:187-250)
__global__ void test_sums_kernel(const double *__restrict__ dtemp, const double *__restrict__ dd,
                                 const double *__restrict__ f, const double *__restrict__ fp,
                                 const double *__restrict__ q, const double *__restrict__ fip, double *part, long n)
{
    __shared__ double s[5][128];
    double a[5] = {0, 0, 0, 0, 0};
    for (long i = blockIdx.x * 128L + threadIdx.x; i < n; i += gridDim.x * 128L) {
        a[0] += dd[i] * dd[i];
        a[1] += dtemp[i] * dtemp[i];
        a[2] += (q[i] - f[i]) * (q[i] - f[i]);
        a[3] += (q[i] - fp[i]) * (q[i] - fp[i]);
        a[4] += dd[i] * (q[i] - fip[i]);
    }
    for (int k = 0; k < 5; ++k) s[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int k = 0; k < 5; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 5; ++k) part[k * gridDim.x + blockIdx.x] = s[k][0];
}

// skyline <-> band (upper triangle by columns, 1-based maxa; band L(i,j) at
// band[j*ld + (i-j)])
__global__ void sky_to_band_kernel(const double *__restrict__ ss, const long *__restrict__ idx, double *band,
                                   long ld, long nent)
{
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= nent) return;
    band[idx[q]] = ss[q];
}

__global__ void band_to_sky_kernel(const double *__restrict__ band, const long *__restrict__ idx, double *ss,
                                   long nent)
{
    long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= nent) return;
    ss[q] = band[idx[q]];
}

__global__ void keff_diag_kernel(const double *__restrict__ ss, const long *__restrict__ maxa,
                                 const double *__restrict__ sm, double c0, double den, double *keff, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long k = maxa[i] - 1;
    keff[k] = ss[k] + c0 * sm[i] / den;
}

__global__ void reff_kernel(const double *__restrict__ r, const double *__restrict__ sm,
                            const double *__restrict__ vm, const double *__restrict__ am, double alpham,
                            double alphaf, double a2, double a3, double *out, long n)
{
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = r[i] + sm[i] * ((1 - alpham) * (vm[i] * a2 + am[i] * a3) - alpham * am[i]) / (1 - alphaf);
}

// ---- gather maps built from the reference's code arrays ---------------------

struct Map {
    std::vector<int> ptr, src;
    std::vector<long> dst;  // destination index per row
};

// Contributions of element values val[k*ne + e] (k < nd) to destination
// mc[e*nd + k] - 1, rows sorted by destination, elements ascending.
void add_force_contrib(std::vector<std::vector<int>> &lists, const long *mc, long ne, int nd, long base)
{
    for (long e = 0; e < ne; ++e)
        for (int k = 0; k < nd; ++k) {
            const long q = mc[e * nd + k];
            if (q) lists[q - 1].push_back((int)(base + k * ne + e));
        }
}

Map finish(std::vector<std::vector<int>> &lists)
{
    Map m;
    m.ptr.push_back(0);
    for (size_t i = 0; i < lists.size(); ++i) {
        m.src.insert(m.src.end(), lists[i].begin(), lists[i].end());
        m.ptr.push_back((int)m.src.size());
    }
    return m;
}

inline int packed_idx(int ie, int je, int nd) { return ie * nd - ie * (ie - 1) / 2 + (je - ie); }

// Skyline slots of the packed element matrices (ss index k-1 for the pair
// ie <= je, stiff_tr truss.c:170-193 / stiff_fr frame.c:328-344 /
// stiff_sh shell.c:307-329), rows compacted to the touched slots.
Map skyline_map(const long *mc, long ne, int nd, const long *maxa)
{
    std::vector<std::pair<long, int>> all;
    const int np = nd * (nd + 1) / 2;
    all.reserve((size_t)ne * np);
    for (long e = 0; e < ne; ++e)
        for (int je = 0; je < nd; ++je) {
            const long j = mc[e * nd + je];
            if (!j) continue;
            for (int ie = 0; ie <= je; ++ie) {
                const long i = mc[e * nd + ie];
                if (!i) continue;
                const long k = i > j ? maxa[i - 1] + (i - j) : maxa[j - 1] + (j - i);
                all.push_back({k - 1, (int)(packed_idx(ie, je, nd) * ne + e)});
            }
        }
    std::stable_sort(all.begin(), all.end(),
                     [](const std::pair<long, int> &a, const std::pair<long, int> &b) { return a.first < b.first; });
    Map m;
    m.ptr.push_back(0);
    for (size_t q = 0; q < all.size(); ++q) {
        if (q == 0 || all[q].first != all[q - 1].first) {
            if (q) m.ptr.push_back((int)m.src.size());
            m.dst.push_back(all[q].first);
        }
        m.src.push_back(all[q].second);
    }
    m.ptr.push_back((int)m.src.size());
    return m;
}

// host value += device element contributions through a map (force rows are
// all NEQ equations; skyline rows are the touched slots m.dst)
void accumulate(const Map &m, const double *val_dev, double *host, long nrows, bool compact)
{
    cudaStream_t st = ctx().st;
    const int *ptr = upload(S_MAP_PTR, m.ptr);
    const int *src = upload(S_MAP_SRC, m.src);
    std::vector<double> base((size_t)nrows);
    if (compact)
        for (long i = 0; i < nrows; ++i) base[i] = host[m.dst[i]];
    else
        std::memcpy(base.data(), host, sizeof(double) * nrows);
    double *b = upload(S_OUT, base);
    gather_add_kernel<<<nb(nrows), kT, 0, st>>>(ptr, src, val_dev, b, b, nrows);
    DI_CUDA(cudaGetLastError());
    download(base.data(), b, nrows);
    sync();
    if (compact)
        for (long i = 0; i < nrows; ++i) host[m.dst[i]] = base[i];
    else
        std::memcpy(host, base.data(), sizeof(double) * nrows);
}

double device_sum(const double *part, int n)
{
    std::vector<double> h(n);
    download(h.data(), part, n);
    sync();
    double s = 0;
    for (int i = 0; i < n; ++i) s += h[i];
    return s;
}

constexpr int kRedBlocks = 148;

// ---- shells -----------------------------------------------------------------

DevShell upload_shells(const Sizes &z, const double *emod, const double *nu, const double *thick,
                       const double *xlocal, const double *farea, const double *slength, const long *minc,
                       const long *mcode)
{
    const long E = z.e, T = z.t, F = z.f;
    DevShell s;
    std::vector<int> conn(3 * E), eq(18 * E);
    std::vector<double> prop(3 * E);
    for (long e = 0; e < E; ++e) {
        for (int a = 0; a < 3; ++a) conn[a * E + e] = (int)(minc[2 * T + 2 * F + e * 3 + a] - 1);
        for (int k = 0; k < 18; ++k) eq[k * E + e] = (int)mcode[6 * T + 14 * F + e * 18 + k] - 1;
        prop[e] = emod[T + F + e];
        prop[E + e] = nu[e];
        prop[2 * E + e] = thick[e];
    }
    s.conn = upload(S_CONN, conn);
    s.eq = upload(S_EQ, eq);
    s.prop = upload(S_PROP, prop);
    s.xl = upload(S_XL, soa(xlocal, E, 3));
    s.kem = dbuf<double>(S_KEM, 36 * E);
    s.keb = dbuf<double>(S_KEB, 81 * E);
    const double *fa = upload(S_V1, farea, E);
    const double *sl = upload(S_V2, slength, 3 * E);
    shell_props_kernel<<<nb(E), kT, 0, ctx().st>>>(s, fa, sl, E);
    DI_CUDA(cudaGetLastError());
    return s;
}

DevFrame upload_frames(const Sizes &z, const double *emod, const double *gmod, const double *carea,
                       const double *istrong, const double *iweak, const double *ipolar, const double *iwarp,
                       const long *minc, const long *mcode, const double *aux)
{
    const long F = z.f, T = z.t;
    DevFrame fr;
    std::vector<int> conn(2 * F), eq(14 * F);
    std::vector<double> prop(8 * F, 0.0);
    for (long i = 0; i < F; ++i) {
        if (minc) {
            conn[i] = (int)(minc[2 * T + i * 2] - 1);
            conn[F + i] = (int)(minc[2 * T + i * 2 + 1] - 1);
        }
        for (int k = 0; k < 14; ++k) eq[k * F + i] = (int)mcode[6 * T + i * 14 + k] - 1;
        prop[i] = emod[T + i];
        prop[F + i] = gmod[i];
        prop[3 * F + i] = carea[T + i];
        prop[4 * F + i] = istrong[i];
        prop[5 * F + i] = iweak[i];
        prop[6 * F + i] = ipolar[i];
        prop[7 * F + i] = iwarp[i];
    }
    fr.conn = upload(S_CONN, conn);
    fr.eq = upload(S_EQ, eq);
    fr.prop = upload(S_PROP, prop);
    if (aux) fr.aux = upload(S_AUX, soa(aux, F, 3));
    return fr;
}

void check_frames_plain(const Sizes &z, const int *osflag, const int *mendrel, const double *efFE, const char *fn)
{
    for (long i = 0; i < z.f; ++i) {
        if (osflag && osflag[i]) throw std::runtime_error(std::string(fn) + ": member end offsets are not supported");
        if (mendrel && mendrel[i * 5]) throw std::runtime_error(std::string(fn) + ": member end releases are not supported");
        if (efFE)
            for (int k = 0; k < 14; ++k)
                if (efFE[i * 14 + k] != 0)
                    throw std::runtime_error(std::string(fn) + ": fixed-end forces of distributed loads are not supported");
    }
}

// ---- band factor of a skyline ---------------------------------------------------

// Band index of every skyline entry: column n (1-based), row i = n - off.
std::vector<long> sky_index(const long *maxa, long neq, long ld)
{
    std::vector<long> idx((size_t)(maxa[neq] - 1));
    for (long n = 1; n <= neq; ++n) {
        const long h = maxa[n] - maxa[n - 1] - 1;
        for (long off = 0; off <= h; ++off) idx[maxa[n - 1] - 1 + off] = (n - off - 1) * ld + off;
    }
    return idx;
}

long skyline_bw(const long *maxa, long neq)
{
    long bw = 0;
    for (long n = 0; n < neq; ++n) bw = std::max(bw, maxa[n + 1] - maxa[n] - 1);
    return bw;
}

void ensure_band(long neq, long bw)
{
    Ctx &c = ctx();
    if (c.bf.band && c.bf.n == neq && c.bf.bw == std::max(1L, bw)) return;
    if (c.bf.band) cb::band_free(c.bf);
    cb::band_alloc(c.bf, neq, bw, false);
    c.factored_ss = nullptr;
}

// Load a skyline into the band (zero elsewhere).
void load_band(const long *maxa, const double *ss, long neq)
{
    Ctx &c = ctx();
    const long lss = maxa[neq] - 1;
    ensure_band(neq, skyline_bw(maxa, neq));
    cb::BandFactor &f = c.bf;
    DI_CUDA(cudaMemsetAsync(f.band, 0, sizeof(double) * (size_t)f.ld * f.nblk * f.s, c.st));
    std::vector<long> idx = sky_index(maxa, neq, f.ld);
    const long *di = upload(S_SKYIDX, idx);
    const double *ds = upload(S_SKY, ss, lss);
    sky_to_band_kernel<<<nb(lss), kT, 0, c.st>>>(ds, di, (double *)f.band, f.ld, lss);
    DI_CUDA(cudaGetLastError());
}

void store_band(const long *maxa, double *ss, long neq)
{
    Ctx &c = ctx();
    const long lss = maxa[neq] - 1;
    std::vector<long> idx = sky_index(maxa, neq, c.bf.ld);
    const long *di = upload(S_SKYIDX, idx);
    double *ds = dbuf<double>(S_SKY, lss);
    band_to_sky_kernel<<<nb(lss), kT, 0, c.st>>>((const double *)c.bf.band, di, ds, lss);
    DI_CUDA(cudaGetLastError());
    download(ss, ds, lss);
    sync();
}

void report(const char *fn, const std::exception &e) { std::fprintf(stderr, "cubens %s: %s\n", fn, e.what()); }

}  // namespace

extern "C" {

void updatc(double *px_temp, double *px_ip, double *pxfr_temp, double *pdd, double *pdefllen_i,
            double *pdeffarea_i, double *pdefslen_i, double *poffset, int *posflag, double *pauxpt,
            double *pc1_i, double *pc2_i, double *pc3_i, long *pminc, long *pjcode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        cudaStream_t st = ctx().st;
        const long T = z.t, F = z.f, E = z.e, NJ3 = z.nj * 3;
        double *x = upload(S_X, px_temp, NJ3);
        double *xip = dbuf<double>(S_XIP, NJ3);
        const double *dd = upload(S_DD, pdd, z.neq);
        const long *jc = upload(S_SKYIDX, pjcode, z.nj * 7);
        upd_joints_kernel<<<nb(NJ3), kT, 0, st>>>(jc, dd, x, xip, z.nj);
        const long nminc = 2 * T + 2 * F + 3 * E;
        const long *mi = (const long *)upload(S_MAP_DST, pminc, nminc);
        const double *aux = F ? upload(S_AUX, pauxpt, 3 * F) : nullptr;
        const double *off = F ? upload(S_V3, poffset, 6 * F) : nullptr;
        const int *osf = F ? upload(S_EQ, posflag, F) : nullptr;
        const long nc = T + 3 * F + 3 * E;
        double *len = dbuf<double>(S_LENI, T + F), *area = dbuf<double>(S_AI, E), *slen = dbuf<double>(S_V4, 3 * E);
        double *c1 = dbuf<double>(S_OUT2, nc), *c2 = dbuf<double>(S_OUT3, nc), *c3 = dbuf<double>(S_OUT4, nc);
        double *xfr = dbuf<double>(S_V5, 6 * F);
        upd_elements_kernel<<<nb(T + F + E), kT, 0, st>>>(x, mi, aux, off, osf, T, F, E, len, area, slen, c1, c2,
                                                           c3, xfr);
        DI_CUDA(cudaGetLastError());
        download(px_temp, x, NJ3);
        if (px_ip) download(px_ip, xip, NJ3);
        if (F && pxfr_temp) download(pxfr_temp, xfr, 6 * F);
        download(pdefllen_i, len, T + F);
        if (E) {
            download(pdeffarea_i, area, E);
            download(pdefslen_i, slen, 3 * E);
        }
        download(pc1_i, c1, nc);
        download(pc2_i, c2, nc);
        download(pc3_i, c3, nc);
        sync();
    } catch (const std::exception &e) {
        report("updatc", e);
    }
}

void forces_tr(double *pf_temp, double *pef_i, double *pd, double *pemod, double *pcarea, double *pllength,
               double *pdefllen_i, double *pyield, double *pc1_i, double *pc2_i, double *pc3_i, long *pmcode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        require_ana2(z, "forces_tr");
        const long T = z.t;
        if (!T) return;
        std::vector<double> ea(T), dir(3 * T);
        for (long e = 0; e < T; ++e) {
            ea[e] = pemod[e] * pcarea[e];
            dir[e] = pc1_i[e];
            dir[T + e] = pc2_i[e];
            dir[2 * T + e] = pc3_i[e];
        }
        const double *dea = upload(S_PROP, ea), *dl0 = upload(S_LEN0, pllength, T), *dl = upload(S_LENI, pdefllen_i, T);
        const double *ddir = upload(S_DIR, dir);
        double *ef = dbuf<double>(S_EFI, 2 * T), *fe = dbuf<double>(S_FE, 6 * T);
        truss_force_dropin_kernel<<<nb(T), kT, 0, ctx().st>>>(dea, dl0, dl, ddir, ef, fe, T);
        DI_CUDA(cudaGetLastError());
        download(pef_i, ef, 2 * T);
        std::vector<std::vector<int>> lists(z.neq);
        add_force_contrib(lists, pmcode, T, 6, 0);
        accumulate(finish(lists), fe, pf_temp, z.neq, false);
    } catch (const std::exception &e) {
        report("forces_tr", e);
    }
}

void stiff_tr(double *pss, double *pemod, double *pcarea, double *plength, double *pdefllen_ip, double *pyield,
              double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pef_ip, long *pmaxa, long *pmcode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        require_ana2(z, "stiff_tr");
        const long T = z.t;
        if (!T) return;
        DevTruss t;
        std::vector<double> ea(T), dir(3 * T), n(T);
        for (long e = 0; e < T; ++e) {
            ea[e] = pemod[e] * pcarea[e];
            dir[e] = pc1_ip[e];
            dir[T + e] = pc2_ip[e];
            dir[2 * T + e] = pc3_ip[e];
            n[e] = pef_ip[2 * e];
        }
        t.ea = upload(S_PROP, ea);
        t.len0 = upload(S_LEN0, plength, T);
        t.len_c = upload(S_LENI, pdefllen_ip, T);
        t.dir_c = upload(S_DIR, dir);
        t.n_c = upload(S_N, n);
        double *kel = dbuf<double>(S_KEL, 21 * T);
        cb::launch_truss_tangent<double>(t, kel, T, ctx().st);
        DI_CUDA(cudaGetLastError());
        Map m = skyline_map(pmcode, T, 6, pmaxa);
        accumulate(m, kel, pss, (long)m.dst.size(), true);
    } catch (const std::exception &e) {
        report("stiff_tr", e);
    }
}

int forces_fr(double *pf_temp, double *pef_ip, double *pef_i, double *pefFE_ref, double *pefFE_ip,
              double *pefFE_i, int *pyldflag, double *pdd, double *pemod, double *pgmod, double *pcarea,
              double *poffset, int *posflag, double *pllength, double *pdefllen_ip, double *pistrong,
              double *piweak, double *pipolar, double *piwarp, double *pyield, double *pzstrong, double *pzweak,
              double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pc1_i, double *pc2_i, double *pc3_i,
              int *pmendrel, long *pmcode, double *pdlpf, int *pitecnt)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        require_ana2(z, "forces_fr");
        const long F = z.f, T = z.t;
        if (!F) return 0;
        check_frames_plain(z, posflag, pmendrel, pefFE_ip, "forces_fr");
        cudaStream_t st = ctx().st;
        // the member triads of the current iteration come from updatc in c_i;
        // the kernel forms them from coordinates, so hand it end points that
        // reproduce them: x_temp is not an argument of forces_fr
        DevFrame fr = upload_frames(z, pemod, pgmod, pcarea, pistrong, piweak, pipolar, piwarp, nullptr, pmcode,
                                    nullptr);
        fr.c_ip = upload(S_CIP, triads(pc1_ip, pc2_ip, pc3_ip, F, T));
        fr.ef_ip = upload(S_EFIP, soa(pef_ip, F, 14, 2 * T));
        fr.len_ip = upload(S_LENIP, pdefllen_ip + T, F);
        const double *ci = upload(S_CI, triads(pc1_i, pc2_i, pc3_i, F, T));
        fr.ef_i = dbuf<double>(S_EFI, 14 * F);
        const double *lref = upload(S_LEN0, pllength + T, F);
        const double *dd = upload(S_DD, pdd, z.neq);
        double *fe = dbuf<double>(S_FE, 14 * F);
        cb::launch_frame_forces_given_triads(fr, ci, dd, lref, fe, F, st);
        DI_CUDA(cudaGetLastError());
        std::vector<double> efs(14 * F);
        download(efs.data(), fr.ef_i, 14 * F);
        sync();
        for (long i = 0; i < F; ++i)
            for (int k = 0; k < 14; ++k) {
                pef_i[2 * T + i * 14 + k] = efs[(size_t)k * F + i];
                if (pefFE_i) pefFE_i[i * 14 + k] = 0.0;
            }
        std::vector<std::vector<int>> lists(z.neq);
        add_force_contrib(lists, pmcode + 6 * T, F, 14, 0);
        accumulate(finish(lists), fe, pf_temp, z.neq, false);
        return 0;
    } catch (const std::exception &e) {
        report("forces_fr", e);
        return 1;
    }
}

void stiff_fr(double *pss, double *pemod, double *pgmod, double *pcarea, double *poffset, int *posflag,
              double *pllength, double *pdefllen_ip, double *pistrong, double *piweak, double *pipolar,
              double *piwarp, int *pyldflag, double *pyield, double *pzstrong, double *pzweak, double *pc1_ip,
              double *pc2_ip, double *pc3_ip, double *pef_ip, double *pefFE_ip, int *pmendrel, long *pmaxa,
              long *pmcode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        require_ana2(z, "stiff_fr");
        const long F = z.f, T = z.t;
        if (!F) return;
        check_frames_plain(z, posflag, pmendrel, pefFE_ip, "stiff_fr");
        DevFrame fr = upload_frames(z, pemod, pgmod, pcarea, pistrong, piweak, pipolar, piwarp, nullptr, pmcode,
                                    nullptr);
        const double *c = upload(S_CIP, triads(pc1_ip, pc2_ip, pc3_ip, F, T));
        const double *ef = upload(S_EFIP, soa(pef_ip, F, 14, 2 * T));
        const double *len = upload(S_LENIP, pdefllen_ip + T, F);
        const double *lref = upload(S_LEN0, pllength + T, F);
        double *kel = dbuf<double>(S_KEL, 105 * F);
        cb::launch_frame_tangent<double>(fr, c, ef, len, lref, kel, F, ctx().st);
        DI_CUDA(cudaGetLastError());
        Map m = skyline_map(pmcode + 6 * T, F, 14, pmaxa);
        accumulate(m, kel, pss, (long)m.dst.size(), true);
    } catch (const std::exception &e) {
        report("stiff_fr", e);
    }
}

void mass_fr(double *psm, double *pcarea, double *pllength, double *pistrong, double *piweak, double *pipolar,
             double *piwarp, double *pdens, int *posflag, double *poffset, double *px, double *pxfr, long *pminc,
             long *pmcode, double *pjac)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        const long F = z.f, T = z.t;
        if (!F) return;
        check_frames_plain(z, posflag, nullptr, nullptr, "mass_fr");
        if (T) throw std::runtime_error("mass_fr: models with trusses and frames are not supported (the "
                                        "reference reads the members' area, density and length at the truss "
                                        "indices, frame.c:1357-1363)");
        // frame-only models: the member's area, density and length sit at
        // index i (frame.c:1320-1363)
        cudaStream_t st = ctx().st;
        DevFrame fr;
        std::vector<int> conn(2 * F);
        std::vector<double> prop(8 * F, 0.0);
        for (long i = 0; i < F; ++i) {
            conn[i] = (int)(pminc[2 * T + i * 2] - 1);
            conn[F + i] = (int)(pminc[2 * T + i * 2 + 1] - 1);
            prop[2 * F + i] = pdens[i];
            prop[3 * F + i] = pcarea[i];
        }
        fr.conn = upload(S_CONN, conn);
        fr.prop = upload(S_PROP, prop);
        const double *x = upload(S_X, px, z.nj * 3);
        double *lt = dbuf<double>(S_LENI, F), *me = dbuf<double>(S_FE, 14 * F);
        cb::launch_frame_mass(fr, x, lt, me, F, st);
        DI_CUDA(cudaGetLastError());
        std::vector<double> L(F);
        download(L.data(), lt, F);
        sync();
        for (long i = 0; i < F; ++i) {
            pllength[T + i] = L[i];
            for (int l = 0; l < 3; ++l) {
                pxfr[i * 6 + l] = px[conn[i] * 3 + l];
                pxfr[i * 6 + 3 + l] = px[conn[F + i] * 3 + l];
            }
        }
        // mass_fr adds to sm with mcode at index i*14 (no truss offset)
        std::vector<std::vector<int>> lists(z.neq);
        add_force_contrib(lists, pmcode, F, 14, 0);
        accumulate(finish(lists), me, psm, z.neq, false);
    } catch (const std::exception &e) {
        report("mass_fr", e);
    }
}

int forces_sh(double *pf_temp, double *pef_ip, double *pef_i, double *pefN_temp, double *pefM_temp, double *pdd,
              double *pd_temp, double *pchi_temp, double *px_temp, double *px_ip, double *pemod, double *pnu,
              double *pxlocal, double *pthick, double *pfarea, double *pdeffarea_ip, double *pslength,
              double *pdefslen_ip, double *pyield, double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pc1_i,
              double *pc2_i, double *pc3_i, long *pminc, long *pmcode, long *pjcode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        require_ana2(z, "forces_sh");
        const long E = z.e, T = z.t, F = z.f;
        if (!E) return 0;
        cudaStream_t st = ctx().st;
        DevShell s = upload_shells(z, pemod, pnu, pthick, pxlocal, pfarea, pslength, pminc, pmcode);
        s.c_ip = upload(S_CIP, triads(pc1_ip, pc2_ip, pc3_ip, E, T + 3 * F));
        s.ef_ip = upload(S_EFIP, soa(pef_ip, E, 18, 2 * T + 14 * F));
        s.c_i = dbuf<double>(S_CI, 9 * E);
        s.a_i = dbuf<double>(S_AI, E);
        s.ef_i = dbuf<double>(S_EFI, 18 * E);
        const double *x = upload(S_X, px_temp, z.nj * 3);
        const double *dd = upload(S_DD, pdd, z.neq);
        double *fe = dbuf<double>(S_FE, 18 * E);
        cb::launch_shell_forces(s, x, dd, fe, E, st);
        DI_CUDA(cudaGetLastError());
        std::vector<double> efs(18 * E);
        download(efs.data(), s.ef_i, 18 * E);
        sync();
        for (long e = 0; e < E; ++e)
            for (int k = 0; k < 18; ++k) pef_i[2 * T + 14 * F + e * 18 + k] = efs[(size_t)k * E + e];
        std::vector<std::vector<int>> lists(z.neq);
        add_force_contrib(lists, pmcode + 6 * T + 14 * F, E, 18, 0);
        accumulate(finish(lists), fe, pf_temp, z.neq, false);
        return 0;
    } catch (const std::exception &e) {
        report("forces_sh", e);
        return 1;
    }
}

void stiff_sh(double *pss, double *pemod, double *pnu, double *px_temp, double *pxlocal, double *pthick,
              double *pfarea, double *pdeffarea_ip, double *pslength, double *pdefslen_ip, double *pyield,
              double *pc1_ip, double *pc2_ip, double *pc3_ip, double *pef_ip, double *pd_temp, double *pchi_temp,
              double *pefN_temp, double *pefM_temp, long *pmaxa, long *pminc, long *pmcode)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        require_ana2(z, "stiff_sh");
        const long E = z.e, T = z.t, F = z.f;
        if (!E) return;
        DevShell s = upload_shells(z, pemod, pnu, pthick, pxlocal, pfarea, pslength, pminc, pmcode);
        s.c_c = upload(S_CIP, triads(pc1_ip, pc2_ip, pc3_ip, E, T + 3 * F));
        s.a_c = upload(S_AI, pdeffarea_ip, E);
        const double *x = upload(S_X, px_temp, z.nj * 3);
        double *kel = dbuf<double>(S_KEL, 171 * E);
        cb::launch_shell_tangent<double>(s, x, kel, E, ctx().st);
        DI_CUDA(cudaGetLastError());
        Map m = skyline_map(pmcode + 6 * T + 14 * F, E, 18, pmaxa);
        accumulate(m, kel, pss, (long)m.dst.size(), true);
    } catch (const std::exception &e) {
        report("stiff_sh", e);
    }
}

int skyfact(long *pmaxa, double *pss_temp, double *pssd, double *pdd, int fact, int *pdet)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        *pdet = 0;
        if (fact != 0) return 0;
        const long N = z.neq;
        load_band(pmaxa, pss_temp, N);
        Ctx &c = ctx();
        cb::band_factor(c.bf, c.st, false, nullptr);
        int fl[2] = {0, 0};
        std::vector<double> piv(N);
        download(fl, c.bf.flags, 2);
        download(piv.data(), c.bf.ssd, N);
        store_band(pmaxa, pss_temp, N);
        c.factored_ss = pss_temp;
        c.factored_neq = N;
        if (z.alg != 3) {
            // solve.c:558-561: the first pivot <= 0 ends the factorisation with 1
            for (long n = 0; n < N; ++n)
                if (!(piv[n] > 0)) {
                    std::fprintf(stderr, "\n***ERROR*** Non-positive definite stiffness matrix\n");
                    return 1;
                }
            return 0;
        }
        for (long n = 0; n < N; ++n) {
            pssd[n] = piv[n];
            if (piv[n] == 0) {
                std::fprintf(stderr, "\n***ERROR*** Singular stiffness matrix\n");
                return 1;
            }
            if (!(piv[n] > 0)) *pdet = 1;
        }
        return 0;
    } catch (const std::exception &e) {
        report("skyfact", e);
        return 1;
    }
}

int skysolve(long *pmaxa, double *pss, double *pssd, double *pdd, int fact, int *pdet)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        Ctx &c = ctx();
        const long N = z.neq;
        if (c.factored_ss != pss || c.factored_neq != N) {
            load_band(pmaxa, pss, N);
            cb::band_use_factored(c.bf, c.st);
            c.factored_ss = pss;
            c.factored_neq = N;
        }
        double *rhs = upload(S_V6, pdd, N);
        double *x = dbuf<double>(S_OUT, N);
        cb::band_solve(c.bf, rhs, x, c.st, false, nullptr);
        DI_CUDA(cudaGetLastError());
        cb::GridBarrier bar{};
        download(pdd, x, N);
        download(&bar, c.bf.bar, 1);
        sync();
        if (bar.err) throw std::runtime_error("a grid barrier of the solve timed out");
        return 0;
    } catch (const std::exception &e) {
        report("skysolve", e);
        return 1;
    }
}

int solve(long *pjcode_fsi, double *pss, double *pss_fsi, double *psm, double *psm_fsi, double *psd_fsi,
          double *pr, double *pdd, long *pmaxa, double *pssd, int *pdet, double *pum, double *pvm, double *pam,
          double *puc, double *pvc, double *pac, double *pqdyn, double *ptstps, double *pKeff, double *pReff,
          double *pMeff, int *pAp, int *pAi, double *pAx, double alpham, double alphaf, int *pipiv, int fact,
          double ddt, double *ppdisp, long *pkht, int *piter, int *pii, int *pij, int tstp)
{
    Sizes z;
    try {
        z = sizes();
        if (z.slv != 0) throw std::runtime_error("solve: only SLVFLAG 0 (skyline) is on the GPU path");
        if (&NBC && NBC != 0) throw std::runtime_error("solve: prescribed motion (NBC > 0) is not supported");
    } catch (const std::exception &e) {
        report("solve", e);
        return 1;
    }
    const long N = z.neq;
    std::memcpy(pdd, pr, sizeof(double) * N);
    if (z.alg < 4) {
        // solve.c:83-90: skyfact's return is not checked
        skyfact(pmaxa, pss, pssd, pdd, fact, pdet);
        skysolve(pmaxa, pss, pssd, pdd, fact, pdet);
        return 0;
    }
    if (z.alg != 5) {
        std::fprintf(stderr, "cubens solve: ALGFLAG %d is not on the GPU path\n", z.alg);
        return 1;
    }
    // solve.c:139-222 and 469-533: Keff = K + a0 (1 - am)/(1 - af) M on the
    // diagonal, factored; Reff from the current iteration's vm, am (the
    // caller passes uc_i, vc_i, ac_i in those positions)
    const double alpha = std::pow(1 - alpham + alphaf, 2) / 4;
    const double dt_temp = ddt * (&dt ? dt : 0.0);
    const double a0 = 1 / (alpha * std::pow(dt_temp, 2));
    const double a2 = 1 / (alpha * dt_temp);
    const double a3 = 1 / (2 * alpha) - 1;
    const long lss = pmaxa[N] - 1;
    try {
        std::lock_guard<std::mutex> lock(g_mu);
        cudaStream_t st = ctx().st;
        const double *ss = upload(S_SKY, pss, lss);
        double *keff = dbuf<double>(S_V5, lss);
        DI_CUDA(cudaMemcpyAsync(keff, ss, sizeof(double) * lss, cudaMemcpyDeviceToDevice, st));
        const long *maxa = (const long *)upload(S_MAP_DST, pmaxa, N + 1);
        const double *sm = upload(S_V1, psm, N);
        keff_diag_kernel<<<nb(N), kT, 0, st>>>(ss, maxa, sm, a0 * (1 - alpham), 1 - alphaf, keff, N);
        const double *r = upload(S_V2, pr, N), *vm = upload(S_V3, pvm, N), *am = upload(S_V4, pam, N);
        double *reff = dbuf<double>(S_V6, N);
        reff_kernel<<<nb(N), kT, 0, st>>>(r, sm, vm, am, alpham, alphaf, a2, a3, reff, N);
        DI_CUDA(cudaGetLastError());
        std::vector<double> hk(lss), hr(N);
        download(hk.data(), keff, lss);
        download(hr.data(), reff, N);
        sync();
        std::memcpy(pKeff, hk.data(), sizeof(double) * lss);
        std::memcpy(pReff, hr.data(), sizeof(double) * N);
    } catch (const std::exception &e) {
        report("solve", e);
        return 1;
    }
    skyfact(pmaxa, pKeff, pssd, pdd, fact, pdet);
    skysolve(pmaxa, pKeff, pssd, pReff, fact, pdet);
    std::memcpy(pdd, pReff, sizeof(double) * N);
    return 0;
}

int quad(double *pa, double *pb, double *pc, double *pdt, double *pdp, double *pddr, double *pddq, double *pdd,
         double *pdlpf, double *plpft)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        const long N = z.neq;
        const double a = *pa, b = *pb, c = *pc;
        if (!(b * b - 4 * a * c > 0)) return 2;  // imaginary roots (arc.c:85-93)
        const double r1 = (-b + std::sqrt(b * b - 4 * a * c)) / (2 * a);
        const double r2 = (-b - std::sqrt(b * b - 4 * a * c)) / (2 * a);
        cudaStream_t st = ctx().st;
        double *dt = upload(S_V1, pdt, N);
        const double *dp = upload(S_V2, pdp, N), *ddr = upload(S_V3, pddr, N), *ddq = upload(S_V4, pddq, N);
        double *part = dbuf<double>(S_RED, 2 * kRedBlocks);
        quad_gamma_kernel<<<kRedBlocks, 256, 0, st>>>(dt, dp, ddr, ddq, r1, r2, part, N);
        DI_CUDA(cudaGetLastError());
        std::vector<double> h(2 * kRedBlocks);
        download(h.data(), part, 2 * kRedBlocks);
        sync();
        double g1 = 0, g2 = 0;
        for (int i = 0; i < kRedBlocks; ++i) {
            g1 += h[2 * i];
            g2 += h[2 * i + 1];
        }
        double root;
        if (g1 > g2 && g1 > 0) root = r1;
        else if (g2 > g1 && g2 > 0) root = r2;
        else return 3;  // arc.c:131-135
        double *dd = dbuf<double>(S_V5, N);
        quad_apply_kernel<<<nb(N), kT, 0, st>>>(dt, dp, ddr, ddq, dd, root, N);
        DI_CUDA(cudaGetLastError());
        download(pdt, dt, N);
        download(pdd, dd, N);
        sync();
        *pdlpf = root;
        *plpft += root;
        return 0;
    } catch (const std::exception &e) {
        report("quad", e);
        return 4;
    }
}

int test(double *pd_temp, double *pdd, double *pf_temp, double *pfp, double *pqtot, double *pf_ip,
         double *pintener1, int *pconvchk, double *ptoldisp, double *ptolfor, double *ptolener)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        const Sizes z = sizes();
        const long N = z.neq;
        cudaStream_t st = ctx().st;
        const double *dtp = upload(S_V1, pd_temp, N), *dd = upload(S_V2, pdd, N), *f = upload(S_V3, pf_temp, N);
        const double *fp = upload(S_V4, pfp, N), *q = upload(S_V5, pqtot, N), *fip = upload(S_V6, pf_ip, N);
        double *part = dbuf<double>(S_RED, 5 * kRedBlocks);
        test_sums_kernel<<<kRedBlocks, 128, 0, st>>>(dtp, dd, f, fp, q, fip, part, N);
        DI_CUDA(cudaGetLastError());
        std::vector<double> h(5 * kRedBlocks);
        download(h.data(), part, 5 * kRedBlocks);
        sync();
        double s[5] = {0, 0, 0, 0, 0};
        for (int k = 0; k < 5; ++k)
            for (int i = 0; i < kRedBlocks; ++i) s[k] += h[k * kRedBlocks + i];
        *pconvchk = 0;
        if (*ptoldisp < 1) {
            if (s[1] == 0) {
                std::fprintf(stderr, "\n***ERROR*** Zero total displacement in convergence test\n");
                return 1;
            }
            if (std::sqrt(s[0]) / std::sqrt(s[1]) > *ptoldisp) *pconvchk += 10;
        }
        if (*ptolfor < 1) {
            if (s[3] == 0) {
                std::fprintf(stderr, "\n***ERROR*** Zero unbalanced force in convergence test\n");
                return 1;
            }
            if (std::sqrt(s[2]) / std::sqrt(s[3]) > *ptolfor) *pconvchk += 100;
        }
        if (*ptolener < 1) {
            if (*pintener1 == 0) {
                std::fprintf(stderr, "\n***ERROR*** Zero internal energy in convergence test\n");
                return 1;
            }
            if (std::fabs(s[4] / *pintener1) > *ptolener) *pconvchk += 1000;
        }
        return 0;
    } catch (const std::exception &e) {
        report("test", e);
        return 1;
    }
}

double dot(double *pa, double *pb, int n)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        if (n <= 0) return 0.0;
        const double *a = upload(S_V1, pa, n), *b = upload(S_V2, pb, n);
        double *part = dbuf<double>(S_RED, kRedBlocks);
        dot_partial_kernel<<<kRedBlocks, 256, 0, ctx().st>>>(a, b, part, n);
        DI_CUDA(cudaGetLastError());
        return device_sum(part, kRedBlocks);
    } catch (const std::exception &e) {
        report("dot", e);
        return NAN;
    }
}

}  // extern "C"
