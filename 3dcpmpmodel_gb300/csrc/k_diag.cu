// k_diag.cu -- device diagnostics: FP64 mass / max-speed / non-finite
// reduction (CalcMacroCPU, FluidCuda.cu:1626-1657), the contact angle of the
// x-z slice (ContactAngle, FluidCuda.cu:557-734) and the Laplace-law probe
// (SaveDataOriDen, FluidCuda.cu:1159-1199).  All reductions are warp-shuffle
// then shared memory, in a fixed order, so results are run-to-run identical.
#include <cfloat>
#include <climits>
#include <cstdint>
#include <mutex>
#include <string>

#include "cpmp.h"
#include "kernels.h"

namespace cpmp {

namespace {
constexpr int kRedThreads = 256;
constexpr int kMaxRedBlocks = 1024;
// Blocks of a reduction over a large box: 6 on each of the 152 SMs (48 warps
// per SM), so that every SM gets the same share of a grid-stride pass.
constexpr int kRedBlocks = 912;
static_assert(kRedBlocks <= kMaxRedBlocks, "partial arrays hold kMaxRedBlocks triples");

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_or(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_min_i(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max_i(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
}  // namespace

int diag_partial_blocks(long long n)
{
    long long b = (n + kRedThreads - 1) / kRedThreads;
    if (b > kRedBlocks) b = kRedBlocks;
    if (b < 1) b = 1;
    return (int)b;
}

namespace {
// vec flags of k_mass_partial: bit 0 when n is a multiple of 4 with type
// 4-byte and rho 16-byte aligned, bit 1 when MV is 16-byte aligned as well.
int mass_vec_flags(const void *type, const void *rho, const void *mv, long long n)
{
    if (n % 4 != 0 || (reinterpret_cast<uintptr_t>(type) & 3) || (reinterpret_cast<uintptr_t>(rho) & 15)) return 0;
    return 1 | ((mv && !(reinterpret_cast<uintptr_t>(mv) & 15)) ? 2 : 0);
}
}  // namespace

// Running sums of one thread of the mass pass.  FP32 fields: the sum is an
// exact FP32 pair (TwoSum: hi + lo equals the sum of the values added, up to
// the rounding of lo), so the FP64 pipe -- a small fraction of the FP32 rate
// on this part -- only joins the threads' partials; the sign test and |MV|^2
// stay in FP32 as the fields are.  FP64 fields: plain FP64 sums.
template <class R>
struct MassAcc {
    double s = 0.0, m2 = 0.0;
    int bad = 0;
    __device__ __forceinline__ void add(double d)
    {
        if (!(d >= 0.0)) bad = 1;  // NaN or negative (FluidCuda.cu:1632)
        s += d;
    }
    __device__ __forceinline__ void speed(double a, double b, double c) { m2 = fmax(m2, a * a + b * b + c * c); }
    __device__ __forceinline__ double sum() const { return s; }
    __device__ __forceinline__ double max2() const { return m2; }
};
template <>
struct MassAcc<float> {
    float hi = 0.f, lo = 0.f, m2 = 0.f;
    int bad = 0;
    __device__ __forceinline__ void add(float d)
    {
        if (!(d >= 0.f)) bad = 1;  // NaN or negative (FluidCuda.cu:1632)
        const float t = hi + d, bp = t - hi;
        lo += (hi - (t - bp)) + (d - bp);
        hi = t;
    }
    __device__ __forceinline__ void speed(float a, float b, float c) { m2 = fmaxf(m2, fmaf(a, a, fmaf(b, b, c * c))); }
    __device__ __forceinline__ double sum() const { return (double)hi + (double)lo; }
    __device__ __forceinline__ double max2() const { return (double)m2; }
};

// Four consecutive values of a field starting at node 4g (16-byte aligned).
__device__ __forceinline__ void load4(const float *__restrict__ p, long long g, float (&v)[4])
{
    const float4 t = reinterpret_cast<const float4 *>(p)[g];
    v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
}
__device__ __forceinline__ void load4(const double *__restrict__ p, long long g, double (&v)[4])
{
    const double2 a = reinterpret_cast<const double2 *>(p)[2 * g], b = reinterpret_cast<const double2 *>(p)[2 * g + 1];
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
}

// Adds the fluid nodes of group g (nodes 4g .. 4g+3) in node order.
template <class R>
__device__ __forceinline__ void mass_group(MassAcc<R> &acc, const uint8_t *__restrict__ type,
                                           const R *__restrict__ rho, const R *__restrict__ mv, long long n,
                                           long long g, int vec)
{
    const uchar4 t4 = reinterpret_cast<const uchar4 *>(type)[g];
    const uint8_t t[4] = {t4.x, t4.y, t4.z, t4.w};
    R d[4];
    load4(rho, g, d);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (t[k] == FLUID) acc.add(d[k]);
    if (mv) {
        R a[4], b[4], c[4];
        if (vec & 2) {
            load4(mv, g, a);
            load4(mv + n, g, b);
            load4(mv + 2 * n, g, c);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) a[k] = mv[4 * g + k], b[k] = mv[n + 4 * g + k], c[k] = mv[2 * n + 4 * g + k];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (t[k] == FLUID) acc.speed(a[k], b[k], c[k]);
    }
}

// Per-block partial (sum of rho, max |MV|^2, non-finite flag) over the fluid
// nodes.  With vec bit 0 set (n a multiple of 4, type 4-byte and rho 16-byte
// aligned) each thread takes groups of four nodes -- one 4-byte type load and
// 16-byte field loads -- two groups per loop trip, both loaded before either
// is added, so that every warp keeps two groups of loads in flight; bit 1
// says MV is 16-byte aligned too.  The order in which a thread adds its
// nodes does not depend on MV, so the mass is the same with or without it.
// One block of the pass: thread tid of `stride` threads; the block's triple
// goes to part[0..2].
template <class R>
__device__ __forceinline__ void mass_partial_block(const uint8_t *__restrict__ type, const R *__restrict__ rho,
                                                   const R *__restrict__ mv, long long n, int vec, long long tid,
                                                   long long stride, double *__restrict__ part)
{
    MassAcc<R> acc;
    long long first = 0;  // first node of the scalar loop
    if (vec & 1) {
        const long long ng = n >> 2;
        first = ng << 2;
        long long g = tid;
        for (; g + stride < ng; g += 2 * stride) {
            mass_group(acc, type, rho, mv, n, g, vec);
            mass_group(acc, type, rho, mv, n, g + stride, vec);
        }
        if (g < ng) mass_group(acc, type, rho, mv, n, g, vec);
    }
    for (long long I = first + tid; I < n; I += stride) {
        if (type[I] != FLUID) continue;
        acc.add(rho[I]);
        if (mv) acc.speed(mv[I], mv[I + n], mv[I + 2 * n]);
    }
    double s = acc.sum(), mx = acc.max2();
    int bad = acc.bad;
    __shared__ double ss[kRedThreads / 32], sm[kRedThreads / 32];
    __shared__ int sb[kRedThreads / 32];
    s = warp_sum(s);
    mx = warp_max(mx);
    bad = warp_or(bad);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        ss[w] = s;
        sm[w] = mx;
        sb[w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ts = 0.0, tm = 0.0;
        int tb = 0;
        for (int k = 0; k < kRedThreads / 32; ++k) {
            ts += ss[k];
            tm = fmax(tm, sm[k]);
            tb |= sb[k];
        }
        part[0] = ts;
        part[1] = tm;
        part[2] = (double)tb;
    }
}

// FP32 fields: at most 40 registers, so that the 6 blocks per SM of a large
// box are resident together (FP64 fields: 64, 4 blocks).
template <class R>
__global__ void __launch_bounds__(kRedThreads, sizeof(R) == 4 ? kRedBlocks / 152 : 4)
    k_mass_partial(const uint8_t *__restrict__ type, const R *__restrict__ rho, const R *__restrict__ mv,
                   long long n, int vec, double *__restrict__ part)
{
    mass_partial_block<R>(type, rho, mv, n, vec, (long long)blockIdx.x * kRedThreads + threadIdx.x,
                          (long long)gridDim.x * kRedThreads, part + 3 * blockIdx.x);
}

// Joins nb partial triples (one block of kRedThreads threads).
__device__ __forceinline__ void mass_final_block(const double *__restrict__ part, int nb, double *__restrict__ out,
                                                 int take_sqrt)
{
    __shared__ double ss[kRedThreads], sm[kRedThreads], sb[kRedThreads];
    double s = 0.0, mx = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        s += part[3 * k];
        mx = fmax(mx, part[3 * k + 1]);
        b = fmax(b, part[3 * k + 2]);
    }
    ss[threadIdx.x] = s;
    sm[threadIdx.x] = mx;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int o = kRedThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
            sb[threadIdx.x] = fmax(sb[threadIdx.x], sb[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = ss[0];
        out[1] = take_sqrt ? sqrt(sm[0]) : sm[0];
        out[2] = sb[0];
    }
}

__global__ void __launch_bounds__(kRedThreads) k_mass_final(const double *__restrict__ part, int nb,
                                                           double *__restrict__ out, int take_sqrt)
{
    mass_final_block(part, nb, out, take_sqrt);
}

// ------------------------------------------------ droplet-impact sums ----
// ComputeEnergy (FluidCuda.cu:737-787) and Computetangential_velocity
// (:790-898): over fluid nodes with rho > mid in 2 <= i < DX-2,
// 2 <= j < DY-2, 2 <= k < DZ-2 -- sum |MV|, |MV_xy|, MVz, the same weighted
// by rho, the kinetic energies rho |MV|^2 / 2 (all, xy, z), and the
// velocity along the azimuth about (DX/2, DY/2) and its rho-weighted sum;
// SaveSpreadtime (:1128-1150): over every node with rho > mid and
// 2 <= k < DZ-2, the sums of rho |MV| and rho.  Per-block FP64 partials in a
// fixed order, then a fixed-order sum per quantity.
constexpr int kImpactQ = 13;
template <class R>
__global__ void __launch_bounds__(kRedThreads) k_impact_partial(const uint8_t *__restrict__ type,
                                                               const R *__restrict__ rho,
                                                               const R *__restrict__ mv, int dx, int dy, int dz,
                                                               double mid, double *__restrict__ part)
{
    const double PI = 3.14159265358979323846264338327950288;
    const long long n = (long long)dx * dy * dz;
    double acc[kImpactQ];
#pragma unroll
    for (int q = 0; q < kImpactQ; ++q) acc[q] = 0.0;
    for (long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x; I < n;
         I += (long long)gridDim.x * blockDim.x) {
        const double d = (double)rho[I];
        if (!(d > mid)) continue;
        const int k = (int)(I % dz), j = (int)((I / dz) % dy), i = (int)(I / ((long long)dz * dy));
        if (k < 2 || k >= dz - 2) continue;
        const double a = (double)mv[I], b = (double)mv[I + n], c = (double)mv[I + 2 * n];
        const double s2 = a * a + b * b, s3 = s2 + c * c;
        acc[11] += d * sqrt(s3);
        acc[12] += d;
        if (type[I] != FLUID || i < 2 || i >= dx - 2 || j < 2 || j >= dy - 2) continue;
        const double v3 = sqrt(s3), v2 = sqrt(s2);
        acc[0] += v3;
        acc[1] += v2;
        acc[2] += c;
        acc[3] += d * v3;
        acc[4] += d * v2;
        acc[5] += d * c;
        acc[6] += d * s3 / 2;
        acc[7] += d * s2 / 2;
        acc[8] += d * (c * c) / 2;
        double al = atan2((double)(j - dy / 2), (double)(i - dx / 2)) / PI * 180;
        if (al < 0) al = al + 360;
        al = al / 180 * PI;
        const double t = a * sin(al) + b * cos(al);
        acc[9] += t;
        acc[10] += t * d;
    }
    __shared__ double sw[kRedThreads / 32][kImpactQ];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < kImpactQ; ++q) {
        const double v = warp_sum(acc[q]);
        if (l == 0) sw[w][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < kImpactQ) {
        double v = 0.0;
        for (int ww = 0; ww < kRedThreads / 32; ++ww) v += sw[ww][threadIdx.x];
        part[(long long)blockIdx.x * kImpactQ + threadIdx.x] = v;
    }
}

__global__ void k_impact_final(const double *__restrict__ part, int nb, double *__restrict__ out)
{
    const int q = threadIdx.x;
    if (q >= kImpactQ) return;
    double v = 0.0;
    for (int b = 0; b < nb; ++b) v += part[(long long)b * kImpactQ + q];
    out[q] = v;
}

template <class R>
void diag_launch_impact(const uint8_t *type, const R *rho, const R *mv, int dx, int dy, int dz, double mid,
                        double *partials, double *out, cudaStream_t st)
{
    const int nb = diag_partial_blocks((long long)dx * dy * dz);
    k_impact_partial<R><<<nb, kRedThreads, 0, st>>>(type, rho, mv, dx, dy, dz, mid, partials);
    k_impact_final<<<1, 32, 0, st>>>(partials, nb, out);
}
int diag_impact_quantities() { return kImpactQ; }

template <class R>
void diag_launch_mass(const uint8_t *type, const R *rho, const R *mv, long long n, double *partials,
                      double *out, cudaStream_t st)
{
    const int nb = diag_partial_blocks(n);
    k_mass_partial<R><<<nb, kRedThreads, 0, st>>>(type, rho, mv, n, mass_vec_flags(type, rho, mv, n), partials);
    k_mass_final<<<1, kRedThreads, 0, st>>>(partials, nb, out, 0);
}

// --------------------------------------------------------- contact angle ----
// One block.  Warp w < 8 searches row k = 2 + w/2 for the left (w even) or
// right (w odd) mid-density crossing; the reference scans left-to-right
// (right-to-left) and stops at the first hit, i.e. the minimum (maximum)
// index satisfying the crossing test, found here by a warp min (max).
// Warp 8 then finds the top of the cap on the centre column (the reference
// keeps the last hit, the maximum k).  Thread 0 does the extrapolation and
// angle arithmetic in FP64 exactly as the reference.
template <class R>
__device__ __forceinline__ void contact_angle_block(const R *__restrict__ rho, int dx, int dy, int dz, int tier,
                                                    double mid, double *__restrict__ out)
{
    __shared__ double px[8];
    __shared__ int ic_s;
    __shared__ double H_s;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    auto T = [&](int i, int k) -> double { return (double)rho[((long long)i * dy + tier) * dz + k]; };
    if (w < 8) {
        const int row = 2 + w / 2;
        if ((w & 1) == 0) {
            int best = INT_MAX;
            for (int i = l; i < dx / 2 + 2; i += 32) {
                const double t1 = T(i + 1, row), t2 = T(i + 2, row);
                if (t1 < mid && t2 >= mid) best = min(best, i);
            }
            best = warp_min_i(best);
            if (l == 0) {
                double v = 0.0;
                if (best != INT_MAX) {
                    const double t1 = T(best + 1, row), t2 = T(best + 2, row);
                    v = (double)(best + 1) + (t1 - mid) / (t1 - t2);
                }
                px[w] = v;
            }
        } else {
            int best = INT_MIN;
            for (int i = dx - 2 - l; i > dx / 2 - 2; i -= 32) {
                const double t1 = T(i - 1, row), t2 = T(i - 2, row);
                if (t1 < mid && t2 >= mid) best = max(best, i);
            }
            best = warp_max_i(best);
            if (l == 0) {
                double v = 0.0;
                if (best != INT_MIN) {
                    const double t1 = T(best - 1, row), t2 = T(best - 2, row);
                    v = (double)(best - 1) - (t1 - mid) / (t1 - t2);
                }
                px[w] = v;
            }
        }
    }
    __syncthreads();
    const bool have = px[0] != 0.0 && px[1] != 0.0;
    if (threadIdx.x == 0) ic_s = (int)((px[4] + px[5]) / 2 + 0.5);
    __syncthreads();
    if (w == 8) {
        int best = INT_MIN;
        const int ic = ic_s;
        if (have && ic >= 0 && ic < dx) {
            for (int k = 2 + l; k < dz - 2; k += 32) {
                const double t = T(ic, k), t1 = T(ic, k + 1);
                if (t >= mid && t1 < mid) best = max(best, k);
            }
        }
        best = warp_max_i(best);
        if (l == 0) {
            double H = 0.0;
            if (best != INT_MIN) {
                const double t = T(ic, best), t1 = T(ic, best + 1);
                H = (double)best + (t - mid) / (t - t1) - 2.0;
            }
            H_s = H;
        }
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double PI = 3.14159265358979323846264338327950288;
    const double y0 = 2, y1 = 3, y2 = 4;
    double xl, xr, cl, cr, cap = 0.0, H = 0.0, L = 0.0;
    if (have) {
        xl = px[2] * ((y0 - y2) / (y1 - y2)) + px[4] * ((y0 - y1) / (y2 - y1));
        xr = px[3] * ((y0 - y2) / (y1 - y2)) + px[5] * ((y0 - y1) / (y2 - y1));
        double ca = atan((y1 - y0) / (px[2] - xl));
        if (ca < 0) ca += PI;
        cl = ca / PI * 180;
        ca = atan(-(y1 - y0) / (px[3] - xr));
        if (ca < 0) ca += PI;
        cr = ca / PI * 180;
        L = xr - xl;
        H = H_s;
        if (L <= 0) {
            L = px[3] - px[2];
            H = H - 0.5;
        }
        if (xl > dy / 2 && xr < dy / 2) {
            xl = dy / 2;
            xr = dy / 2;
        }
        const double Rr = (H * H * 4 + L * L) / H / 8;
        cap = atan(L / (Rr - H) / 2);
        if (cap < 0) cap += PI;
        cap = cap / PI * 180;
    } else {
        xl = xr = dy / 2;
        cl = cr = 0;
    }
    out[0] = cl;
    out[1] = cr;
    out[2] = cap;
    out[3] = xl;
    out[4] = xr;
    out[5] = H;
    out[6] = L;
}

template <class R>
__global__ void __launch_bounds__(288) k_contact_angle(const R *__restrict__ rho, int dx, int dy, int dz, int tier,
                                                       double mid, double *__restrict__ out)
{
    contact_angle_block<R>(rho, dx, dy, dz, tier, mid, out);
}

template <class R>
void diag_launch_contact_angle(const R *rho, int dx, int dy, int dz, int tier, double den_g,
                               double den_l, double *out, cudaStream_t st)
{
    k_contact_angle<R><<<1, 288, 0, st>>>(rho, dx, dy, dz, tier, (den_g + den_l) / 2, out);
}

// ------------------------------------------------------------ Laplace ----
__device__ double eos_pressure(int eos, double A, double B, double T, double r)
{
    if (eos == 1) return T * r / (1.0 - B * r) - A * r * r;
    if (eos == 2) {
        const double e = B * r, om = 1.0 - e;
        return r * T * (1 + e + e * e - e * e * e) / (om * om * om) - A * r * r;
    }
    if (eos == 3) return T * r / (1.0 - B * r) - A * r * r / (1.0 + B * r);
    return T * r / (1.0 - B * r) - A * r * r / (1.0 + B * r * 2 - (B * r) * (B * r));
}

template <class R>
__device__ __forceinline__ void laplace_warp(const R *__restrict__ rho, int dx, int dy, int dz, int eos, double A,
                                             double B, double T, double kk, double *__restrict__ out)
{
    const int l = threadIdx.x;
    auto D = [&](int j) -> double { return (double)rho[((long long)(dx / 2) * dy + j) * dz + dz / 2]; };
    const double tout = D(0), tin = D(dy / 2);
    const double mid = (tout + tin) / 2;
    int best = INT_MAX;
    for (int j = l; j <= dy / 2 && j + 1 < dy; j += 32) {
        const double t1 = D(j), t2 = D(j + 1);
        if (t1 <= mid && t2 > mid) best = min(best, j);
    }
    best = warp_min_i(best);
    if (l != 0) return;
    double Rr = 0.0;
    if (best != INT_MAX) {
        const double t1 = D(best), t2 = D(best + 1);
        const double pos = (double)best + (mid - t1) / (t2 - t1);
        Rr = (double)(dy / 2) - pos;
    }
    const double dp = eos_pressure(eos, A, B, T, tin) - eos_pressure(eos, A, B, T, tout);
    out[0] = Rr;
    out[1] = dp;
    out[2] = kk * dp * Rr / 2;
}

template <class R>
__global__ void k_laplace(const R *__restrict__ rho, int dx, int dy, int dz, int eos, double A, double B, double T,
                          double kk, double *__restrict__ out)
{
    laplace_warp<R>(rho, dx, dy, dz, eos, A, B, T, kk, out);
}

template <class R>
void diag_launch_laplace(const R *rho, int dx, int dy, int dz, int eos, double A, double B, double T,
                         double kk, double *out, cudaStream_t st)
{
    k_laplace<R><<<1, 32, 0, st>>>(rho, dx, dy, dz, eos, A, B, T, kk, out);
}

// ------------------------------------------------ batched diagnostics ----
// The diagnostics of every box of a batch in four launches: the mass pass
// over a flattened grid (box b owns mass blocks blk0 .. blk0 + nb - 1, and
// each of them does what block (local index) of the box's own mass pass
// does, over the same threads and nodes), then one block per box for the
// join, the contact angle and the Laplace probe.  Every box's results are
// those of its own reduction, bit for bit.
__global__ void __launch_bounds__(kRedThreads, kRedBlocks / 152)
    k_mass_partial_batch(const DiagBox *__restrict__ boxes, int nbox, int par)
{
    const long long g = blockIdx.x;
    int lo = 0, hi = nbox - 1;
    while (lo < hi) {  // the last box whose first block is at most g
        const int mid = (lo + hi + 1) >> 1;
        if (boxes[mid].blk0 <= g) lo = mid;
        else hi = mid - 1;
    }
    const DiagBox &d = boxes[lo];
    const long long local = g - d.blk0;
    mass_partial_block<float>(d.type, d.rho[par], nullptr, d.n, d.vec, local * kRedThreads + threadIdx.x,
                              (long long)d.nb * kRedThreads, d.part + 3 * local);
}

__global__ void __launch_bounds__(kRedThreads) k_mass_final_batch(const DiagBox *__restrict__ boxes,
                                                                 double *__restrict__ out)
{
    const DiagBox &d = boxes[blockIdx.x];
    mass_final_block(d.part, d.nb, out + kDiagStride * blockIdx.x, 0);
}

__global__ void __launch_bounds__(288) k_contact_angle_batch(const DiagBox *__restrict__ boxes, int par,
                                                             double *__restrict__ out)
{
    const DiagBox &d = boxes[blockIdx.x];
    if (!d.angle) return;  // the whole block: a box too small for the slice search
    contact_angle_block<float>(d.rho[par], d.dx, d.dy, d.dz, d.tier, d.mid, out + kDiagStride * blockIdx.x + 4);
}

__global__ void __launch_bounds__(32) k_laplace_batch(const DiagBox *__restrict__ boxes, int par,
                                                      double *__restrict__ out)
{
    const DiagBox &d = boxes[blockIdx.x];
    laplace_warp<float>(d.rho[par], d.dx, d.dy, d.dz, d.eos, d.A, d.B, d.T, d.kk,
                        out + kDiagStride * blockIdx.x + 12);
}

void diag_launch_batch(const DiagBox *boxes, int nbox, long long mass_blocks, int par, double *out,
                       cudaStream_t st)
{
    k_mass_partial_batch<<<(unsigned)mass_blocks, kRedThreads, 0, st>>>(boxes, nbox, par);
    k_mass_final_batch<<<nbox, kRedThreads, 0, st>>>(boxes, out);
    k_contact_angle_batch<<<nbox, 288, 0, st>>>(boxes, par, out);
    k_laplace_batch<<<nbox, 32, 0, st>>>(boxes, par, out);
}

int diag_mass_vec_flags(const void *type, const void *rho, const void *mv, long long n)
{
    return mass_vec_flags(type, rho, mv, n);
}

__global__ void k_mv(const uint8_t *type, const float *rho, const float *u, const float *F, float *mv,
                     long long n)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= n || type[I] != FLUID) return;
    const float r = rho[I];
    for (int a = 0; a < 3; ++a) mv[I + a * n] = u[I + a * n] + F[I + a * n] / r * 0.5f;
}

void diag_launch_mv(const uint8_t *type, const float *rho, const float *u, const float *F, float *mv,
                    long long n, cudaStream_t st)
{
    k_mv<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(type, rho, u, F, mv, n);
}

// ------------------------------------------------- no-allocation variant ----
// Partials of cpmp_mass_noalloc live in this file-scope device array instead
// of a buffer the handle allocates.  Host code cannot use the array's name as
// an address (it is a host-side stand-in); the device address comes from
// cudaGetSymbolAddress with the device current, on the first call on a
// device (which has to come before any stream capture) and again on later
// calls (the lookup allocates nothing and follows the module if a device
// reset or a new primary context reloaded it at another address).  Each call
// writes every partial triple it later reads, so nothing has to be cleared
// between calls; calls that overlap on the GPU share the array and race.
static __device__ __align__(256) double g_noalloc_partials[3 * kMaxRedBlocks];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double *g_noalloc_addr[kMaxDevices] = {nullptr};

cudaError_t noalloc_partials(cudaStream_t st, double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(st, &cap)) != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        if ((e = cudaGetSymbolAddress(&p, g_noalloc_partials)) != cudaSuccess) return e;
        g_noalloc_addr[dev] = static_cast<double *>(p);
    } else if (!g_noalloc_addr[dev]) {
        return cudaErrorStreamCaptureUnsupported;
    }
    *out = g_noalloc_addr[dev];
    return cudaSuccess;
}
}  // namespace

}  // namespace cpmp

extern "C" cpmp_status cpmp_mass_noalloc(const uint8_t *type, const float *rho, const float *mv, long long n,
                                         void *stream, double *out)
{
    using namespace cpmp;
    if (!type || !rho || !out) {
        cpmp_internal_set_error("cpmp_mass_noalloc: null type, rho or out pointer");
        return CPMP_ERR_PARAM;
    }
    if (n < 1 || n > CPMP_NOALLOC_MAX_NODES) {
        cpmp_internal_set_error("cpmp_mass_noalloc: n must lie in [1, CPMP_NOALLOC_MAX_NODES = 2^34]");
        return CPMP_ERR_SIZE;
    }
    double *part = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = noalloc_partials(st, &part);
    if (e != cudaSuccess) {
        cpmp_internal_set_error((std::string("cpmp_mass_noalloc: cudaGetSymbolAddress: ") +
                                 cudaGetErrorString(e)).c_str());
        return CPMP_ERR_CUDA;
    }
    const int nb = diag_partial_blocks(n);  // <= the array's kMaxRedBlocks triples
    k_mass_partial<float><<<nb, kRedThreads, 0, st>>>(type, rho, mv, n, mass_vec_flags(type, rho, mv, n), part);
    k_mass_final<<<1, kRedThreads, 0, st>>>(part, nb, out, 1);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        cpmp_internal_set_error((std::string("cpmp_mass_noalloc: launch: ") + cudaGetErrorString(e)).c_str());
        return CPMP_ERR_CUDA;
    }
    return CPMP_OK;
}

namespace cpmp {

template void diag_launch_mass<float>(const uint8_t *, const float *, const float *, long long, double *, double *, cudaStream_t);
template void diag_launch_mass<double>(const uint8_t *, const double *, const double *, long long, double *, double *, cudaStream_t);
template void diag_launch_contact_angle<float>(const float *, int, int, int, int, double, double, double *, cudaStream_t);
template void diag_launch_contact_angle<double>(const double *, int, int, int, int, double, double, double *, cudaStream_t);
template void diag_launch_laplace<float>(const float *, int, int, int, int, double, double, double, double, double *, cudaStream_t);
template void diag_launch_laplace<double>(const double *, int, int, int, int, double, double, double, double, double *, cudaStream_t);
template void diag_launch_impact<float>(const uint8_t *, const float *, const float *, int, int, int, double, double *, double *, cudaStream_t);
template void diag_launch_impact<double>(const uint8_t *, const double *, const double *, int, int, int, double, double *, double *, cudaStream_t);

}  // namespace cpmp
