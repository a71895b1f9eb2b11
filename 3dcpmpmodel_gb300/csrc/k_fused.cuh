// k_fused.cuh -- the FUSED scheme.
//
// Storage (one in-place A-A lattice):
//   f0[2][N]  FP32 rest population, double-buffered by step parity;
//   h[18][N]  moving populations q = 1..18 as S (half / bfloat16 / float),
//             each stored as a deviation from rest equilibrium of the node
//             that collided it:  h = f_q / w_q - a / w_0,  a = that node's
//             post-collision f_0.
// The anchor a of the population read from direction q at node x is the
// f_0 of its source x - e_q, or of x itself when the source is solid (the
// value is then x's own bounced-back population).  Anchoring on the writer's
// own rest population keeps |h| at the scale of rho*u, so the 11-bit FP16
// mantissa resolves the velocity part of the populations in both phases of
// a 145:1 density ratio.
//
// A-A addressing (parity P = step % 2):
//   P = 0: read  h[q][x];                          write h[opp q][x]
//   P = 1: read  h[opp q][x - e_q]  (h[q][x] if x - e_q solid);
//          write h[q][x + e_q]      (h[opp q][x] if x + e_q solid)
// Each node reads and writes the same slots, so the update is in place.
// Readers use f0[P]; writers write f0[1-P].
//
// Per step: wall pass(es) -> fused collide (2.5-D x-march) -> density pass.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lbm_core.cuh"
#include "launch.h"

namespace cpmp {

template <class S>
__device__ __forceinline__ float s2f(S v);
template <>
__device__ __forceinline__ float s2f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float s2f<__half>(__half v) { return __half2float(v); }
template <>
__device__ __forceinline__ float s2f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <class S>
__device__ __forceinline__ S f2s(float v);
template <>
__device__ __forceinline__ float f2s<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half f2s<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 f2s<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

__device__ __forceinline__ int wrap1(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// w_q / w_0 and 1 / w_q
__host__ __device__ __forceinline__ constexpr float ratio0(int q) { return q <= 6 ? 1.0f / 6.0f : 1.0f / 12.0f; }
__host__ __device__ __forceinline__ constexpr float inv_w(int q) { return q <= 6 ? 18.0f : 36.0f; }

// Post-stream populations of node (i,j,k) at parity P.
template <class S>
__device__ __forceinline__ void gather_pops(const KParams<float> &p, int P, const S *__restrict__ h,
                                            const float *__restrict__ f0, int i, int j, int k,
                                            long long I, float f[Q])
{
    const long long n = p.n;
    const float a0 = f0[I];
    f[0] = a0;
#pragma unroll
    for (int q = 1; q < Q; ++q) {
        const int si = wrap1(i - cx(q), p.dx), sj = wrap1(j - cy(q), p.dy), sk = wrap1(k - cz(q), p.dz);
        const bool ss = solid_k(p.wall_mode, sk, p.dz);
        const long long src = ((long long)si * p.dy + sj) * p.dz + sk;
        const float a = ss ? a0 : __ldg(f0 + src);
        float hv;
        if (P == 0)
            hv = s2f<S>(h[(long long)(q - 1) * n + I]);
        else
            hv = s2f<S>(ss ? h[(long long)(q - 1) * n + I] : h[(long long)(opp(q) - 1) * n + src]);
        f[q] = wgt<float>(q) * hv + ratio0(q) * a;
    }
}

// Store post-collision populations of node (i,j,k) at parity P.
template <class S>
__device__ __forceinline__ void scatter_pops(const KParams<float> &p, int P, S *__restrict__ h,
                                             float *__restrict__ f0n, int i, int j, int k, long long I,
                                             const float f[Q])
{
    const long long n = p.n;
    const float a = f[0];
    f0n[I] = a;
#pragma unroll
    for (int q = 1; q < Q; ++q) {
        const S hv = f2s<S>((f[q] - ratio0(q) * a) * inv_w(q));
        if (P == 0) {
            h[(long long)(opp(q) - 1) * n + I] = hv;
        } else {
            const int di = wrap1(i + cx(q), p.dx), dj = wrap1(j + cy(q), p.dy), dk = wrap1(k + cz(q), p.dz);
            if (solid_k(p.wall_mode, dk, p.dz))
                h[(long long)(opp(q) - 1) * n + I] = hv;
            else
                h[(long long)(q - 1) * n + ((long long)di * p.dy + dj) * p.dz + dk] = hv;
        }
    }
}

// ------------------------------------------------------------ density ----
// rho = sum of the post-stream populations (MacroCalculate's density,
// FluidCuda.cu:357-361) on fluid nodes.
template <class S>
__global__ void __launch_bounds__(256) k_density(KParams<float> p, int P, const S *__restrict__ h,
                                                 const float *__restrict__ f0, float *__restrict__ rho)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    const int k = (int)(I % p.dz);
    if (solid_k(p.wall_mode, k, p.dz)) return;
    const int j = (int)((I / p.dz) % p.dy), i = (int)(I / p.dz / p.dy);
    float f[Q];
    gather_pops<S>(p, P, h, f0, i, j, k, I, f);
    float r = 0.f;
#pragma unroll
    for (int q = 0; q < Q; ++q) r += f[q];
    rho[I] = r;
}

// --------------------------------------------------------- fused step ----
__device__ __forceinline__ int ring_slot(int x, int nr) { return ((x % nr) + nr) % nr; }

// One CTA owns a TY x TZ column tile of (y, z) and marches over XL planes of
// x.  Rings of shared-memory planes:
//   rho: planes p-3 .. p+3+L with a (3+L)-deep y/z halo (L = 2 for the
//        five-point Laplacian, 3 for the seven-point one);
//   mu : planes p-3 .. p+3 with a 3-deep halo.
// For output plane p the CTA loads rho(p+3+L), evaluates mu(p+3) (EOS +
// Laplacian, wall potential on solid nodes), then for every fluid node of
// plane p: F = -rho grad7(mu) + grad7(rho)/3, gathers the populations,
// collides (MRT + exact-difference forcing) and streams A-A in place.
template <class S, int TY, int TZ, int L>
__global__ void __launch_bounds__(TY *TZ, 1)
    k_fused_collide(KParams<float> p, int P, S *__restrict__ h, const float *__restrict__ f0c,
                    float *__restrict__ f0n, const float *__restrict__ rho, int xl)
{
    constexpr int RH = 3 + L;
    constexpr int RY = TY + 2 * RH, RZ = TZ + 2 * RH;
    constexpr int NR = 7 + L;
    constexpr int MY = TY + 6, MZ = TZ + 6;
    constexpr int NT = TY * TZ;
    extern __shared__ float sm[];
    float *srho = sm;
    float *smu = sm + NR * RY * RZ;

    const int tz = threadIdx.x % TZ, ty = threadIdx.x / TZ;
    const int z0 = blockIdx.x * TZ, y0 = blockIdx.y * TY;
    const int x0 = blockIdx.z * xl;
    const int x1 = min(x0 + xl, p.dx);

    auto load_rho = [&](int xlog) {
        const int gx = wrapm(xlog, p.dx);
        float *dst = srho + ring_slot(xlog, NR) * (RY * RZ);
        const long long base = (long long)gx * p.dy;
        for (int e = threadIdx.x; e < RY * RZ; e += NT) {
            const int ly = e / RZ, lz = e - ly * RZ;
            const int gy = wrapm(y0 - RH + ly, p.dy), gz = wrapm(z0 - RH + lz, p.dz);
            dst[e] = __ldg(rho + (base + gy) * p.dz + gz);
        }
    };
    auto comp_mu = [&](int xlog) {
        const int gx = wrapm(xlog, p.dx);
        float *dst = smu + ring_slot(xlog, 7) * (MY * MZ);
        const float *rc = srho + ring_slot(xlog, NR) * (RY * RZ);
        const float *rm1 = srho + ring_slot(xlog - 1, NR) * (RY * RZ);
        const float *rp1 = srho + ring_slot(xlog + 1, NR) * (RY * RZ);
        const float *rm2 = srho + ring_slot(xlog - 2, NR) * (RY * RZ);
        const float *rp2 = srho + ring_slot(xlog + 2, NR) * (RY * RZ);
        for (int e = threadIdx.x; e < MY * MZ; e += NT) {
            const int my = e / MZ, mz = e - my * MZ;
            const int gz = wrapm(z0 - 3 + mz, p.dz);
            if (solid_k(p.wall_mode, gz, p.dz)) {
                const int gy = wrapm(y0 - 3 + my, p.dy);
                dst[e] = p.wall[(gz < 3 ? 0 : (long long)p.dx * p.dy) + (long long)gx * p.dy + gy];
                continue;
            }
            const int c = (my + L) * RZ + (mz + L);
            const float r0 = rc[c];
            float lap;
            if (L == 2) {
                lap = (-r0 * 90.f + (-rm2[c] + rm1[c] * 16.f + rp1[c] * 16.f - rp2[c]) +
                       (-rc[c - 2 * RZ] + rc[c - RZ] * 16.f + rc[c + RZ] * 16.f - rc[c + 2 * RZ]) +
                       (-rc[c - 2] + rc[c - 1] * 16.f + rc[c + 1] * 16.f - rc[c + 2])) /
                      12.f;
            } else {
                const float *rm3 = srho + ring_slot(xlog - 3, NR) * (RY * RZ);
                const float *rp3 = srho + ring_slot(xlog + 3, NR) * (RY * RZ);
                lap = (-r0 * 1470.f +
                       (2.f * rm3[c] - 27.f * rm2[c] + 270.f * rm1[c] + 270.f * rp1[c] - 27.f * rp2[c] + 2.f * rp3[c]) +
                       (2.f * rc[c - 3 * RZ] - 27.f * rc[c - 2 * RZ] + 270.f * rc[c - RZ] + 270.f * rc[c + RZ] -
                        27.f * rc[c + 2 * RZ] + 2.f * rc[c + 3 * RZ]) +
                       (2.f * rc[c - 3] - 27.f * rc[c - 2] + 270.f * rc[c - 1] + 270.f * rc[c + 1] -
                        27.f * rc[c + 2] + 2.f * rc[c + 3])) /
                      180.f;
            }
            dst[e] = p.kk * mu0<float>(p.eos, p.A, p.B, p.T, r0) - p.ka * lap;
        }
    };

    // prologue: mu(x0-3 .. x0+2)
    for (int x = x0 - 3 - L; x <= x0 - 3 + L; ++x) load_rho(x);
    __syncthreads();
    comp_mu(x0 - 3);
    __syncthreads();
    for (int x = x0 - 2; x <= x0 + 2; ++x) {
        load_rho(x + L);
        __syncthreads();
        comp_mu(x);
        __syncthreads();
    }

    const int gy = y0 + ty, gz = z0 + tz;
    const bool active = gy < p.dy && gz < p.dz && !solid_k(p.wall_mode, gz, p.dz);
    for (int x = x0; x < x1; ++x) {
        load_rho(x + 3 + L);
        __syncthreads();
        comp_mu(x + 3);
        __syncthreads();
        if (active) {
            // gradients from the rings
            float gm[3] = {0.f, 0.f, 0.f}, gr[3] = {0.f, 0.f, 0.f};
            const float *mpl[7], *rpl[7];
#pragma unroll
            for (int d = -3; d <= 3; ++d) {
                mpl[d + 3] = smu + ring_slot(x + d, 7) * (MY * MZ);
                rpl[d + 3] = srho + ring_slot(x + d, NR) * (RY * RZ);
            }
            const int mc = (ty + 3) * MZ + (tz + 3);
            const int rcn = (ty + RH) * RZ + (tz + RH);
            // first difference along line s at distance d: c_d (v(+d) - v(-d))
            auto line = [&](int sx, int sy, int sz, float &om, float &orr) {
                float am = 0.f, ar = 0.f;
#pragma unroll
                for (int d = 1; d <= 3; ++d) {
                    const float c = d == 1 ? 45.f : (d == 2 ? -9.f : 1.f);
                    const int mo = sy * d * MZ + sz * d, ro = sy * d * RZ + sz * d;
                    am += c * (mpl[3 + sx * d][mc + mo] - mpl[3 - sx * d][mc - mo]);
                    ar += c * (rpl[3 + sx * d][rcn + ro] - rpl[3 - sx * d][rcn - ro]);
                }
                om = am;
                orr = ar;
            };
            float lm, lr;
            line(1, 0, 0, lm, lr); gm[0] += 2.f * lm; gr[0] += 2.f * lr;
            line(0, 1, 0, lm, lr); gm[1] += 2.f * lm; gr[1] += 2.f * lr;
            line(0, 0, 1, lm, lr); gm[2] += 2.f * lm; gr[2] += 2.f * lr;
            line(1, 1, 0, lm, lr); gm[0] += lm; gm[1] += lm; gr[0] += lr; gr[1] += lr;
            line(1, -1, 0, lm, lr); gm[0] += lm; gm[1] -= lm; gr[0] += lr; gr[1] -= lr;
            line(1, 0, 1, lm, lr); gm[0] += lm; gm[2] += lm; gr[0] += lr; gr[2] += lr;
            line(1, 0, -1, lm, lr); gm[0] += lm; gm[2] -= lm; gr[0] += lr; gr[2] -= lr;
            line(0, 1, 1, lm, lr); gm[1] += lm; gm[2] += lm; gr[1] += lr; gr[2] += lr;
            line(0, 1, -1, lm, lr); gm[1] += lm; gm[2] -= lm; gr[1] += lr; gr[2] -= lr;
            const float inv360 = 1.0f / 360.0f;
            const float r = rpl[3][rcn];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                gm[a] *= inv360;
                gr[a] *= inv360;
            }
            const float Fx = -gm[0] * r + gr[0] * (1.0f / 3.0f);
            const float Fy = -gm[1] * r + gr[1] * (1.0f / 3.0f);
            const float Fz = -gm[2] * r + gr[2] * (1.0f / 3.0f);

            const int gxw = wrapm(x, p.dx);
            const long long I = ((long long)gxw * p.dy + gy) * p.dz + gz;
            float f[Q];
            gather_pops<S>(p, P, h, f0c, gxw, gy, gz, I, f);
            const float ir = 1.0f / r;
            const float ux = (f[1] + f[7] + f[9] + f[11] + f[13] - f[2] - f[8] - f[10] - f[12] - f[14]) * ir;
            const float uy = (f[3] + f[7] + f[8] + f[15] + f[17] - f[4] - f[9] - f[10] - f[16] - f[18]) * ir;
            const float uz = (f[5] + f[11] + f[12] + f[15] + f[16] - f[6] - f[13] - f[14] - f[17] - f[18]) * ir;
            float qp[Q];
            const float *qpp = nullptr;
            if (p.qp) {
#pragma unroll
                for (int a = 0; a < Q; ++a) qp[a] = 0.f;
                qp[1] = -19.f * (p.k1 + 3.f * p.k2) * (gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
                qp[9] = -p.k1 * (2.f * gr[0] * gr[0] - gr[1] * gr[1] - gr[2] * gr[2]);
                qp[11] = -p.k1 * (gr[1] * gr[1] - gr[2] * gr[2]);
                qp[13] = -p.k1 * gr[0] * gr[1];
                qp[14] = -p.k1 * gr[2] * gr[1];
                qp[15] = -p.k1 * gr[0] * gr[2];
                qpp = qp;
            }
            collide_mrt_edm<float>(f, r, ux, uy, uz, Fx, Fy, Fz, p.ts, qpp);
            scatter_pops<S>(p, P, h, f0n, gxw, gy, gz, I, f);
        }
        __syncthreads();
    }
}

template <int TY, int TZ, int L>
constexpr size_t fused_smem_bytes()
{
    return sizeof(float) * ((size_t)(7 + L) * (TY + 2 * (3 + L)) * (TZ + 2 * (3 + L)) + (size_t)7 * (TY + 6) * (TZ + 6));
}

// ------------------------------------------------------------ init etc ----
// Pass 1 of the FUSED initial state: tags, density, rest population.
__global__ void k_init_fused_a(KParams<float> p, DropletDev d, uint8_t *type, float *rho, float *f0);
// Pass 2: moving populations f_q = w_q rho, anchored on the sources' f0.
template <class S>
__global__ void k_init_fused_b(KParams<float> p, const float *rho, const float *f0, S *h)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    const int k = (int)(I % p.dz), j = (int)((I / p.dz) % p.dy), i = (int)(I / p.dz / p.dy);
    if (solid_k(p.wall_mode, k, p.dz)) return;
    const float rx = rho[I];
    for (int q = 1; q < Q; ++q) {
        const int si = wrap1(i - cx(q), p.dx), sj = wrap1(j - cy(q), p.dy), sk = wrap1(k - cz(q), p.dz);
        const bool ss = solid_k(p.wall_mode, sk, p.dz);
        const long long src = ((long long)si * p.dy + sj) * p.dz + sk;
        const float a = ss ? f0[I] : f0[src];
        const float fq = wgt<float>(q) * rx;
        h[(long long)(q - 1) * p.n + I] = f2s<S>((fq - ratio0(q) * a) * inv_w(q));
    }
}

}  // namespace cpmp
