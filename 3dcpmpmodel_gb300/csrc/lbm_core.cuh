// lbm_core.cuh -- device building blocks shared by every step scheme:
// D3Q19 lattice, equation-of-state chemical potential, the factored MRT
// collision with exact-difference forcing, and the kernel parameter block.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace cpmp {

constexpr int Q = 19;
constexpr uint8_t FLUID = 1;  // reference Common.h:37
constexpr uint8_t SOLID = 2;  // reference Common.h:38

// D3Q19 velocities in the reference's order (Common.h:96-98); the opposite
// map is Re[] (Common.h:99) and the weights Alpha[] (Common.h:100).
__host__ __device__ __forceinline__ constexpr int cx(int q)
{
    return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
         : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ __forceinline__ constexpr int cy(int q)
{
    return (q == 3 || q == 7 || q == 8 || q == 15 || q == 17) ? 1
         : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ __forceinline__ constexpr int cz(int q)
{
    return (q == 5 || q == 11 || q == 12 || q == 15 || q == 16) ? 1
         : (q == 6 || q == 13 || q == 14 || q == 17 || q == 18) ? -1 : 0;
}
__host__ __device__ __forceinline__ constexpr int opp(int q)
{
    return q == 0 ? 0 : ((q <= 6) ? ((q & 1) ? q + 1 : q - 1)
                                  : ((q <= 14) ? (q <= 10 ? 17 - q : 25 - q) : 33 - q));
}
template <class R>
__host__ __device__ __forceinline__ constexpr R wgt(int q)
{
    return q == 0 ? R(1) / R(3) : (q <= 6 ? R(1) / R(18) : R(1) / R(36));
}

// Parameter block passed by value to every kernel.
template <class R>
struct KParams {
    int dx, dy, dz;
    long long n;       // dx*dy*dz
    int wall_mode;     // 0 periodic, 1 solid layers k<3 and k>dz-4
    int eos;           // 0 PR (reference), 1 VdW, 2 CS, 3 RK
    int lap_order;     // 5 or 7
    int complex_bc;    // layered wall extrapolation
    int qp;            // K1/K2 pressure-tensor term active
    R kk;              // K^2
    R A, B, T, ka, k1, k2;
    R ts[Q];
    R omts[Q];         // 1 - ts, rounded once on the host
    const R *wall;     // [2][dx*dy] wall chemical potential, bottom then top
    // FUSED collide: max over fluid nodes of |MV|^2 (float bits, atomicMax)
    // into mvmax[P * mvmax_stride] at parity P (null: not accumulated)
    unsigned *mvmax;
    int mvmax_stride;
};

__host__ __device__ __forceinline__ bool solid_k(int wall_mode, int k, int dz)
{
    return wall_mode == 1 && (k < 3 || k > dz - 4);
}

__device__ __forceinline__ int wrapm(int a, int n)
{
    a %= n;
    return a < 0 ? a + n : a;
}

// ---------------------------------------------------------------------------
// Bulk chemical potential mu0(rho) with the reference's density soft cap
// (FluidCuda.cu:450-451).  PR is the reference's expression
// (FluidCuda.cu:453); the other forms are d(psi)/d(rho) of the same
// free-energy convention psi = rho T ln(rho/(1-B rho)) + attraction.
template <class R>
__device__ __forceinline__ R eos_log(R x);
template <>
__device__ __forceinline__ float eos_log<float>(float x) { return logf(x); }
template <>
__device__ __forceinline__ double eos_log<double>(double x) { return log(x); }

template <class R>
__device__ __forceinline__ R mu0(int eos, R A, R B, R T, R rho)
{
    const R R0 = R(9.7), W0 = R(1.5);
    R d = rho;
    if (d > R0) d = R0 + (d - R0) / (R(1) + (d - R0) * W0);
    const R bd = B * d;
    if (eos == 1) {
        return T * eos_log<R>(d / (R(1) - bd)) + T / (R(1) - bd) - R(2) * A * d;
    } else if (eos == 2) {
        const R om = R(1) - bd;
        return T * eos_log<R>(d) + T + T * (R(8) * bd - R(9) * bd * bd + R(3) * bd * bd * bd) / (om * om * om) -
               R(2) * A * d;
    } else if (eos == 3) {
        return T * eos_log<R>(d / (R(1) - bd)) + T / (R(1) - bd) - A / B * eos_log<R>(R(1) + bd) -
               A * d / (R(1) + bd);
    }
    const R s2 = R(1.4142135623730950488016887242097);
    return T * eos_log<R>(d / (R(1) - bd)) - A / (s2 * R(2) * B) * eos_log<R>((s2 - R(1) + bd) / (s2 + R(1) - bd)) +
           T / (R(1) - bd) - A * d / (R(1) + bd * R(2) - bd * bd);
}

// Single-precision mu0 for the fused kernel: the same expressions with the
// per-launch constants hoisted, one reciprocal per distinct denominator
// (__fdividef: 2 ulp) and the hardware log2 (__logf: absolute error 2^-21.4
// near 1, 3 ulp elsewhere); mu is a sum of O(0.1) terms, so this stays at
// FP32 rounding level.
#ifdef __CUDACC__
struct EosFast {
    int eos;
    float A, B, T, c_att;  // c_att: A/(2 sqrt2 B) (PR) or A/B (RK)
};
__device__ __forceinline__ EosFast make_eos_fast(int eos, float A, float B, float T)
{
    EosFast e{eos, A, B, T, 0.f};
    if (eos == 0) e.c_att = A / (1.41421356237f * 2.0f * B);
    if (eos == 3) e.c_att = A / B;
    return e;
}
__device__ __forceinline__ float mu0_fast(const EosFast &e, float rho)
{
    const float R0 = 9.7f, W0 = 1.5f;
    float d = rho;
    if (d > R0) d = R0 + __fdividef(d - R0, 1.0f + (d - R0) * W0);
    const float bd = e.B * d;
    const float ir = __fdividef(1.0f, 1.0f - bd);
    if (e.eos == 2) {
        const float om3 = ir * ir * ir;
        return e.T * __logf(d) + e.T + e.T * (8.f * bd - 9.f * bd * bd + 3.f * bd * bd * bd) * om3 - 2.f * e.A * d;
    }
    const float base = e.T * __logf(d * ir) + e.T * ir;
    if (e.eos == 1) return base - 2.f * e.A * d;
    if (e.eos == 3) return base - e.c_att * __logf(1.0f + bd) - e.A * d * __fdividef(1.0f, 1.0f + bd);
    const float s2 = 1.41421356237f;
    return base - e.c_att * __logf((s2 - 1.0f + bd) * __fdividef(1.0f, s2 + 1.0f - bd)) -
           e.A * d * __fdividef(1.0f, 1.0f + bd * 2.0f - bd * bd);
}
#endif  // __CUDACC__

// ---------------------------------------------------------------------------
// MRT collision + exact-difference forcing, in moment space.
//
// Reference: LocalCollideMrt + GlobalCollide (FluidCuda.cu:245-347):
//   m = M f;  m <- m - S (m - meq(rho, u)) + S Qp;  f = M^-1 m;
//   f_i += feq_i(rho, u + F/rho) - feq_i(rho, u).
// Because M feq(rho, v) == meq(rho, v) exactly for this basis, the forcing
// increment is meq(rho, u + F/rho) - meq(rho, u) in moment space, and the
// whole update needs one forward and one inverse transform.  M is orthogonal
// with row norms 19, 2394, 252, 10, 40, 10, 40, 10, 40, 36, 72, 12, 24, 4, 4,
// 4, 8, 8, 8, so M^-1 = M^T diag(1/norm).  Both transforms are written out
// with shared partial sums over the axis pairs and the three diagonal planes.
template <class R>
__device__ __forceinline__ void meq_moments(R rho, R ux, R uy, R uz, R me[Q])
{
    const R u2 = ux * ux + uy * uy + uz * uz;
    me[0] = rho;
    me[1] = rho * (R(-11) + R(19) * u2);
    me[2] = rho * (R(3) - R(5.5) * u2);
    me[3] = rho * ux;
    me[4] = rho * ux * R(-2.0 / 3.0);
    me[5] = rho * uy;
    me[6] = rho * uy * R(-2.0 / 3.0);
    me[7] = rho * uz;
    me[8] = rho * uz * R(-2.0 / 3.0);
    const R pxx = rho * (ux * ux * R(2) - uy * uy - uz * uz);
    const R pww = rho * (uy * uy - uz * uz);
    me[9] = pxx;
    me[10] = pxx * R(-0.5);
    me[11] = pww;
    me[12] = pww * R(-0.5);
    me[13] = rho * ux * uy;
    me[14] = rho * uy * uz;
    me[15] = rho * ux * uz;
    me[16] = me[17] = me[18] = R(0);
}

template <class R>
__device__ __forceinline__ void moments(const R f[Q], R m[Q])
{
    const R a1 = f[1] + f[2], a2 = f[3] + f[4], a3 = f[5] + f[6];
    const R d1 = f[1] - f[2], d2 = f[3] - f[4], d3 = f[5] - f[6];
    // xy plane: 7(+,+) 8(-,+) 9(+,-) 10(-,-)
    const R sxy = (f[7] + f[10]) + (f[8] + f[9]);
    const R xxy = (f[7] - f[10]) - (f[8] - f[9]);  // x-momentum part
    const R yxy = (f[7] - f[10]) + (f[8] - f[9]);  // y-momentum part
    const R kxy = (f[7] + f[10]) - (f[8] + f[9]);
    // xz plane: 11(+,+) 12(-,+) 13(+,-) 14(-,-)
    const R sxz = (f[11] + f[14]) + (f[12] + f[13]);
    const R xxz = (f[11] - f[14]) - (f[12] - f[13]);
    const R zxz = (f[11] - f[14]) + (f[12] - f[13]);
    const R kxz = (f[11] + f[14]) - (f[12] + f[13]);
    // yz plane: 15(+,+) 16(-,+) 17(+,-) 18(-,-)
    const R syz = (f[15] + f[18]) + (f[16] + f[17]);
    const R yyz = (f[15] - f[18]) - (f[16] - f[17]);
    const R zyz = (f[15] - f[18]) + (f[16] - f[17]);
    const R kyz = (f[15] + f[18]) - (f[16] + f[17]);
    const R es = a1 + a2 + a3, ds = sxy + sxz + syz;
    m[0] = f[0] + es + ds;
    m[1] = R(-30) * f[0] - R(11) * es + R(8) * ds;
    m[2] = R(12) * f[0] - R(4) * es + ds;
    m[3] = d1 + xxy + xxz;
    m[4] = R(-4) * d1 + xxy + xxz;
    m[5] = d2 + yxy + yyz;
    m[6] = R(-4) * d2 + yxy + yyz;
    m[7] = d3 + zxz + zyz;
    m[8] = R(-4) * d3 + zxz + zyz;
    m[9] = R(2) * a1 - a2 - a3 + sxy + sxz - R(2) * syz;
    m[10] = R(-4) * a1 + R(2) * (a2 + a3) + sxy + sxz - R(2) * syz;
    m[11] = a2 - a3 + sxy - sxz;
    m[12] = R(-2) * (a2 - a3) + sxy - sxz;
    m[13] = kxy;
    m[14] = kyz;
    m[15] = kxz;
    m[16] = xxy - xxz;
    m[17] = yyz - yxy;
    m[18] = zxz - zyz;
}

// f = M^-1 m = M^T (m / norm)
template <class R>
__device__ __forceinline__ void inverse_moments(const R m[Q], R f[Q])
{
    // multiply by the rounded reciprocals of the row norms (no divisions)
    const R n0 = m[0] * (R(1) / R(19)), n1 = m[1] * (R(1) / R(2394)), n2 = m[2] * (R(1) / R(252));
    const R n3 = m[3] * R(0.1), n4 = m[4] * R(0.025), n5 = m[5] * R(0.1), n6 = m[6] * R(0.025);
    const R n7 = m[7] * R(0.1), n8 = m[8] * R(0.025);
    const R n9 = m[9] * (R(1) / R(36)), n10 = m[10] * (R(1) / R(72)), n11 = m[11] * (R(1) / R(12));
    const R n12 = m[12] * (R(1) / R(24));
    const R n13 = m[13] * R(0.25), n14 = m[14] * R(0.25), n15 = m[15] * R(0.25);
    const R n16 = m[16] * R(0.125), n17 = m[17] * R(0.125), n18 = m[18] * R(0.125);
    f[0] = n0 - R(30) * n1 + R(12) * n2;
    const R be = n0 - R(11) * n1 - R(4) * n2;  // axis directions
    const R bd = n0 + R(8) * n1 + n2;           // diagonal directions
    const R jx = n3 - R(4) * n4, jy = n5 - R(4) * n6, jz = n7 - R(4) * n8;
    const R pxa = R(2) * n9 - R(4) * n10;      // x-axis pair
    const R pyz = -n9 + R(2) * n10;             // y/z-axis pairs
    const R qw = n11 - R(2) * n12;
    f[1] = be + jx + pxa;
    f[2] = be - jx + pxa;
    f[3] = be + jy + pyz + qw;
    f[4] = be - jy + pyz + qw;
    f[5] = be + jz + pyz - qw;
    f[6] = be - jz + pyz - qw;
    const R gx = n3 + n4, gy = n5 + n6, gz = n7 + n8;
    // xy plane: diag part n9 + n10 + n11 + n12
    const R pxy = bd + n9 + n10 + n11 + n12;
    f[7] = pxy + gx + gy + n13 + n16 - n17;
    f[8] = pxy - gx + gy - n13 - n16 - n17;
    f[9] = pxy + gx - gy - n13 + n16 + n17;
    f[10] = pxy - gx - gy + n13 - n16 + n17;
    // xz plane: n9 + n10 - n11 - n12
    const R pxz = bd + n9 + n10 - n11 - n12;
    f[11] = pxz + gx + gz + n15 - n16 + n18;
    f[12] = pxz - gx + gz - n15 + n16 + n18;
    f[13] = pxz + gx - gz - n15 - n16 - n18;
    f[14] = pxz - gx - gz + n15 + n16 - n18;
    // yz plane: -2 n9 - 2 n10
    const R pyzd = bd - R(2) * n9 - R(2) * n10;
    f[15] = pyzd + gy + gz + n14 + n17 - n18;
    f[16] = pyzd - gy + gz - n14 - n17 - n18;
    f[17] = pyzd + gy - gz - n14 + n17 + n18;
    f[18] = pyzd - gy - gz + n14 - n17 + n18;
}

// In: f (post-stream), rho, bare u, force F, rates, optional Qp (pressure
// tensor, FluidCuda.cu:260-266).  Out: f (post-collision incl. forcing).
template <class R>
__device__ __forceinline__ void collide_mrt_edm(R f[Q], R rho, R ux, R uy, R uz, R Fx, R Fy, R Fz,
                                                const R ts[Q], const R *qp)
{
    R m[Q], me[Q], me1[Q];
    moments<R>(f, m);
    meq_moments<R>(rho, ux, uy, uz, me);
    const R ir = R(1) / rho;
    meq_moments<R>(rho, ux + Fx * ir, uy + Fy * ir, uz + Fz * ir, me1);
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        R v = m[a] - ts[a] * (m[a] - me[a]) + (me1[a] - me[a]);
        if (qp) v += qp[a] * ts[a];
        m[a] = v;
    }
    inverse_moments<R>(m, f);
}

// FP32 moment transforms of the FUSED kernel with every fused multiply-add
// written out (the FUSED translation unit is compiled without implicit
// contraction, so its rounding does not depend on how the compiler schedules
// a particular instantiation).  Same algebra as meq_moments / moments /
// inverse_moments.
__device__ __forceinline__ void meq_moments_x(float rho, float ux, float uy, float uz, float me[Q])
{
    const float uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
    const float u2 = uxx + uyy + uzz;
    const float jx = rho * ux, jy = rho * uy, jz = rho * uz;
    me[0] = rho;
    me[1] = rho * fmaf(19.f, u2, -11.f);
    me[2] = rho * fmaf(-5.5f, u2, 3.f);
    me[3] = jx;
    me[4] = jx * (-2.f / 3.f);
    me[5] = jy;
    me[6] = jy * (-2.f / 3.f);
    me[7] = jz;
    me[8] = jz * (-2.f / 3.f);
    const float pxx = rho * fmaf(2.f, uxx, -(uyy + uzz));
    const float pww = rho * (uyy - uzz);
    me[9] = pxx;
    me[10] = pxx * -0.5f;
    me[11] = pww;
    me[12] = pww * -0.5f;
    me[13] = jx * uy;
    me[14] = jy * uz;
    me[15] = jx * uz;
    me[16] = me[17] = me[18] = 0.f;
}

__device__ __forceinline__ void moments_x(const float f[Q], float m[Q])
{
    const float a1 = f[1] + f[2], a2 = f[3] + f[4], a3 = f[5] + f[6];
    const float d1 = f[1] - f[2], d2 = f[3] - f[4], d3 = f[5] - f[6];
    const float sxy = (f[7] + f[10]) + (f[8] + f[9]);
    const float xxy = (f[7] - f[10]) - (f[8] - f[9]);
    const float yxy = (f[7] - f[10]) + (f[8] - f[9]);
    const float kxy = (f[7] + f[10]) - (f[8] + f[9]);
    const float sxz = (f[11] + f[14]) + (f[12] + f[13]);
    const float xxz = (f[11] - f[14]) - (f[12] - f[13]);
    const float zxz = (f[11] - f[14]) + (f[12] - f[13]);
    const float kxz = (f[11] + f[14]) - (f[12] + f[13]);
    const float syz = (f[15] + f[18]) + (f[16] + f[17]);
    const float yyz = (f[15] - f[18]) - (f[16] - f[17]);
    const float zyz = (f[15] - f[18]) + (f[16] - f[17]);
    const float kyz = (f[15] + f[18]) - (f[16] + f[17]);
    const float es = a1 + a2 + a3, ds = sxy + sxz + syz;
    m[0] = f[0] + es + ds;
    m[1] = fmaf(-30.f, f[0], fmaf(-11.f, es, 8.f * ds));
    m[2] = fmaf(12.f, f[0], fmaf(-4.f, es, ds));
    const float sx = xxy + xxz, sy = yxy + yyz, sz = zxz + zyz;
    m[3] = d1 + sx;
    m[4] = fmaf(-4.f, d1, sx);
    m[5] = d2 + sy;
    m[6] = fmaf(-4.f, d2, sy);
    m[7] = d3 + sz;
    m[8] = fmaf(-4.f, d3, sz);
    const float t9 = fmaf(-2.f, syz, sxy + sxz);
    m[9] = fmaf(2.f, a1, t9 - (a2 + a3));
    m[10] = fmaf(-4.f, a1, fmaf(2.f, a2 + a3, t9));
    m[11] = (a2 - a3) + (sxy - sxz);
    m[12] = fmaf(-2.f, a2 - a3, sxy - sxz);
    m[13] = kxy;
    m[14] = kyz;
    m[15] = kxz;
    m[16] = xxy - xxz;
    m[17] = yyz - yxy;
    m[18] = zxz - zyz;
}

// f = M^-1 m = M^T (m / norm), the row-norm scalings folded into the
// fused multiply-adds of the shared partial sums
__device__ __forceinline__ void inverse_moments_x(const float m[Q], float f[Q])
{
    const float n0 = m[0] * (1.f / 19.f), n1 = m[1] * (1.f / 2394.f), n2 = m[2] * (1.f / 252.f);
    f[0] = fmaf(-30.f, n1, fmaf(12.f, n2, n0));
    const float be = fmaf(-11.f, n1, fmaf(-4.f, n2, n0));
    const float bd = fmaf(8.f, n1, n0 + n2);
    const float jx = fmaf(m[3], 0.1f, m[4] * -0.1f), gx = fmaf(m[3], 0.1f, m[4] * 0.025f);
    const float jy = fmaf(m[5], 0.1f, m[6] * -0.1f), gy = fmaf(m[5], 0.1f, m[6] * 0.025f);
    const float jz = fmaf(m[7], 0.1f, m[8] * -0.1f), gz = fmaf(m[7], 0.1f, m[8] * 0.025f);
    const float pxa = fmaf(m[9], 2.f / 36.f, m[10] * (-4.f / 72.f));
    const float pyz = fmaf(m[9], -1.f / 36.f, m[10] * (2.f / 72.f));
    const float qw = fmaf(m[11], 1.f / 12.f, m[12] * (-2.f / 24.f));
    f[1] = be + jx + pxa;
    f[2] = be - jx + pxa;
    f[3] = be + jy + pyz + qw;
    f[4] = be - jy + pyz + qw;
    f[5] = be + jz + pyz - qw;
    f[6] = be - jz + pyz - qw;
    const float s910 = fmaf(m[9], 1.f / 36.f, m[10] * (1.f / 72.f));
    const float s1112 = fmaf(m[11], 1.f / 12.f, m[12] * (1.f / 24.f));
    const float n13 = m[13] * 0.25f, n14 = m[14] * 0.25f, n15 = m[15] * 0.25f;
    const float n16 = m[16] * 0.125f, n17 = m[17] * 0.125f, n18 = m[18] * 0.125f;
    const float pxy = bd + s910 + s1112;
    f[7] = pxy + gx + gy + n13 + n16 - n17;
    f[8] = pxy - gx + gy - n13 - n16 - n17;
    f[9] = pxy + gx - gy - n13 + n16 + n17;
    f[10] = pxy - gx - gy + n13 - n16 + n17;
    const float pxz = bd + s910 - s1112;
    f[11] = pxz + gx + gz + n15 - n16 + n18;
    f[12] = pxz - gx + gz - n15 + n16 + n18;
    f[13] = pxz + gx - gz - n15 - n16 - n18;
    f[14] = pxz - gx - gz + n15 + n16 - n18;
    const float pyzd = fmaf(-2.f, s910, bd);
    f[15] = pyzd + gy + gz + n14 + n17 - n18;
    f[16] = pyzd - gy + gz - n14 - n17 - n18;
    f[17] = pyzd + gy - gz - n14 + n17 + n18;
    f[18] = pyzd - gy - gz + n14 - n17 + n18;
}

// The collision of the FUSED kernel: the relaxation written as
// m* = (1 - s) (m - meq(u)) + meq(u + F/rho), two operations per moment
// (mathematically the reference's update; rounding differs).
__device__ __forceinline__ void collide_mrt_edm_fused(float f[Q], float rho, float ux, float uy, float uz,
                                                      float Fx, float Fy, float Fz, const float ts[Q],
                                                      const float omts[Q], const float *qp)
{
    float m[Q], me[Q], me1[Q];
    moments_x(f, m);
    meq_moments_x(rho, ux, uy, uz, me);
    const float ir = 1.0f / rho;
    meq_moments_x(rho, fmaf(Fx, ir, ux), fmaf(Fy, ir, uy), fmaf(Fz, ir, uz), me1);
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        float v = a >= 16 ? omts[a] * m[a] : fmaf(omts[a], m[a] - me[a], me1[a]);  // meq = 0 for 16..18
        if (qp) v = fmaf(qp[a], ts[a], v);
        m[a] = v;
    }
    inverse_moments_x(m, f);
}

#ifdef __CUDACC__
// Two nodes at once (lane x, lane y) with the paired FP32 instructions:
// the same operations in the same order as the _x versions above, so a pair
// gives exactly the bits of two single-node evaluations.
namespace p2 {
__device__ __forceinline__ float2 K(float c) { return make_float2(c, c); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
}  // namespace p2

__device__ __forceinline__ void meq_moments_x2(float2 rho, float2 ux, float2 uy, float2 uz, float2 me[Q])
{
    using namespace p2;
    const float2 uxx = mul(ux, ux), uyy = mul(uy, uy), uzz = mul(uz, uz);
    const float2 u2 = add(add(uxx, uyy), uzz);
    const float2 jx = mul(rho, ux), jy = mul(rho, uy), jz = mul(rho, uz);
    me[0] = rho;
    me[1] = mul(rho, fma(K(19.f), u2, K(-11.f)));
    me[2] = mul(rho, fma(K(-5.5f), u2, K(3.f)));
    me[3] = jx;
    me[4] = mul(jx, K(-2.f / 3.f));
    me[5] = jy;
    me[6] = mul(jy, K(-2.f / 3.f));
    me[7] = jz;
    me[8] = mul(jz, K(-2.f / 3.f));
    const float2 pxx = mul(rho, fma(K(2.f), uxx, neg(add(uyy, uzz))));
    const float2 pww = mul(rho, sub(uyy, uzz));
    me[9] = pxx;
    me[10] = mul(pxx, K(-0.5f));
    me[11] = pww;
    me[12] = mul(pww, K(-0.5f));
    me[13] = mul(jx, uy);
    me[14] = mul(jy, uz);
    me[15] = mul(jx, uz);
    me[16] = me[17] = me[18] = K(0.f);
}

__device__ __forceinline__ void moments_x2(const float2 f[Q], float2 m[Q])
{
    using namespace p2;
    const float2 a1 = add(f[1], f[2]), a2 = add(f[3], f[4]), a3 = add(f[5], f[6]);
    const float2 d1 = sub(f[1], f[2]), d2 = sub(f[3], f[4]), d3 = sub(f[5], f[6]);
    const float2 sxy = add(add(f[7], f[10]), add(f[8], f[9]));
    const float2 xxy = sub(sub(f[7], f[10]), sub(f[8], f[9]));
    const float2 yxy = add(sub(f[7], f[10]), sub(f[8], f[9]));
    const float2 kxy = sub(add(f[7], f[10]), add(f[8], f[9]));
    const float2 sxz = add(add(f[11], f[14]), add(f[12], f[13]));
    const float2 xxz = sub(sub(f[11], f[14]), sub(f[12], f[13]));
    const float2 zxz = add(sub(f[11], f[14]), sub(f[12], f[13]));
    const float2 kxz = sub(add(f[11], f[14]), add(f[12], f[13]));
    const float2 syz = add(add(f[15], f[18]), add(f[16], f[17]));
    const float2 yyz = sub(sub(f[15], f[18]), sub(f[16], f[17]));
    const float2 zyz = add(sub(f[15], f[18]), sub(f[16], f[17]));
    const float2 kyz = sub(add(f[15], f[18]), add(f[16], f[17]));
    const float2 es = add(add(a1, a2), a3), ds = add(add(sxy, sxz), syz);
    m[0] = add(add(f[0], es), ds);
    m[1] = fma(K(-30.f), f[0], fma(K(-11.f), es, mul(K(8.f), ds)));
    m[2] = fma(K(12.f), f[0], fma(K(-4.f), es, ds));
    const float2 sx = add(xxy, xxz), sy = add(yxy, yyz), sz = add(zxz, zyz);
    m[3] = add(d1, sx);
    m[4] = fma(K(-4.f), d1, sx);
    m[5] = add(d2, sy);
    m[6] = fma(K(-4.f), d2, sy);
    m[7] = add(d3, sz);
    m[8] = fma(K(-4.f), d3, sz);
    const float2 t9 = fma(K(-2.f), syz, add(sxy, sxz));
    m[9] = fma(K(2.f), a1, sub(t9, add(a2, a3)));
    m[10] = fma(K(-4.f), a1, fma(K(2.f), add(a2, a3), t9));
    m[11] = add(sub(a2, a3), sub(sxy, sxz));
    m[12] = fma(K(-2.f), sub(a2, a3), sub(sxy, sxz));
    m[13] = kxy;
    m[14] = kyz;
    m[15] = kxz;
    m[16] = sub(xxy, xxz);
    m[17] = sub(yyz, yxy);
    m[18] = sub(zxz, zyz);
}

__device__ __forceinline__ void inverse_moments_x2(const float2 m[Q], float2 f[Q])
{
    using namespace p2;
    const float2 n0 = mul(m[0], K(1.f / 19.f)), n1 = mul(m[1], K(1.f / 2394.f)), n2 = mul(m[2], K(1.f / 252.f));
    f[0] = fma(K(-30.f), n1, fma(K(12.f), n2, n0));
    const float2 be = fma(K(-11.f), n1, fma(K(-4.f), n2, n0));
    const float2 bd = fma(K(8.f), n1, add(n0, n2));
    const float2 jx = fma(m[3], K(0.1f), mul(m[4], K(-0.1f))), gx = fma(m[3], K(0.1f), mul(m[4], K(0.025f)));
    const float2 jy = fma(m[5], K(0.1f), mul(m[6], K(-0.1f))), gy = fma(m[5], K(0.1f), mul(m[6], K(0.025f)));
    const float2 jz = fma(m[7], K(0.1f), mul(m[8], K(-0.1f))), gz = fma(m[7], K(0.1f), mul(m[8], K(0.025f)));
    const float2 pxa = fma(m[9], K(2.f / 36.f), mul(m[10], K(-4.f / 72.f)));
    const float2 pyz = fma(m[9], K(-1.f / 36.f), mul(m[10], K(2.f / 72.f)));
    const float2 qw = fma(m[11], K(1.f / 12.f), mul(m[12], K(-2.f / 24.f)));
    f[1] = add(add(be, jx), pxa);
    f[2] = add(sub(be, jx), pxa);
    f[3] = add(add(add(be, jy), pyz), qw);
    f[4] = add(add(sub(be, jy), pyz), qw);
    f[5] = sub(add(add(be, jz), pyz), qw);
    f[6] = sub(add(sub(be, jz), pyz), qw);
    const float2 s910 = fma(m[9], K(1.f / 36.f), mul(m[10], K(1.f / 72.f)));
    const float2 s1112 = fma(m[11], K(1.f / 12.f), mul(m[12], K(1.f / 24.f)));
    const float2 n13 = mul(m[13], K(0.25f)), n14 = mul(m[14], K(0.25f)), n15 = mul(m[15], K(0.25f));
    const float2 n16 = mul(m[16], K(0.125f)), n17 = mul(m[17], K(0.125f)), n18 = mul(m[18], K(0.125f));
    const float2 pxy = add(add(bd, s910), s1112);
    f[7] = sub(add(add(add(add(pxy, gx), gy), n13), n16), n17);
    f[8] = sub(sub(sub(add(sub(pxy, gx), gy), n13), n16), n17);
    f[9] = add(add(sub(sub(add(pxy, gx), gy), n13), n16), n17);
    f[10] = add(sub(add(sub(sub(pxy, gx), gy), n13), n16), n17);
    const float2 pxz = sub(add(bd, s910), s1112);
    f[11] = add(sub(add(add(add(pxz, gx), gz), n15), n16), n18);
    f[12] = add(add(sub(add(sub(pxz, gx), gz), n15), n16), n18);
    f[13] = sub(sub(sub(sub(add(pxz, gx), gz), n15), n16), n18);
    f[14] = sub(add(add(sub(sub(pxz, gx), gz), n15), n16), n18);
    const float2 pyzd = fma(K(-2.f), s910, bd);
    f[15] = sub(add(add(add(add(pyzd, gy), gz), n14), n17), n18);
    f[16] = sub(sub(sub(add(sub(pyzd, gy), gz), n14), n17), n18);
    f[17] = add(add(sub(sub(add(pyzd, gy), gz), n14), n17), n18);
    f[18] = add(sub(add(sub(sub(pyzd, gy), gz), n14), n17), n18);
}

// collide_mrt_edm_fused for two nodes; ir = 1 / rho per lane.
__device__ __forceinline__ void collide_mrt_edm_fused2(float2 f[Q], float2 rho, float2 ir, float2 ux, float2 uy,
                                                       float2 uz, float2 Fx, float2 Fy, float2 Fz,
                                                       const float ts[Q], const float omts[Q], const float2 *qp)
{
    using namespace p2;
    float2 m[Q], me[Q], me1[Q];
    moments_x2(f, m);
    meq_moments_x2(rho, ux, uy, uz, me);
    meq_moments_x2(rho, fma(Fx, ir, ux), fma(Fy, ir, uy), fma(Fz, ir, uz), me1);
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        float2 v = a >= 16 ? mul(K(omts[a]), m[a]) : fma(K(omts[a]), sub(m[a], me[a]), me1[a]);
        if (qp) v = fma(qp[a], K(ts[a]), v);
        m[a] = v;
    }
    inverse_moments_x2(m, f);
}
#endif  // __CUDACC__

}  // namespace cpmp
