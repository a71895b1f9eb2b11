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
    // FUSED collide: set to non-zero when a bounded wait for a shared-memory
    // copy gave up (null: not reported)
    unsigned *err;
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
    if (sizeof(R) == 4) {
        // FP32: the rest population is the remainder of the mass moment after
        // the 18 moving populations (pairwise sums), so a node emits the mass
        // it holds to one rounding.  The rounded reciprocal of 19 in
        // inverse_moments gives every population m0 * fl(1/19), which raises
        // each node's mass by 19 fl(1/19) - 1 = 7.5e-9 every step in FP32: a
        // linear drift of the density (7.5e-6 after 1000 steps).  In exact
        // arithmetic both forms give the same f0 (row 0 of M sums the
        // populations); FP64 keeps the reference's expression.
        const R a = (f[1] + f[2]) + (f[3] + f[4]) + (f[5] + f[6]);
        const R b = ((f[7] + f[8]) + (f[9] + f[10])) + ((f[11] + f[12]) + (f[13] + f[14]));
        const R c = (f[15] + f[16]) + (f[17] + f[18]);
        f[0] = m[0] - ((a + c) + b);
    }
}

}  // namespace cpmp
