// k_adjoint.cuh -- reverse (adjoint) of one PLAIN time step.
//
// Forward step n on fluid nodes (FluidCuda.cu:1279-1291):
//   rho, u   = moments of f^n                       (MacroCalculate of step n-1)
//   rho_s    = W(rho)        wall layers            (ChemBoundary)
//   mu       = K^2 mu0(rho) - ka Lap(rho); mu_s = w (ChemPotential, wall field)
//   F        = -rho G(mu) + G(rho)/3                (NonidealForce)
//   f*       = M^-1 [ (I-S) M f + S meq(rho,u) + meq(rho, u+F/rho) - meq(rho,u) ]
//   f^{n+1}  = stream(f*) with half-way bounce-back (GlobalCollide)
// dJ/df^n is kept in factored form: lamp_q(x) + lamrho(x) on fluid nodes
// (0 on solid ones), so the sum is never written out.  Given that pair for
// step n+1 the reverse step produces the pair of step n and accumulates
// dJ/dw (wall field) and dJ/dka:
//   R2  k_adj_collide : pull dJ/df^{n+1} = lamp + lamrho through the streaming
//       (bounce-back transposed), collision adjoint in moment space ->
//       lamp (partial dJ/df), dJ/dF, the collision's dJ/drho
//   R3  k_adj_force   : dJ/dmu(y) = sum_a G_a(rho lamF_a)(y),
//       dJ/drho(y) += -sum_a G_a(lamF_a)(y)/3 - lamF(y).G(mu)(y)
//       (the gradient stencils are antisymmetric, so their transpose is the
//       negated stencil)
//   R4  k_adj_mu      : dJ/drho(y) += K^2 mu0'(rho) lam_mu - ka Lap(lam_mu on
//       fluid)(y) (the Laplacian is symmetric); dJ/dka += -sum lam_mu Lap(rho)
//   R5  k_adj_wall    : wall layers back onto the first fluid layer (the
//       6-point average is symmetric), dJ/dw += lam_mu on the solid layers
//   (R6, dJ/df^n_q = lamp_q + lamrho, is folded into the next R2's gather)
// The K1/K2 pressure-tensor term is not differentiated (callers get
// CPMP_ERR_UNSUPPORTED when it is active).
#pragma once

#include <type_traits>

#include "k_plain.cuh"
#include "kernels.h"

namespace cpmp {

// d(mu0)/d(rho) including the density soft cap, matching mu0<R>.
template <class R>
__device__ __forceinline__ R dmu0(int eos, R A, R B, R T, R rho)
{
    const R R0 = R(9.7), W0 = R(1.5);
    R d = rho, dd = R(1);
    if (d > R0) {
        const R del = d - R0, den = R(1) + del * W0;
        d = R0 + del / den;
        dd = R(1) / (den * den);
    }
    const R b = B, bd = b * d, om = R(1) - bd;
    R m;
    if (eos == 1) {
        m = T / d + T * b / om + T * b / (om * om) - R(2) * A;
    } else if (eos == 2) {
        m = T / d + T * b * (R(8) - R(2) * bd) / (om * om * om * om) - R(2) * A;
    } else if (eos == 3) {
        const R op = R(1) + bd;
        m = T / d + T * b / om + T * b / (om * om) - A / op - A / (op * op);
    } else {
        const R s2 = R(1.4142135623730950488016887242097);
        const R c = A / (s2 * R(2) * b);
        const R den = R(1) + bd * R(2) - bd * bd;
        m = T / d + T * b / om - c * b / (s2 - R(1) + bd) - c * b / (s2 + R(1) - bd) + T * b / (om * om) -
            A * (R(1) + bd * bd) / (den * den);
    }
    return m * dd;
}

// Adjoint of meq(rho, v) for adjoint weights Aw[19]: adds d/drho and d/dv.
template <class R>
__device__ __forceinline__ void meq_adjoint(R rho, R vx, R vy, R vz, const R Aw[Q], R &a_rho, R &avx, R &avy,
                                            R &avz)
{
    R me[Q];
    meq_moments<R>(rho, vx, vy, vz, me);
    R s = R(0);
#pragma unroll
    for (int a = 0; a < Q; ++a) s += Aw[a] * me[a];
    a_rho += s / rho;  // every equilibrium moment is linear in rho
    const R k1 = Aw[1] * R(38) - Aw[2] * R(11);   // from v^2 terms
    const R p9 = Aw[9] - R(0.5) * Aw[10];          // 2vx^2 - vy^2 - vz^2
    const R p11 = Aw[11] - R(0.5) * Aw[12];        // vy^2 - vz^2
    avx += rho * (k1 * vx + (Aw[3] - R(2.0 / 3.0) * Aw[4]) + p9 * R(4) * vx + Aw[13] * vy + Aw[15] * vz);
    avy += rho * (k1 * vy + (Aw[5] - R(2.0 / 3.0) * Aw[6]) - p9 * R(2) * vy + p11 * R(2) * vy + Aw[13] * vx +
                  Aw[14] * vz);
    avz += rho * (k1 * vz + (Aw[7] - R(2.0 / 3.0) * Aw[8]) - p9 * R(2) * vz - p11 * R(2) * vz + Aw[14] * vy +
                  Aw[15] * vx);
}

// R2: collision + streaming adjoint (one thread per node, 3-D grid).
template <class R>
__global__ void __launch_bounds__(128) k_adj_collide(KParams<R> p, const uint8_t *type, const R *rho,
                                                     const R *u, const R *F, const R *lamp_next,
                                                     const R *lamrho_next, R *lamp, R *lamF, R *lamrho)
{
    NODE3D(p);
    const long long n = p.n;
    if (type[I] != FLUID) {
#pragma unroll
        for (int q = 0; q < Q; ++q) lamp[q * n + I] = R(0);
        lamF[I] = lamF[I + n] = lamF[I + 2 * n] = R(0);
        lamrho[I] = R(0);
        return;
    }
    // lambda* (adjoint of the post-collision populations): pull through the
    // push streaming; a population bounced back at a solid destination came
    // back into slot opp(q) of this node
    R ls[Q];
    const R lr_here = lamrho_next[I];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int ii = wrap_off(i + cx(q), p.dx), jj = wrap_off(j + cy(q), p.dy), kk = wrap_off(k + cz(q), p.dz);
        const long long D = nid(p, ii, jj, kk);
        ls[q] = type[D] == FLUID ? lamp_next[q * n + D] + lamrho_next[D] : lamp_next[opp(q) * n + I] + lr_here;
    }
    // mu* = M^-T lambda* = diag(1/norm) M lambda*
    R ms[Q];
    moments<R>(ls, ms);
    const R inv_norm[Q] = {R(1) / R(19), R(1) / R(2394), R(1) / R(252), R(0.1), R(0.025), R(0.1), R(0.025),
                           R(0.1),       R(0.025),       R(1) / R(36),  R(1) / R(72), R(1) / R(12), R(1) / R(24),
                           R(0.25),      R(0.25),        R(0.25),       R(0.125),     R(0.125),     R(0.125)};
    R am[Q], a0[Q], a1[Q];
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        const R mu_a = ms[a] * inv_norm[a];
        am[a] = (R(1) - p.ts[a]) * mu_a;
        a0[a] = (p.ts[a] - R(1)) * mu_a;
        a1[a] = mu_a;
    }
    const R r = rho[I], ux = u[I], uy = u[I + n], uz = u[I + 2 * n];
    const R Fx = F[I], Fy = F[I + n], Fz = F[I + 2 * n];
    const R ir = R(1) / r;
    const R v1x = ux + Fx * ir, v1y = uy + Fy * ir, v1z = uz + Fz * ir;
    R a_rho = R(0), aux = R(0), auy = R(0), auz = R(0), av1x = R(0), av1y = R(0), av1z = R(0);
    meq_adjoint<R>(r, ux, uy, uz, a0, a_rho, aux, auy, auz);
    meq_adjoint<R>(r, v1x, v1y, v1z, a1, a_rho, av1x, av1y, av1z);
    // v1 = u + F/rho
    aux += av1x;
    auy += av1y;
    auz += av1z;
    lamF[I] = av1x * ir;
    lamF[I + n] = av1y * ir;
    lamF[I + 2 * n] = av1z * ir;
    a_rho -= (av1x * Fx + av1y * Fy + av1z * Fz) * ir * ir;
    // u = j / rho
    const R ajx = aux * ir, ajy = auy * ir, ajz = auz * ir;
    a_rho -= (aux * ux + auy * uy + auz * uz) * ir;
    lamrho[I] = a_rho;
    // m = M f  ->  M^T am ;  j = sum e f  ->  e . aj
    R fm[Q];
    // M^T x = diag(norm) M^-1 x  (M^-1 = M^T diag(1/norm))
    R amn[Q];
    const R norm[Q] = {R(19), R(2394), R(252), R(10), R(40), R(10), R(40), R(10), R(40), R(36),
                       R(72), R(12),   R(24),  R(4),  R(4),  R(4),  R(8),  R(8),  R(8)};
#pragma unroll
    for (int a = 0; a < Q; ++a) amn[a] = am[a] * norm[a];
    inverse_moments<R>(amn, fm);
#pragma unroll
    for (int q = 0; q < Q; ++q) lamp[q * n + I] = fm[q] + R(cx(q)) * ajx + R(cy(q)) * ajy + R(cz(q)) * ajz;
}

// R3: force adjoint (stencil gathers).
template <class R>
__global__ void __launch_bounds__(128) k_adj_force(KParams<R> p, const uint8_t *type, const R *rho, const R *mu,
                                                   const R *lamF, R *lammu, R *lamrho)
{
    NODE3D(p);
    const long long n = p.n;
    int a[7], b[7], c[7];
#pragma unroll
    for (int d = -3; d <= 3; ++d) {
        a[d + 3] = wrap_off(i + d, p.dx);
        b[d + 3] = wrap_off(j + d, p.dy);
        c[d + 3] = wrap_off(k + d, p.dz);
    }
    // for each lattice line (sx, sy, sz) with weight vector w (2 e on the
    // axes, e on the diagonals): sum_d c_d (v(+d) - v(-d)) of v = w . lamF
    // and of rho v; only the nonzero components of w are loaded
    R gm = R(0), gr = R(0);
    auto acc = [&](auto SX, auto SY, auto SZ) {
        constexpr int sx = decltype(SX)::value, sy = decltype(SY)::value, sz = decltype(SZ)::value;
        constexpr int axis = (sx != 0) + (sy != 0) + (sz != 0) == 1;
        constexpr int wx = axis ? 2 * sx : sx, wy = axis ? 2 * sy : sy, wz = axis ? 2 * sz : sz;
        auto lw = [&](long long P) -> R {
            R v = R(0);
            if constexpr (wx != 0) v += R(wx) * lamF[P];
            if constexpr (wy != 0) v += R(wy) * lamF[P + n];
            if constexpr (wz != 0) v += R(wz) * lamF[P + 2 * n];
            return v;
        };
#pragma unroll
        for (int d = 1; d <= 3; ++d) {
            const R cd = d == 1 ? R(45) : (d == 2 ? R(-9) : R(1));
            const long long P_ = nid(p, a[3 + sx * d], b[3 + sy * d], c[3 + sz * d]);
            const long long M_ = nid(p, a[3 - sx * d], b[3 - sy * d], c[3 - sz * d]);
            const R lp = lw(P_), lm = lw(M_);
            gm += cd * (rho[P_] * lp - rho[M_] * lm);
            gr += cd * (lp - lm);
        }
    };
    using P1 = std::integral_constant<int, 1>;
    using Z0 = std::integral_constant<int, 0>;
    using M1 = std::integral_constant<int, -1>;
    acc(P1{}, Z0{}, Z0{});
    acc(Z0{}, P1{}, Z0{});
    acc(Z0{}, Z0{}, P1{});
    acc(P1{}, P1{}, Z0{});
    acc(P1{}, M1{}, Z0{});
    acc(P1{}, Z0{}, P1{});
    acc(P1{}, Z0{}, M1{});
    acc(Z0{}, P1{}, P1{});
    acc(Z0{}, P1{}, M1{});
    lammu[I] = gm / R(360);
    R add = -gr / R(360) / R(3);
    if (type[I] == FLUID) {
        R g[3];
        grad7_g(p, mu, i, j, k, g);
        add -= lamF[I] * g[0] + lamF[I + n] * g[1] + lamF[I + 2 * n] * g[2];
    }
    lamrho[I] += add;
}

// Laplacians of an R field evaluated in FP64 (for the kappa gradient).
template <class R>
__device__ __forceinline__ double lap5_d(const KParams<R> &p, const R *x, int i, int j, int k)
{
    auto X = [&](int a, int b, int c) -> double { return (double)x[nid(p, a, b, c)]; };
    const int im2 = wrap_off(i - 2, p.dx), im1 = wrap_off(i - 1, p.dx), ip1 = wrap_off(i + 1, p.dx),
              ip2 = wrap_off(i + 2, p.dx);
    const int jm2 = wrap_off(j - 2, p.dy), jm1 = wrap_off(j - 1, p.dy), jp1 = wrap_off(j + 1, p.dy),
              jp2 = wrap_off(j + 2, p.dy);
    const int km2 = wrap_off(k - 2, p.dz), km1 = wrap_off(k - 1, p.dz), kp1 = wrap_off(k + 1, p.dz),
              kp2 = wrap_off(k + 2, p.dz);
    return (-X(i, j, k) * 90.0 + (-X(im2, j, k) + X(im1, j, k) * 16.0 + X(ip1, j, k) * 16.0 - X(ip2, j, k)) +
            (-X(i, jm2, k) + X(i, jm1, k) * 16.0 + X(i, jp1, k) * 16.0 - X(i, jp2, k)) +
            (-X(i, j, km2) + X(i, j, km1) * 16.0 + X(i, j, kp1) * 16.0 - X(i, j, kp2))) /
           12.0;
}
template <class R>
__device__ __forceinline__ double lap7_d(const KParams<R> &p, const R *x, int i, int j, int k)
{
    auto X = [&](int a, int b, int c) -> double { return (double)x[nid(p, a, b, c)]; };
    double s = -X(i, j, k) * 1470.0;
#pragma unroll
    for (int d = 1; d <= 3; ++d) {
        const double w = d == 1 ? 270.0 : (d == 2 ? -27.0 : 2.0);
        s += w * (X(wrap_off(i + d, p.dx), j, k) + X(wrap_off(i - d, p.dx), j, k) + X(i, wrap_off(j + d, p.dy), k) +
                  X(i, wrap_off(j - d, p.dy), k) + X(i, j, wrap_off(k + d, p.dz)) + X(i, j, wrap_off(k - d, p.dz)));
    }
    return s / 180.0;
}

// R4: chemical-potential adjoint; per-block FP64 partials of dJ/dka.
template <class R>
__global__ void __launch_bounds__(128) k_adj_mu(KParams<R> p, const uint8_t *type, const R *rho, const R *lammu,
                                                R *lamrho, double *ka_part)
{
    __shared__ double red[128];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    double gka = 0.0;
    if (k < p.dz) {
        const long long I = ((long long)i * p.dy + j) * p.dz + k;
        // Laplacian of lam_mu restricted to fluid nodes (symmetric stencil)
        auto lm = [&](int ii, int jj, int kk) -> R {
            const long long J = nid(p, ii, jj, kk);
            return type[J] == FLUID ? lammu[J] : R(0);
        };
        R lap;
        if (p.lap_order == 7) {
            int a[7], b[7], c[7];
#pragma unroll
            for (int d = -3; d <= 3; ++d) {
                a[d + 3] = wrap_off(i + d, p.dx);
                b[d + 3] = wrap_off(j + d, p.dy);
                c[d + 3] = wrap_off(k + d, p.dz);
            }
            lap = -lm(i, j, k) * R(1470);
#pragma unroll
            for (int d = 1; d <= 3; ++d) {
                const R w = d == 1 ? R(270) : (d == 2 ? R(-27) : R(2));
                lap += w * (lm(a[3 + d], j, k) + lm(a[3 - d], j, k) + lm(i, b[3 + d], k) + lm(i, b[3 - d], k) +
                            lm(i, j, c[3 + d]) + lm(i, j, c[3 - d]));
            }
            lap /= R(180);
        } else {
            const int im2 = wrap_off(i - 2, p.dx), im1 = wrap_off(i - 1, p.dx), ip1 = wrap_off(i + 1, p.dx),
                      ip2 = wrap_off(i + 2, p.dx);
            const int jm2 = wrap_off(j - 2, p.dy), jm1 = wrap_off(j - 1, p.dy), jp1 = wrap_off(j + 1, p.dy),
                      jp2 = wrap_off(j + 2, p.dy);
            const int km2 = wrap_off(k - 2, p.dz), km1 = wrap_off(k - 1, p.dz), kp1 = wrap_off(k + 1, p.dz),
                      kp2 = wrap_off(k + 2, p.dz);
            lap = (-lm(i, j, k) * R(90) + (-lm(im2, j, k) + lm(im1, j, k) * R(16) + lm(ip1, j, k) * R(16) - lm(ip2, j, k)) +
                   (-lm(i, jm2, k) + lm(i, jm1, k) * R(16) + lm(i, jp1, k) * R(16) - lm(i, jp2, k)) +
                   (-lm(i, j, km2) + lm(i, j, km1) * R(16) + lm(i, j, kp1) * R(16) - lm(i, j, kp2))) /
                  R(12);
        }
        R add = -p.ka * lap;
        if (type[I] == FLUID) {
            const R r = rho[I];
            add += p.kk * dmu0<R>(p.eos, p.A, p.B, p.T, r) * lammu[I];
            // the Laplacian of this term in FP64: it is a small difference of
            // O(rho_l) values summed over every node and step
            const double lr = p.lap_order == 7 ? lap7_d(p, rho, i, j, k) : lap5_d(p, rho, i, j, k);
            gka = -(double)lammu[I] * lr;
        }
        lamrho[I] += add;
    }
    red[threadIdx.x] = gka;
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        ka_part[((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = red[0];
}

// R5: wall adjoint per column; pass 0 also gathers dJ/dw from the solid mu.
template <class R>
__global__ void k_adj_wall(KParams<R> p, int pass, const R *lammu, R *lamrho, double *gwall)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)p.dx * p.dy) return;
    const int i = (int)(c / p.dy), j = (int)(c % p.dy), D = p.dz;
    // E^T = E: (2 centre + 4 xy-diagonal neighbours) / 6 of the adjoint layer
    auto E = [&](int kk) -> R { return wall_extrap<R>(p, lamrho, i, j, kk); };
    if (pass == 0) {
        const long long np = (long long)p.dx * p.dy;
        gwall[c] += (double)lammu[nid(p, i, j, 0)] + (double)lammu[nid(p, i, j, 1)] + (double)lammu[nid(p, i, j, 2)];
        gwall[np + c] += (double)lammu[nid(p, i, j, D - 3)] + (double)lammu[nid(p, i, j, D - 2)] +
                         (double)lammu[nid(p, i, j, D - 1)];
    }
    if (p.complex_bc) {
        // forward: L2 = E(L3), L1 = E(L2), L0 = E(L1)  ->  reverse in the opposite order
        if (pass == 0) {
            const R b = E(0), t = E(D - 1);
            lamrho[nid(p, i, j, 1)] += b;
            lamrho[nid(p, i, j, D - 2)] += t;
        } else if (pass == 1) {
            const R b = E(1), t = E(D - 2);
            lamrho[nid(p, i, j, 2)] += b;
            lamrho[nid(p, i, j, D - 3)] += t;
        } else {
            const R b = E(2), t = E(D - 3);
            lamrho[nid(p, i, j, 3)] += b;
            lamrho[nid(p, i, j, D - 4)] += t;
        }
    } else if (pass == 0) {
        // forward: L0 = L1 = L2 = E(L3)
        const R b = E(0) + E(1) + E(2), t = E(D - 1) + E(D - 2) + E(D - 3);
        lamrho[nid(p, i, j, 3)] += b;
        lamrho[nid(p, i, j, D - 4)] += t;
    }
}

// Loss J = sum over fluid nodes of (rho - target)^2 (FP64 partials) and the
// terminal adjoint dJ/df^T_q = 2 (rho - target) for every q, in factored
// form: lamp = 0, lamrho = 2 (rho - target).
template <class R>
__global__ void __launch_bounds__(128) k_adj_loss(KParams<R> p, const uint8_t *type, const R *rho,
                                                  const double *target, R *lamp, R *lamrho, double *part)
{
    __shared__ double red[128];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    double l = 0.0;
    if (k < p.dz) {
        const long long I = ((long long)i * p.dy + j) * p.dz + k;
        R g = R(0);
        if (type[I] == FLUID) {
            const double d = (double)rho[I] - target[I];
            l = d * d;
            g = (R)(2.0 * d);
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) lamp[q * p.n + I] = R(0);
        lamrho[I] = g;
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = red[0];
}

// Sum of nb doubles in fixed order, added to *acc (single thread block).
static __global__ void k_adj_sum(const double *part, long long nb, double *acc, int add)
{
    __shared__ double red[256];
    double s = 0.0;
    for (long long b = threadIdx.x; b < nb; b += blockDim.x) s += part[b];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *acc = (add ? *acc : 0.0) + red[0];
}

// ------------------------------------------------------------ launchers ----

template <class R>
void adj_launch_loss(const KParams<R> &p, const uint8_t *type, const R *rho, const double *target, AdjBufs<R> &b,
                     cudaStream_t st)
{
    const dim3 g = grid3(p, 128);
    k_adj_loss<R><<<g, 128, 0, st>>>(p, type, rho, target, b.lamp_next, b.lamrho_next, b.ka_part);
    k_adj_sum<<<1, 256, 0, st>>>(b.ka_part, (long long)g.x * g.y * g.z, b.loss, 0);
}

// One reverse step.  rho/u/mu/F hold the forward intermediates of step n
// (recomputed from f^n by the caller); (b.lamp_next, b.lamrho_next) =
// dJ/df^{n+1} on entry, (b.lamp, b.lamrho) = dJ/df^n on exit.
template <class R>
void adj_launch_step(const KParams<R> &p, const uint8_t *type, const R *rho, const R *u, const R *mu, const R *F,
                     AdjBufs<R> &b, cudaStream_t st)
{
    const dim3 g = grid3(p, 128);
    k_adj_collide<R><<<g, 128, 0, st>>>(p, type, rho, u, F, b.lamp_next, b.lamrho_next, b.lamp, b.lamF,
                                        b.lamrho);
    k_adj_force<R><<<g, 128, 0, st>>>(p, type, rho, mu, b.lamF, b.lammu, b.lamrho);
    k_adj_mu<R><<<g, 128, 0, st>>>(p, type, rho, b.lammu, b.lamrho, b.ka_part);
    k_adj_sum<<<1, 256, 0, st>>>(b.ka_part, (long long)g.x * g.y * g.z, b.gka, 1);
    if (p.wall_mode == 1) {
        const long long np = (long long)p.dx * p.dy;
        const unsigned gw = (unsigned)((np + 127) / 128);
        for (int s = 0; s < (p.complex_bc ? 3 : 1); ++s) k_adj_wall<R><<<gw, 128, 0, st>>>(p, s, b.lammu, b.lamrho, b.gwall);
    }
}

}  // namespace cpmp
