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
//       dJ/drho(y) += -sum_a G_a(lamF_a)(y)/3 - lamF(y).G(mu)(y); R2 hands
//       lamF over packed with rho, (lamF_x, lamF_y, lamF_z, rho) per node, so
//       each stencil point is one vector load; G(mu) is the one the forward
//       replay stored
//       (the gradient stencils are antisymmetric, so their transpose is the
//       negated stencil)
//   R4  k_adj_mu      : dJ/drho(y) += K^2 mu0'(rho) lam_mu - ka Lap(lam_mu on
//       fluid)(y) (the Laplacian is symmetric); dJ/dka += -sum lam_mu Lap(rho),
//       products and sums in FP64
//   R5  k_adj_wall    : wall layers back onto the first fluid layer (the
//       6-point average is symmetric), dJ/dw += lam_mu on the solid layers;
//       one launch for all three layers
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

// Neighbour (i+a, j+b, k+c) of node I: plain offsets for nodes at least
// `radius` away from every face (INTERIOR), periodic wrap otherwise.
template <bool INTERIOR, class R>
struct Nb {
    const KParams<R> &p;
    int i, j, k;
    long long I, plane;
    __device__ __forceinline__ long long operator()(int a, int b, int c) const
    {
        if (INTERIOR) return I + a * plane + (long long)b * p.dz + c;
        return nid(p, wrap_off(i + a, p.dx), wrap_off(j + b, p.dy), wrap_off(k + c, p.dz));
    }
};
template <class R>
__device__ __forceinline__ bool interior_node(const KParams<R> &p, int i, int j, int k, int radius)
{
    return i >= radius && i < p.dx - radius && j >= radius && j < p.dy - radius && k >= radius && k < p.dz - radius;
}

// R2: collision + streaming adjoint (one thread per node, 3-D grid).
template <class R>
__global__ void __launch_bounds__(128) k_adj_collide(KParams<R> p, const uint8_t *type, const R *rho,
                                                     const R *u, const R *F, const R *lamp_next,
                                                     const R *lamrho_next, R *lamp, Pack4<R> *lamF,
                                                     R *lamrho)
{
    NODE3D(p);
    const long long n = p.n;
    if (type[I] != FLUID) {
#pragma unroll
        for (int q = 0; q < Q; ++q) lamp[q * n + I] = R(0);
        lamF[I] = Pack4<R>{R(0), R(0), R(0), rho[I]};
        lamrho[I] = R(0);
        return;
    }
    // lambda* (adjoint of the post-collision populations): pull through the
    // push streaming; a population bounced back at a solid destination came
    // back into slot opp(q) of this node
    R ls[Q];
    const R lr_here = lamrho_next[I];
    auto gather = [&](auto nb, auto CHECK) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const long long D = nb(cx(q), cy(q), cz(q));
            const bool dfl = decltype(CHECK)::value ? type[D] == FLUID : true;
            ls[q] = dfl ? lamp_next[q * n + D] + lamrho_next[D] : lamp_next[opp(q) * n + I] + lr_here;
        }
    };
    const long long plane = (long long)p.dy * p.dz;
    // node tags are the wall layers alone, so a node at least two layers
    // from the walls has fluid neighbours only
    const bool no_wall = p.wall_mode == 0 || (k >= 4 && k <= p.dz - 5);
    if (interior_node(p, i, j, k, 1) && no_wall)
        gather(Nb<true, R>{p, i, j, k, I, plane}, std::false_type{});
    else if (interior_node(p, i, j, k, 1))
        gather(Nb<true, R>{p, i, j, k, I, plane}, std::true_type{});
    else
        gather(Nb<false, R>{p, i, j, k, I, plane}, std::true_type{});
    // mu* = M^-T lambda* = diag(1/norm) M lambda*
    R ms[Q];
    moments<R>(ls, ms);
    const R inv_norm[Q] = {R(1) / R(19), R(1) / R(2394), R(1) / R(252), R(0.1), R(0.025), R(0.1), R(0.025),
                           R(0.1),       R(0.025),       R(1) / R(36),  R(1) / R(72), R(1) / R(12), R(1) / R(24),
                           R(0.25),      R(0.25),        R(0.25),       R(0.125),     R(0.125),     R(0.125)};
    // y = (1 - S) M lambda*; the adjoint weights of meq(u) and meq(u + F/rho)
    // are a0 = -diag(1/norm) y and a1 = diag(1/norm) M lambda*
    R y[Q], a0[Q], a1[Q];
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        y[a] = p.omts[a] * ms[a];
        a0[a] = -y[a] * inv_norm[a];
        a1[a] = ms[a] * inv_norm[a];
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
    lamF[I] = Pack4<R>{av1x * ir, av1y * ir, av1z * ir, r};
    a_rho -= (av1x * Fx + av1y * Fy + av1z * Fz) * ir * ir;
    // u = j / rho
    const R ajx = aux * ir, ajy = auy * ir, ajz = auz * ir;
    a_rho -= (aux * ux + auy * uy + auz * uz) * ir;
    lamrho[I] = a_rho;
    // m = M f -> M^T (diag(1/norm) y) = M^-1 y ;  j = sum e f -> e . aj
    R fm[Q];
    inverse_moments<R>(y, fm);
#pragma unroll
    for (int q = 0; q < Q; ++q) lamp[q * n + I] = fm[q] + R(cx(q)) * ajx + R(cy(q)) * ajy + R(cz(q)) * ajz;
}

// R3: force adjoint.  A CTA owns an FF_Y x FT_Z column tile and marches
// over FT_X planes of x; the packed (lamF, rho) of planes x-3 .. x+3 with a
// halo of 3 in y and z sit in an eight-plane shared-memory ring (plane x+4 is
// copied in with cp.async while plane x is computed), so every one of the 54
// stencil points of a node is one shared-memory vector load and each global
// value is loaded once per CTA plus halo.  Periodic wrap in y and z comes from
// per-CTA coordinate tables, in x from the plane index.
constexpr int FT_Y = 8, FT_Z = 32, FT_X = 16;  // R4's tile
constexpr int FH_Y = FT_Y + 6, FH_Z = FT_Z + 6;
constexpr int FF_Y = 4, FFH_Y = FF_Y + 6;      // R3's tile height (its 16-byte ring rows are larger)
// CTAs of the tiled R3 / R4 launches
__host__ __device__ constexpr long long adj_mu_blocks(int dx, int dy, int dz)
{
    return (long long)((dz + FT_Z - 1) / FT_Z) * ((dy + FT_Y - 1) / FT_Y) * ((dx + FT_X - 1) / FT_X);
}
template <class R>
constexpr size_t adj_force_smem()
{
    return sizeof(Pack4<R>) * 8 * FFH_Y * FH_Z + sizeof(int) * (FFH_Y + FH_Z);
}
template <class R>
__global__ void __launch_bounds__(FF_Y *FT_Z) k_adj_force(KParams<R> p, const uint8_t *type, const R *gm,
                                                           const Pack4<R> *lamF, R *lammu, Pack2<R> *lmr, R *lamrho)
{
    extern __shared__ __align__(16) unsigned char fsm[];
    Pack4<R> *ring = reinterpret_cast<Pack4<R> *>(fsm);
    int *tabY = reinterpret_cast<int *>(ring + 8 * FFH_Y * FH_Z);
    int *tabZ = tabY + FFH_Y;
    constexpr int NT = FF_Y * FT_Z, PL = FFH_Y * FH_Z;
    const int z0 = blockIdx.x * FT_Z, y0 = blockIdx.y * FF_Y, x0 = blockIdx.z * FT_X;
    const int x1 = min(x0 + FT_X, p.dx);
    const long long n = p.n;
    for (int e = threadIdx.x; e < FFH_Y + FH_Z; e += NT) {
        if (e < FFH_Y) tabY[e] = wrap_off(y0 - 3 + e, p.dy);
        else tabZ[e - FFH_Y] = wrap_off(z0 - 3 + (e - FFH_Y), p.dz);
    }
    __syncthreads();
    auto slot = [](int x) { return x & 7; };
    auto load = [&](int x) {
        const long long base = (long long)wrap_off(x, p.dx) * p.dy;
        Pack4<R> *dst = ring + slot(x) * PL;
        for (int e = threadIdx.x; e < PL; e += NT) {
            const int ly = e / FH_Z, lz = e - ly * FH_Z;
            const Pack4<R> *src = lamF + (base + tabY[ly]) * p.dz + tabZ[lz];
#pragma unroll
            for (int b = 0; b < (int)sizeof(Pack4<R>); b += 16) {
                const unsigned sa = (unsigned)__cvta_generic_to_shared(reinterpret_cast<char *>(dst + e) + b);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa),
                             "l"(reinterpret_cast<const char *>(src) + b)
                             : "memory");
            }
        }
    };
    for (int x = x0 - 3; x <= x0 + 3; ++x) load(x);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    const int tz = threadIdx.x % FT_Z, ty = threadIdx.x / FT_Z;
    const int j = y0 + ty, k = z0 + tz;
    const bool active = j < p.dy && k < p.dz;
    const int c = (ty + 3) * FH_Z + (tz + 3);
    for (int x = x0; x < x1; ++x) {
        load(x + 4);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // planes up to x+3 have landed
        __syncthreads();
        if (active) {
            const long long I = ((long long)x * p.dy + j) * p.dz + k;
            // for each lattice line (sx, sy, sz) with weight vector w (2 e on
            // the axes, e on the diagonals): sum_d c_d (v(+d) - v(-d)) of
            // v = w . lamF and of rho v; only the nonzero components of w enter
            R sm = R(0), sr = R(0);
            auto acc = [&](auto SX, auto SY, auto SZ) {
                constexpr int sx = decltype(SX)::value, sy = decltype(SY)::value, sz = decltype(SZ)::value;
                constexpr int axis = (sx != 0) + (sy != 0) + (sz != 0) == 1;
                constexpr int wx = axis ? 2 * sx : sx, wy = axis ? 2 * sy : sy, wz = axis ? 2 * sz : sz;
                auto lw = [&](const Pack4<R> &v4) -> R {
                    R v = R(0);
                    if constexpr (wx != 0) v += R(wx) * v4.x;
                    if constexpr (wy != 0) v += R(wy) * v4.y;
                    if constexpr (wz != 0) v += R(wz) * v4.z;
                    return v;
                };
#pragma unroll
                for (int d = 1; d <= 3; ++d) {
                    const R cd = d == 1 ? R(45) : (d == 2 ? R(-9) : R(1));
                    const int o = sy * d * FH_Z + sz * d;
                    const Pack4<R> vp = ring[slot(x + sx * d) * PL + c + o];
                    const Pack4<R> vm = ring[slot(x - sx * d) * PL + c - o];
                    const R lp = lw(vp), lm = lw(vm);
                    sm += cd * (vp.w * lp - vm.w * lm);
                    sr += cd * (lp - lm);
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
            const R lmu = sm * R(1.0 / 360.0);
            const bool fl = type[I] == FLUID;
            const Pack4<R> own = ring[slot(x) * PL + c];
            lammu[I] = lmu;
            lmr[I] = Pack2<R>{fl ? lmu : R(0), own.w};  // lam_mu on fluid nodes and rho, for R4
            R add = -sr * R(1.0 / 1080.0);
            if (fl)  // grad(mu) of the forward step, stored by its replay
                add -= own.x * gm[I] + own.y * gm[I + n] + own.z * gm[I + 2 * n];
            lamrho[I] += add;
        }
        __syncthreads();  // plane x-3's slot is refilled with x+5 next
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// R4: chemical-potential adjoint, tiled like R3: an eight-plane ring of the
// packed (lam_mu on fluid nodes, rho) with halo 3 (cp.async one plane
// ahead); the Laplacians of both are read from shared memory.  Each CTA adds
// its FP64 partial of dJ/dka to its own running sum (fixed order, so the
// result is deterministic).
template <class R>
constexpr size_t adj_mu_smem()
{
    return sizeof(Pack2<R>) * 8 * FH_Y * FH_Z + sizeof(int) * (FH_Y + FH_Z);
}
template <class R>
__global__ void __launch_bounds__(FT_Y *FT_Z) k_adj_mu(KParams<R> p, const uint8_t *type, const Pack2<R> *lmr,
                                                        R *lamrho, double *ka_part)
{
    extern __shared__ __align__(16) unsigned char msm[];
    Pack2<R> *ring = reinterpret_cast<Pack2<R> *>(msm);
    int *tabY = reinterpret_cast<int *>(ring + 8 * FH_Y * FH_Z);
    int *tabZ = tabY + FH_Y;
    __shared__ double red[FT_Y * FT_Z / 32];
    constexpr int NT = FT_Y * FT_Z, PL = FH_Y * FH_Z;
    const int z0 = blockIdx.x * FT_Z, y0 = blockIdx.y * FT_Y, x0 = blockIdx.z * FT_X;
    const int x1 = min(x0 + FT_X, p.dx);
    for (int e = threadIdx.x; e < FH_Y + FH_Z; e += NT) {
        if (e < FH_Y) tabY[e] = wrap_off(y0 - 3 + e, p.dy);
        else tabZ[e - FH_Y] = wrap_off(z0 - 3 + (e - FH_Y), p.dz);
    }
    __syncthreads();
    auto load = [&](int x) {
        const long long base = (long long)wrap_off(x, p.dx) * p.dy;
        Pack2<R> *dst = ring + (x & 7) * PL;
        for (int e = threadIdx.x; e < PL; e += NT) {
            const int ly = e / FH_Z, lz = e - ly * FH_Z;
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + e);
            const Pack2<R> *src = lmr + (base + tabY[ly]) * p.dz + tabZ[lz];
            if (sizeof(Pack2<R>) == 8)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(src) : "memory");
            else
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
        }
    };
    for (int x = x0 - 3; x <= x0 + 3; ++x) load(x);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    const int tz = threadIdx.x % FT_Z, ty = threadIdx.x / FT_Z;
    const int j = y0 + ty, k = z0 + tz;
    const bool active = j < p.dy && k < p.dz;
    const int c = (ty + 3) * FH_Z + (tz + 3);
    double gka = 0.0;
    for (int x = x0; x < x1; ++x) {
        load(x + 4);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // planes up to x+3 have landed
        __syncthreads();
        if (active) {
            const long long I = ((long long)x * p.dy + j) * p.dz + k;
            // the two Laplacians (the stencil is symmetric, so the adjoint's
            // is the forward's): .x = lam_mu restricted to fluid, .y = rho
            auto at = [&](int a, int b, int cc) -> const Pack2<R> & {
                return ring[((x + a) & 7) * PL + c + b * FH_Z + cc];
            };
            R lx, ly;
            if (p.lap_order == 7) {
                const Pack2<R> &o = at(0, 0, 0);
                lx = -o.x * R(1470);
                ly = -o.y * R(1470);
#pragma unroll
                for (int d = 1; d <= 3; ++d) {
                    const R w = d == 1 ? R(270) : (d == 2 ? R(-27) : R(2));
                    const Pack2<R> &a1 = at(d, 0, 0), &a2 = at(-d, 0, 0), &a3 = at(0, d, 0), &a4 = at(0, -d, 0),
                                   &a5 = at(0, 0, d), &a6 = at(0, 0, -d);
                    lx += w * (a1.x + a2.x + a3.x + a4.x + a5.x + a6.x);
                    ly += w * (a1.y + a2.y + a3.y + a4.y + a5.y + a6.y);
                }
                lx *= R(1.0 / 180.0);
                ly *= R(1.0 / 180.0);
            } else {
                auto l5 = [&](auto f) -> R {
                    return (-f(0, 0, 0) * R(90) + (-f(-2, 0, 0) + f(-1, 0, 0) * R(16) + f(1, 0, 0) * R(16) - f(2, 0, 0)) +
                            (-f(0, -2, 0) + f(0, -1, 0) * R(16) + f(0, 1, 0) * R(16) - f(0, 2, 0)) +
                            (-f(0, 0, -2) + f(0, 0, -1) * R(16) + f(0, 0, 1) * R(16) - f(0, 0, 2))) *
                           R(1.0 / 12.0);
                };
                lx = l5([&](int a, int b, int cc) { return at(a, b, cc).x; });
                ly = l5([&](int a, int b, int cc) { return at(a, b, cc).y; });
            }
            R add = -p.ka * lx;
            if (type[I] == FLUID) {
                const Pack2<R> &o = at(0, 0, 0);
                add += p.kk * dmu0<R>(p.eos, p.A, p.B, p.T, o.y) * o.x;
                gka += -(double)o.x * (double)ly;
            }
            lamrho[I] += add;
        }
        __syncthreads();  // plane x-3's slot is refilled with x+5 next
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    // warp shuffles, then the warp sums in order (deterministic)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gka += __shfl_down_sync(0xffffffffu, gka, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = gka;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < NT / 32; ++w) t += red[w];
        ka_part[((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] += t;
    }
}

// R5: wall adjoint in one launch.  The forward sets layer 2 = E(layer 3),
// layer 1 = E(layer 2), layer 0 = E(layer 1) (or all three = E(layer 3) for
// the single-layer rule), E = (2 centre + 4 xy-diagonal neighbours) / 6
// with periodic wrap, which is symmetric (E^T = E).  Reversed:
// lam1 += E(lam0), lam2 += E(lam1), lam3 += E(lam2).  A CTA owns a 16 x 16
// tile of wall columns of one wall (blockIdx.z: 0 bottom, 1 top); it stages
// the three solid layers' adjoints with halos 3, 2 and 1 in shared memory,
// runs the chain there, and adds the result to the fluid layer next to the
// wall (only that layer's adjoint is read afterwards).  dJ/dw gathers lam_mu
// of the three solid layers.
constexpr int WT = 16;  // wall tile edge (columns)
template <class R>
__global__ void __launch_bounds__(256) k_adj_wall(KParams<R> p, const R *lammu, R *lamrho, double *gwall)
{
    __shared__ R s0[WT + 6][WT + 6], s1[WT + 4][WT + 4], s2[WT + 2][WT + 2];
    const bool top = blockIdx.z == 1;
    const int D = p.dz;
    const int kl0 = top ? D - 1 : 0, kl1 = top ? D - 2 : 1, kl2 = top ? D - 3 : 2, kf = top ? D - 4 : 3;
    const int i0 = blockIdx.x * WT, j0 = blockIdx.y * WT;
    auto col = [&](int a, int b, int k) -> long long {
        return nid(p, wrap_off(a, p.dx), wrap_off(b, p.dy), k);
    };
    if (p.complex_bc) {
        for (int e = threadIdx.x; e < (WT + 6) * (WT + 6); e += blockDim.x) {
            const int a = e / (WT + 6), b = e % (WT + 6);
            s0[a][b] = lamrho[col(i0 - 3 + a, j0 - 3 + b, kl0)];
            if (a < WT + 4 && b < WT + 4) s1[a][b] = lamrho[col(i0 - 2 + a, j0 - 2 + b, kl1)];
            if (a < WT + 2 && b < WT + 2) s2[a][b] = lamrho[col(i0 - 1 + a, j0 - 1 + b, kl2)];
        }
        __syncthreads();
        for (int e = threadIdx.x; e < (WT + 4) * (WT + 4); e += blockDim.x) {
            const int a = e / (WT + 4) + 1, b = e % (WT + 4) + 1;  // centre in s0 coordinates
            s1[a - 1][b - 1] += (s0[a][b] * R(2) + s0[a - 1][b - 1] + s0[a - 1][b + 1] + s0[a + 1][b - 1] +
                                 s0[a + 1][b + 1]) / R(6);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < (WT + 2) * (WT + 2); e += blockDim.x) {
            const int a = e / (WT + 2) + 1, b = e % (WT + 2) + 1;  // centre in s1 coordinates
            s2[a - 1][b - 1] += (s1[a][b] * R(2) + s1[a - 1][b - 1] + s1[a - 1][b + 1] + s1[a + 1][b - 1] +
                                 s1[a + 1][b + 1]) / R(6);
        }
        __syncthreads();
    }
    const int a = threadIdx.x / WT, b = threadIdx.x % WT;
    const int i = i0 + a, j = j0 + b;
    if (i >= p.dx || j >= p.dy) return;
    const long long np = (long long)p.dx * p.dy, c = (long long)i * p.dy + j;
    gwall[(top ? np : 0) + c] += (double)lammu[nid(p, i, j, kl0)] + (double)lammu[nid(p, i, j, kl1)] +
                                 (double)lammu[nid(p, i, j, kl2)];
    R add;
    if (p.complex_bc) {
        add = (s2[a + 1][b + 1] * R(2) + s2[a][b] + s2[a][b + 2] + s2[a + 2][b] + s2[a + 2][b + 2]) / R(6);
    } else {
        auto Ls = [&](int aa, int bb) {
            return lamrho[col(aa, bb, kl0)] + lamrho[col(aa, bb, kl1)] + lamrho[col(aa, bb, kl2)];
        };
        add = (Ls(i, j) * R(2) + Ls(i - 1, j - 1) + Ls(i - 1, j + 1) + Ls(i + 1, j - 1) + Ls(i + 1, j + 1)) / R(6);
    }
    lamrho[nid(p, i, j, kf)] += add;
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
    cudaMemsetAsync(b.ka_acc, 0, sizeof(double) * adj_mu_blocks(p.dx, p.dy, p.dz), st);
}

// dJ/dka: the per-block sums of every reverse step, added up in fixed order.
template <class R>
void adj_launch_finish(const KParams<R> &p, AdjBufs<R> &b, cudaStream_t st)
{
    const dim3 g = grid3(p, 128);
    k_adj_sum<<<1, 256, 0, st>>>(b.ka_acc, adj_mu_blocks(p.dx, p.dy, p.dz), b.gka, 0);
}

// One reverse step.  rho/u/gm/F hold the forward intermediates of step n
// (density with its wall layers, velocity, grad mu, force; recomputed from
// f^n by the caller); (b.lamp_next, b.lamrho_next) = dJ/df^{n+1} on entry,
// (b.lamp, b.lamrho) = dJ/df^n on exit.
template <class R>
void adj_launch_step(const KParams<R> &p, const uint8_t *type, const R *rho, const R *u, const R *gm, const R *F,
                     AdjBufs<R> &b, cudaStream_t st, LaunchHook *hook)
{
    const dim3 g = grid3(p, 128);
    Pack4<R> *lamF = reinterpret_cast<Pack4<R> *>(b.lamF);
    hook_begin(hook, K_ADJ_COLLIDE, st);
    k_adj_collide<R><<<g, 128, 0, st>>>(p, type, rho, u, F, b.lamp_next, b.lamrho_next, b.lamp, lamF, b.lamrho);
    hook_end(hook, K_ADJ_COLLIDE, st);
    {
        // shared-memory opt-in (FP64 needs more than 48 KB), once per device
        static int attr_dev = -1;
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev != attr_dev) {
            cudaFuncSetAttribute(k_adj_force<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)adj_force_smem<R>());
            cudaFuncSetAttribute(k_adj_mu<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_mu_smem<R>());
            attr_dev = dev;
        }
        const dim3 gff((unsigned)((p.dz + FT_Z - 1) / FT_Z), (unsigned)((p.dy + FF_Y - 1) / FF_Y),
                       (unsigned)((p.dx + FT_X - 1) / FT_X));
        const dim3 gf((unsigned)((p.dz + FT_Z - 1) / FT_Z), (unsigned)((p.dy + FT_Y - 1) / FT_Y),
                      (unsigned)((p.dx + FT_X - 1) / FT_X));
        hook_begin(hook, K_ADJ_FORCE, st);
        k_adj_force<R><<<gff, FF_Y * FT_Z, adj_force_smem<R>(), st>>>(p, type, gm, lamF, b.lammu, b.lmr, b.lamrho);
        hook_end(hook, K_ADJ_FORCE, st);
        hook_begin(hook, K_ADJ_MU, st);
        k_adj_mu<R><<<gf, FT_Y * FT_Z, adj_mu_smem<R>(), st>>>(p, type, b.lmr, b.lamrho, b.ka_acc);
        hook_end(hook, K_ADJ_MU, st);
    }
    if (p.wall_mode == 1) {
        const dim3 gw((unsigned)((p.dx + WT - 1) / WT), (unsigned)((p.dy + WT - 1) / WT), 2);
        hook_begin(hook, K_ADJ_WALL, st);
        k_adj_wall<R><<<gw, WT * WT, 0, st>>>(p, b.lammu, b.lamrho, b.gwall);
        hook_end(hook, K_ADJ_WALL, st);
    }
}

}  // namespace cpmp
