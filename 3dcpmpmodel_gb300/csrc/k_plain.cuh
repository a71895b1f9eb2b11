// k_plain.cuh -- the PLAIN scheme: one kernel per reference kernel, two
// population lattices, the reference's launch order (FluidCuda.cu:1279-1291).
// Included by k_plain_f32.cu (FP32, default FMA contraction) and
// k_plain_f64.cu (FP64, compiled without FMA contraction so its results stay
// within a few ulp of the FP64 CPU restatement).
#pragma once

#include "lbm_core.cuh"
#include "launch.h"

namespace cpmp {

__device__ __forceinline__ int wrap_off(int a, int n)
{
    while (a < 0) a += n;
    while (a >= n) a -= n;
    return a;
}

// Node of a 3-D launch: grid (z blocks, DY, DX), threads along z.
#define NODE3D(p)                                                        \
    const int k = blockIdx.x * blockDim.x + threadIdx.x;                 \
    const int j = blockIdx.y, i = blockIdx.z;                            \
    if (k >= (p).dz) return;                                             \
    const long long I = ((long long)i * (p).dy + j) * (p).dz + k

template <class R>
__host__ __forceinline__ dim3 grid3(const KParams<R> &p, int bs)
{
    return dim3((unsigned)((p.dz + bs - 1) / bs), (unsigned)p.dy, (unsigned)p.dx);
}

template <class R>
__device__ __forceinline__ long long nid(const KParams<R> &p, int i, int j, int k)
{
    return ((long long)i * p.dy + j) * p.dz + k;
}

// ----------------------------------------------------------------- init ----
// SetFlowField (FluidCuda.cu:199-241): tags, tanh droplet, solid rho = mu =
// wall potential, f = feq(rho, 0), u = 0.  The droplet radius is evaluated in
// double (the reference's placement takes sqrtf of the squared distance).
template <class R, class S>
__global__ void k_init_plain(KParams<R> p, DropletDev d, uint8_t *type, R *rho, R *mu, R *u,
                             S *f)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    const int k = (int)(I % p.dz), j = (int)((I / p.dz) % p.dy), i = (int)(I / p.dz / p.dy);
    double r0;
    if (solid_k(p.wall_mode, k, p.dz)) {
        type[I] = SOLID;
        const R w = p.wall[(k < 3 ? 0 : (long long)p.dx * p.dy) + (long long)i * p.dy + j];
        rho[I] = w;
        mu[I] = w;
        r0 = (double)w;
    } else {
        type[I] = FLUID;
        mu[I] = R(0);
        r0 = droplet_density(d, i, j, k, p.dx, p.dy);
        rho[I] = (R)r0;
    }
    u[I] = u[I + p.n] = u[I + 2 * p.n] = R(0);
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q * p.n + I] = (S)(r0 * wgt<double>(q));
}

// ----------------------------------------------------------- wall layer ----
// ChemBoundary (FluidCuda.cu:376-401), one launch per layer pass so that the
// layered extrapolation is deterministic:
//   pass 0: layers 0,1,2 <- E(layer 3), layers DZ-3..DZ-1 <- E(layer DZ-4),
//           solid mu <- wall potential;
//   pass 1: layer 1 <- E(layer 2), layer DZ-2 <- E(layer DZ-3);
//   pass 2: layer 0 <- E(layer 1), layer DZ-1 <- E(layer DZ-2);
// with E = (2 centre + four xy-diagonal neighbours) / 6.
template <class R>
__device__ __forceinline__ R wall_extrap(const KParams<R> &p, const R *rho, int i, int j, int k)
{
    const int i1 = i > 0 ? i - 1 : p.dx - 1, i2 = i < p.dx - 1 ? i + 1 : 0;
    const int j1 = j > 0 ? j - 1 : p.dy - 1, j2 = j < p.dy - 1 ? j + 1 : 0;
    return (rho[nid(p, i, j, k)] * R(2) + rho[nid(p, i1, j1, k)] + rho[nid(p, i1, j2, k)] +
            rho[nid(p, i2, j1, k)] + rho[nid(p, i2, j2, k)]) / R(6);
}

template <class R>
__device__ __forceinline__ void wall_column(const KParams<R> &p, int pass, long long c, R *rho, R *mu, R *mirror)
{
    const int i = (int)(c / p.dy), j = (int)(c % p.dy);
    const int D = p.dz;
    if (pass == 0) {
        const R b = wall_extrap(p, rho, i, j, 3), t = wall_extrap(p, rho, i, j, D - 4);
        rho[nid(p, i, j, 0)] = rho[nid(p, i, j, 1)] = rho[nid(p, i, j, 2)] = b;
        rho[nid(p, i, j, D - 3)] = rho[nid(p, i, j, D - 2)] = rho[nid(p, i, j, D - 1)] = t;
        if (mirror) {
            mirror[nid(p, i, j, 0)] = mirror[nid(p, i, j, 1)] = mirror[nid(p, i, j, 2)] = b;
            mirror[nid(p, i, j, D - 3)] = mirror[nid(p, i, j, D - 2)] = mirror[nid(p, i, j, D - 1)] = t;
        }
        if (mu) {
            const R wb = p.wall[c], wt = p.wall[(long long)p.dx * p.dy + c];
            mu[nid(p, i, j, 0)] = mu[nid(p, i, j, 1)] = mu[nid(p, i, j, 2)] = wb;
            mu[nid(p, i, j, D - 3)] = mu[nid(p, i, j, D - 2)] = mu[nid(p, i, j, D - 1)] = wt;
        }
    } else if (pass == 1) {
        const R b = wall_extrap(p, rho, i, j, 2), t = wall_extrap(p, rho, i, j, D - 3);
        rho[nid(p, i, j, 1)] = b;
        rho[nid(p, i, j, D - 2)] = t;
        if (mirror) {
            mirror[nid(p, i, j, 1)] = b;
            mirror[nid(p, i, j, D - 2)] = t;
        }
    } else {
        const R b = wall_extrap(p, rho, i, j, 1), t = wall_extrap(p, rho, i, j, D - 2);
        rho[nid(p, i, j, 0)] = b;
        rho[nid(p, i, j, D - 1)] = t;
        if (mirror) {
            mirror[nid(p, i, j, 0)] = b;
            mirror[nid(p, i, j, D - 1)] = t;
        }
    }
}

template <class R>
__global__ void k_wall_pass(KParams<R> p, int pass, R *rho, R *mu, R *mirror = nullptr)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)p.dx * p.dy) return;
    wall_column<R>(p, pass, c, rho, mu, mirror);
}


// ------------------------------------------------------------- stencils ----
// 4th-order 13-point Laplacian (GradD5, Common.h:189-192) and the 6th-order
// 19-point sum of GradD7 (Common.h:243-246) without its /180.
template <class R>
__device__ __forceinline__ R lap5_g(const KParams<R> &p, const R *x, int i, int j, int k)
{
    const int im2 = wrap_off(i - 2, p.dx), im1 = wrap_off(i - 1, p.dx), ip1 = wrap_off(i + 1, p.dx),
              ip2 = wrap_off(i + 2, p.dx);
    const int jm2 = wrap_off(j - 2, p.dy), jm1 = wrap_off(j - 1, p.dy), jp1 = wrap_off(j + 1, p.dy),
              jp2 = wrap_off(j + 2, p.dy);
    const int km2 = wrap_off(k - 2, p.dz), km1 = wrap_off(k - 1, p.dz), kp1 = wrap_off(k + 1, p.dz),
              kp2 = wrap_off(k + 2, p.dz);
#define XV(a, b, c) x[nid(p, a, b, c)]
    return (-XV(i, j, k) * R(90) +
            (-XV(im2, j, k) + XV(im1, j, k) * R(16) + XV(ip1, j, k) * R(16) - XV(ip2, j, k)) +
            (-XV(i, jm2, k) + XV(i, jm1, k) * R(16) + XV(i, jp1, k) * R(16) - XV(i, jp2, k)) +
            (-XV(i, j, km2) + XV(i, j, km1) * R(16) + XV(i, j, kp1) * R(16) - XV(i, j, kp2))) /
           R(12);
}

template <class R>
__device__ __forceinline__ R lap7sum_g(const KParams<R> &p, const R *x, int i, int j, int k)
{
    int a[7], b[7], c[7];
#pragma unroll
    for (int d = -3; d <= 3; ++d) {
        a[d + 3] = wrap_off(i + d, p.dx);
        b[d + 3] = wrap_off(j + d, p.dy);
        c[d + 3] = wrap_off(k + d, p.dz);
    }
    return (-XV(i, j, k) * R(490) * R(3) +
            (R(2) * XV(a[0], j, k) - R(27) * XV(a[1], j, k) + R(270) * XV(a[2], j, k) +
             R(270) * XV(a[4], j, k) - R(27) * XV(a[5], j, k) + R(2) * XV(a[6], j, k)) +
            (R(2) * XV(i, b[0], k) - R(27) * XV(i, b[1], k) + R(270) * XV(i, b[2], k) +
             R(270) * XV(i, b[4], k) - R(27) * XV(i, b[5], k) + R(2) * XV(i, b[6], k)) +
            (R(2) * XV(i, j, c[0]) - R(27) * XV(i, j, c[1]) + R(270) * XV(i, j, c[2]) +
             R(270) * XV(i, j, c[4]) - R(27) * XV(i, j, c[5]) + R(2) * XV(i, j, c[6])));
}

// D3Q19-weighted 6th-order gradient (Gradx7/y7/z7, Common.h:222-241): five
// lattice lines per component, each the first difference
// -x(-3) + 9x(-2) - 45x(-1) + 45x(+1) - 9x(+2) + x(+3), axis line doubled,
// sum / 360.
template <class R>
__device__ __forceinline__ void grad7_g(const KParams<R> &p, const R *x, int i, int j, int k, R g[3])
{
    int a[7], b[7], c[7];
#pragma unroll
    for (int d = -3; d <= 3; ++d) {
        a[d + 3] = wrap_off(i + d, p.dx);
        b[d + 3] = wrap_off(j + d, p.dy);
        c[d + 3] = wrap_off(k + d, p.dz);
    }
    // line along (sx, sy, sz) in {-1,0,1}^3: point d -> (a[3+sx d], b[3+sy d], c[3+sz d])
#define LN(sx, sy, sz)                                                                              \
    (-XV(a[3 - 3 * (sx)], b[3 - 3 * (sy)], c[3 - 3 * (sz)]) +                                      \
     XV(a[3 - 2 * (sx)], b[3 - 2 * (sy)], c[3 - 2 * (sz)]) * R(9) -                                \
     XV(a[3 - (sx)], b[3 - (sy)], c[3 - (sz)]) * R(45) + XV(a[3 + (sx)], b[3 + (sy)], c[3 + (sz)]) * R(45) - \
     XV(a[3 + 2 * (sx)], b[3 + 2 * (sy)], c[3 + 2 * (sz)]) * R(9) +                                \
     XV(a[3 + 3 * (sx)], b[3 + 3 * (sy)], c[3 + 3 * (sz)]))
    g[0] = (LN(1, 0, 0) * R(2) + LN(1, 0, 1) + LN(1, 0, -1) + LN(1, 1, 0) + LN(1, -1, 0)) / R(360);
    g[1] = (LN(0, 1, 0) * R(2) + LN(0, 1, 1) + LN(0, 1, -1) + LN(1, 1, 0) + LN(-1, 1, 0)) / R(360);
    g[2] = (LN(0, 0, 1) * R(2) + LN(1, 0, 1) + LN(-1, 0, 1) + LN(0, 1, 1) + LN(0, -1, 1)) / R(360);
#undef LN
#undef XV
}

// ChemPotential (FluidCuda.cu:444-463)
template <class R>
__global__ void k_chem_potential(KParams<R> p, const uint8_t *type, const R *rho, R *mu)
{
    NODE3D(p);
    if (type[I] != FLUID) return;
    const R m0 = mu0<R>(p.eos, p.A, p.B, p.T, rho[I]);
    if (p.lap_order == 7)
        mu[I] = p.kk * m0 - p.ka * lap7sum_g(p, rho, i, j, k) / R(180);
    else
        mu[I] = p.kk * m0 - p.ka * lap5_g(p, rho, i, j, k);
}

// NonidealForce (FluidCuda.cu:431-441): F = -rho grad(mu) + grad(rho)/3;
// grad(mu) is also stored when gm_out is non-null (the adjoint's replay).
template <class R>
__global__ void k_force(KParams<R> p, const uint8_t *type, const R *rho, const R *mu, R *F, R *gm_out)
{
    NODE3D(p);
    if (type[I] != FLUID) return;
    R gm[3], gr[3];
    grad7_g(p, mu, i, j, k, gm);
    grad7_g(p, rho, i, j, k, gr);
    const R r = rho[I];
    F[I] = -gm[0] * r + gr[0] / R(3);
    F[I + p.n] = -gm[1] * r + gr[1] / R(3);
    F[I + 2 * p.n] = -gm[2] * r + gr[2] / R(3);
    if (gm_out) {
        gm_out[I] = gm[0];
        gm_out[I + p.n] = gm[1];
        gm_out[I + 2 * p.n] = gm[2];
    }
}

// GlobalCollide (FluidCuda.cu:311-347): MV, MRT + exact-difference forcing,
// push streaming into the other lattice, half-way bounce-back onto the
// source node when the destination is solid.
template <class R, class S>
__global__ void __launch_bounds__(128) k_collide_plain(KParams<R> p, const uint8_t *type,
                                                       const R *rho, const R *u, const R *F,
                                                       const S *fc, S *fn, R *mv)
{
    NODE3D(p);
    if (type[I] != FLUID) return;
    const long long n = p.n;
    const R r = rho[I], ux = u[I], uy = u[I + n], uz = u[I + 2 * n];
    const R Fx = F[I], Fy = F[I + n], Fz = F[I + 2 * n];
    mv[I] = ux + Fx / r * R(0.5);
    mv[I + n] = uy + Fy / r * R(0.5);
    mv[I + 2 * n] = uz + Fz / r * R(0.5);
    R f[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = (R)fc[q * n + I];
    R qp[Q];
    const R *qpp = nullptr;
    if (p.qp) {
        R g[3];
        grad7_g(p, rho, i, j, k, g);
#pragma unroll
        for (int a = 0; a < Q; ++a) qp[a] = R(0);
        qp[1] = R(-19) * (p.k1 + R(3) * p.k2) * (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        qp[9] = -p.k1 * (R(2) * g[0] * g[0] - g[1] * g[1] - g[2] * g[2]);
        qp[11] = -p.k1 * (g[1] * g[1] - g[2] * g[2]);
        qp[13] = -p.k1 * g[0] * g[1];
        qp[14] = -p.k1 * g[2] * g[1];
        qp[15] = -p.k1 * g[0] * g[2];
        qpp = qp;
    }
    collide_mrt_edm<R>(f, r, ux, uy, uz, Fx, Fy, Fz, p.ts, qpp);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int ii = wrap_off(i + cx(q), p.dx), jj = wrap_off(j + cy(q), p.dy),
                  kk = wrap_off(k + cz(q), p.dz);
        const long long D = nid(p, ii, jj, kk);
        if (type[D] == FLUID)
            fn[q * n + D] = (S)f[q];
        else
            fn[opp(q) * n + I] = (S)f[q];
    }
}

// MacroCalculate (FluidCuda.cu:351-372)
template <class R, class S>
__global__ void k_macro(KParams<R> p, const uint8_t *type, const S *f, R *rho, R *u)
{
    NODE3D(p);
    if (type[I] != FLUID) return;
    const long long n = p.n;
    R v[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = (R)f[q * n + I];
    R r = R(0);
#pragma unroll
    for (int q = 0; q < Q; ++q) r += v[q];
    rho[I] = r;
    u[I] = (v[1] + v[7] + v[9] + v[11] + v[13] - v[2] - v[8] - v[10] - v[12] - v[14]) / r;
    u[I + n] = (v[3] + v[7] + v[8] + v[15] + v[17] - v[4] - v[9] - v[10] - v[16] - v[18]) / r;
    u[I + 2 * n] = (v[5] + v[11] + v[12] + v[15] + v[16] - v[6] - v[13] - v[14] - v[17] - v[18]) / r;
}

// ------------------------------------------------------------ launchers ----
template <class R, class S>
void plain_launch_init(const KParams<R> &p, const DropletDev &d, uint8_t *type, R *rho, R *mu, R *u,
                       S *f, cudaStream_t st)
{
    const unsigned g = (unsigned)((p.n + 255) / 256);
    k_init_plain<R, S><<<g, 256, 0, st>>>(p, d, type, rho, mu, u, f);
}

// One step with the density / velocity of step n read from (rho, u) and
// those of step n+1 written to (rho_out, u_out); the wall layers are
// extrapolated into rho in place and mu, F (and grad mu when gm_out is
// non-null) are left in their buffers.
template <class R, class S>
void plain_launch_step_split(const KParams<R> &p, const uint8_t *type, R *rho, R *mu, const R *u, R *F, R *mv,
                             const S *fc, S *fn, R *rho_out, R *u_out, R *gm_out, cudaStream_t st,
                             LaunchHook *hook)
{
    const dim3 g = grid3(p, 128);
    if (p.wall_mode == 1) {
        const long long np = (long long)p.dx * p.dy;
        const unsigned gw = (unsigned)((np + 127) / 128);
        for (int s = 0; s < (p.complex_bc ? 3 : 1); ++s) {
            hook_begin(hook, K_WALL, st);
            k_wall_pass<R><<<gw, 128, 0, st>>>(p, s, rho, mu);
            hook_end(hook, K_WALL, st);
        }
    }
    hook_begin(hook, K_MU, st);
    k_chem_potential<R><<<g, 128, 0, st>>>(p, type, rho, mu);
    hook_end(hook, K_MU, st);
    hook_begin(hook, K_FORCE, st);
    k_force<R><<<g, 128, 0, st>>>(p, type, rho, mu, F, gm_out);
    hook_end(hook, K_FORCE, st);
    hook_begin(hook, K_COLLIDE, st);
    k_collide_plain<R, S><<<g, 128, 0, st>>>(p, type, rho, u, F, fc, fn, mv);
    hook_end(hook, K_COLLIDE, st);
    hook_begin(hook, K_MACRO, st);
    k_macro<R, S><<<g, 128, 0, st>>>(p, type, fn, rho_out, u_out);
    hook_end(hook, K_MACRO, st);
}

// One step of the reference's loop body (FluidCuda.cu:1277-1291), in place.
template <class R, class S>
void plain_launch_step(const KParams<R> &p, const uint8_t *type, R *rho, R *mu, R *u, R *F, R *mv,
                       const S *fc, S *fn, cudaStream_t st, LaunchHook *hook)
{
    plain_launch_step_split<R, S>(p, type, rho, mu, u, F, mv, fc, fn, rho, u, nullptr, st, hook);
}

template <class R, class S>
void plain_launch_macro(const KParams<R> &p, const uint8_t *type, const S *f, R *rho, R *u,
                        cudaStream_t st)
{
    const dim3 g = grid3(p, 128);
    k_macro<R, S><<<g, 128, 0, st>>>(p, type, f, rho, u);
}

// Wall layers of rho only (adjoint recompute).
template <class R>
void plain_launch_wall(const KParams<R> &p, R *rho, cudaStream_t st)
{
    if (p.wall_mode != 1) return;
    const long long np = (long long)p.dx * p.dy;
    const unsigned gw = (unsigned)((np + 127) / 128);
    for (int s = 0; s < (p.complex_bc ? 3 : 1); ++s) k_wall_pass<R><<<gw, 128, 0, st>>>(p, s, rho, nullptr);
}

// mu and F without collision (diagnostic read-back of MU / FORCE); grad(mu)
// into gm_out when it is non-null.
template <class R>
void plain_launch_mu_force(const KParams<R> &p, const uint8_t *type, R *rho, R *mu, R *F,
                           cudaStream_t st, R *gm_out)
{
    const dim3 g = grid3(p, 128);
    if (p.wall_mode == 1) {
        const long long np = (long long)p.dx * p.dy;
        const unsigned gw = (unsigned)((np + 127) / 128);
        for (int s = 0; s < (p.complex_bc ? 3 : 1); ++s) k_wall_pass<R><<<gw, 128, 0, st>>>(p, s, rho, mu);
    }
    k_chem_potential<R><<<g, 128, 0, st>>>(p, type, rho, mu);
    k_force<R><<<g, 128, 0, st>>>(p, type, rho, mu, F, gm_out);
}

}  // namespace cpmp
