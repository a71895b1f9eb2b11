// k_fused2.cuh -- the FUSED collide with two z-adjacent nodes per thread.
//
// Same storage, A-A addressing, shared-memory rings and arithmetic as
// fused_tile (k_fused.cuh); a thread owns the node pair (z, z + 1) of its
// (y, z) column tile, z even.  The collision, decode, encode and velocity
// run as paired FP32 instructions (FFMA2 / FADD2 / FMUL2) through the _x2
// moment transforms, which perform the single-node operations in the same
// order, so a pair gives exactly the bits of two single-node evaluations.
// With an even DZ every node pair starts on an even node index: the
// populations of the pair are one 32-bit (FP16 / BF16) or 64-bit (FP32)
// access wherever the source or destination offset keeps that parity, two
// scalar accesses where it does not (odd z offsets of the A-A odd step, and
// every access of a box with an odd DZ).  Pairs in a wall tile of an interior
// column select their solid-source slots without wrapping; pairs at a
// periodic edge take a per-node general path for their global accesses.
#pragma once

#include "k_fused.cuh"

namespace cpmp {

template <class S>
struct SPair;
template <>
struct SPair<__half> {
    using T = __half2;
    static __device__ __forceinline__ float2 tof(T v) { return __half22float2(v); }
    static __device__ __forceinline__ T fromf(float2 v) { return __float22half2_rn(v); }
    static __device__ __forceinline__ T make(__half a, __half b) { return __halves2half2(a, b); }
    static __device__ __forceinline__ __half lo(T v) { return __low2half(v); }
    static __device__ __forceinline__ __half hi(T v) { return __high2half(v); }
    static __device__ __forceinline__ __half zero() { return __float2half_rn(0.f); }
};
template <>
struct SPair<__nv_bfloat16> {
    using T = __nv_bfloat162;
    static __device__ __forceinline__ float2 tof(T v) { return __bfloat1622float2(v); }
    static __device__ __forceinline__ T fromf(float2 v) { return __float22bfloat162_rn(v); }
    static __device__ __forceinline__ T make(__nv_bfloat16 a, __nv_bfloat16 b) { return __halves2bfloat162(a, b); }
    static __device__ __forceinline__ __nv_bfloat16 lo(T v) { return __low2bfloat16(v); }
    static __device__ __forceinline__ __nv_bfloat16 hi(T v) { return __high2bfloat16(v); }
    static __device__ __forceinline__ __nv_bfloat16 zero() { return __float2bfloat16_rn(0.f); }
};
template <>
struct SPair<float> {
    using T = float2;
    static __device__ __forceinline__ float2 tof(T v) { return v; }
    static __device__ __forceinline__ T fromf(float2 v) { return v; }
    static __device__ __forceinline__ T make(float a, float b) { return make_float2(a, b); }
    static __device__ __forceinline__ float lo(T v) { return v.x; }
    static __device__ __forceinline__ float hi(T v) { return v.y; }
    static __device__ __forceinline__ float zero() { return 0.f; }
};

// The rings of a TY x TZ node tile (TZ even, TY * TZ / 2 threads): those of
// the one-node kernel, except that the rest-population ring has a z halo of 2
// so that every node pair sits on an even (8-byte aligned) index.
template <int TY, int TZ, int L>
using Rings2 = FusedRings<TY, TZ, L, TY * TZ / 2, 2>;

// One CTA owns a TY x TZ column tile and marches over xl planes of x with the
// rings of FusedRings, in the order of work per plane of fused_tile.
template <class S, int TY, int TZ, int L, class SL>
__device__ __forceinline__ void fused_tile2(const KParams<float> &p, int P, const SL &slots,
                                            const float *__restrict__ f0c, float *__restrict__ f0n,
                                            const float *__restrict__ rho, const int z0, const int y0,
                                            const int x0, const int xl, float4 *smem4)
{
    static_assert(TZ % 2 == 0, "node pairs need an even tile height");
    using RG = Rings2<TY, TZ, L>;
    using SP = SPair<S>;
    using T = typename SP::T;
    using namespace p2;
    constexpr int MZ = RG::MZ, AZ = RG::AZ, TH = TZ / 2;
    const int tz = 2 * (threadIdx.x % TH), ty = threadIdx.x / TH;
    const int x1 = min(x0 + xl, p.dx);
    const unsigned plane = (unsigned)(p.dy * p.dz);
    auto slot = [&](int q, unsigned idx) -> S * { return slots(q, idx); };
    const bool yz_fast = z_interior(p, z0, TZ) && y0 >= 1 && y0 + TY <= p.dy - 1;
    RG R(p, rho, f0c, smem4);
    R.setup(y0, z0);

    const int gy = y0 + ty, gz = z0 + tz;
    const bool inA = gy < p.dy && gz < p.dz && !solid_k(p.wall_mode, gz, p.dz);
    const bool inB = gy < p.dy && gz + 1 < p.dz && !solid_k(p.wall_mode, gz + 1, p.dz);
    const bool any = inA || inB, both = inA && inB;
    const bool ev = (p.dz & 1) == 0;  // every pair starts on an even node index

    // one population of node (gx, gy, gzl) through the general A-A read
    auto load_general = [&](int q, int gx, int gzl, unsigned Il) -> S {
        const int si = wrap1(gx - cx(q), p.dx), sj = wrap1(gy - cy(q), p.dy), sk = wrap1(gzl - cz(q), p.dz);
        if (solid_k(p.wall_mode, sk, p.dz)) return *slot(q - 1, Il);
        return *slot(opp(q) - 1, (unsigned)si * plane + (unsigned)(sj * p.dz + sk));
    };
    auto store_general = [&](int q, int gx, int gzl, unsigned Il, S v) {
        const int di = wrap1(gx + cx(q), p.dx), dj = wrap1(gy + cy(q), p.dy), dk = wrap1(gzl + cz(q), p.dz);
        if (solid_k(p.wall_mode, dk, p.dz))
            *slot(opp(q) - 1, Il) = v;
        else
            *slot(q - 1, (unsigned)di * plane + (unsigned)(dj * p.dz + dk)) = v;
    };

    // moving populations of the pair in plane x into registers
    auto fetch = [&](int x, T hv[Q - 1]) {
        if (!any) return;
        const int gx = wrap_small(x, p.dx);
        const unsigned I = (unsigned)gx * plane + (unsigned)(gy * p.dz + gz);
        if (P == 0) {
            if (ev && both) {
#pragma unroll
                for (int q = 1; q < Q; ++q) hv[q - 1] = *reinterpret_cast<const T *>(slot(q - 1, I));
            } else {
#pragma unroll
                for (int q = 1; q < Q; ++q)
                    hv[q - 1] = SP::make(inA ? *slot(q - 1, I) : SP::zero(), inB ? *slot(q - 1, I + 1) : SP::zero());
            }
        } else if (yz_fast && gx >= 1 && gx + 1 < p.dx) {
            if (ev) {
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const S *ptr = slot(opp(q) - 1, I - (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q)));
                    hv[q - 1] = (cz(q) & 1) ? SP::make(ptr[0], ptr[1]) : *reinterpret_cast<const T *>(ptr);
                }
            } else {
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const S *ptr = slot(opp(q) - 1, I - (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q)));
                    hv[q - 1] = SP::make(ptr[0], ptr[1]);
                }
            }
        } else if (p.wall_mode == 1 && gy >= 1 && gy + 1 < p.dy && gx >= 1 && gx + 1 < p.dx) {
            // no wrap: only the sources across a wall layer (z = 3 or dz - 4) are solid
            const bool loA = gz == 3, hiA = gz == p.dz - 4, loB = gz + 1 == 3, hiB = gz + 1 == p.dz - 4;
#pragma unroll
            for (int q = 1; q < Q; ++q) {
                const unsigned src = I - (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q));
                const bool sA = (cz(q) == 1 && loA) || (cz(q) == -1 && hiA);
                const bool sB = (cz(q) == 1 && loB) || (cz(q) == -1 && hiB);
                hv[q - 1] = SP::make(inA ? *(sA ? slot(q - 1, I) : slot(opp(q) - 1, src)) : SP::zero(),
                                     inB ? *(sB ? slot(q - 1, I + 1) : slot(opp(q) - 1, src + 1)) : SP::zero());
            }
        } else {
#pragma unroll
            for (int q = 1; q < Q; ++q)
                hv[q - 1] = SP::make(inA ? load_general(q, gx, gz, I) : SP::zero(),
                                     inB ? load_general(q, gx, gz + 1, I + 1) : SP::zero());
        }
    };

    // force on one node from the (rho, mu) ring, centre index c
    auto force = [&](const float2 *const pl[7], int c, float &r, float gr[3], float F[3]) {
        float2 g0 = make_float2(0.f, 0.f), g1 = g0, g2 = g0;
        auto line = [&](int sx, int sy, int sz) -> float2 {
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int d = 1; d <= 3; ++d) {
                const float k = d == 1 ? 45.f : (d == 2 ? -9.f : 1.f);
                const int mo = sy * d * MZ + sz * d;
                const float2 a = pl[3 + sx * d][c + mo], b = pl[3 - sx * d][c - mo];
                acc = __ffma2_rn(make_float2(k, k), __fadd2_rn(a, make_float2(-b.x, -b.y)), acc);
            }
            return acc;
        };
        const float2 two = make_float2(2.f, 2.f);
        float2 l;
        l = line(1, 0, 0); g0 = __ffma2_rn(two, l, g0);
        l = line(0, 1, 0); g1 = __ffma2_rn(two, l, g1);
        l = line(0, 0, 1); g2 = __ffma2_rn(two, l, g2);
        l = line(1, 1, 0); g0 = __fadd2_rn(g0, l); g1 = __fadd2_rn(g1, l);
        l = line(1, -1, 0); g0 = __fadd2_rn(g0, l); g1 = __fadd2_rn(g1, make_float2(-l.x, -l.y));
        l = line(1, 0, 1); g0 = __fadd2_rn(g0, l); g2 = __fadd2_rn(g2, l);
        l = line(1, 0, -1); g0 = __fadd2_rn(g0, l); g2 = __fadd2_rn(g2, make_float2(-l.x, -l.y));
        l = line(0, 1, 1); g1 = __fadd2_rn(g1, l); g2 = __fadd2_rn(g2, l);
        l = line(0, 1, -1); g1 = __fadd2_rn(g1, l); g2 = __fadd2_rn(g2, make_float2(-l.x, -l.y));
        const float inv360 = 1.0f / 360.0f;
        const float gm[3] = {g0.y * inv360, g1.y * inv360, g2.y * inv360};
        gr[0] = g0.x * inv360;
        gr[1] = g1.x * inv360;
        gr[2] = g2.x * inv360;
        r = pl[3][c].x;
#pragma unroll
        for (int a = 0; a < 3; ++a) F[a] = fmaf(-gm[a], r, gr[a] * (1.0f / 3.0f));
    };

    T hv[Q - 1];
    R.prologue(x0);
    fetch(x0, hv);

    const int mc = (ty + 3) * MZ + (tz + 3);
    const int ac = (ty + 1) * AZ + (tz + 2);  // even
    float mv2 = 0.f;  // max |MV|^2 of this thread's fluid nodes
    for (int x = x0; x < x1; ++x) {
        R.begin_plane(x, x + 1 < x1);
        T hn[Q - 1];
        if (x + 1 < x1) fetch(x + 1, hn);
        R.comp_mu(x + 3);
        __syncthreads();
        if (any) {
            const float2 *pl[7];
#pragma unroll
            for (int d = -3; d <= 3; ++d) pl[d + 3] = R.rm_plane(x + d);
            float rA, rB, grA[3], grB[3], FA[3], FB[3];
            force(pl, mc, rA, grA, FA);
            force(pl, mc + 1, rB, grB, FB);
            const float2 r = make_float2(rA, rB);

            const float *fa[3] = {R.f0_plane(x - 1), R.f0_plane(x), R.f0_plane(x + 1)};
            const float2 a0 = *reinterpret_cast<const float2 *>(fa[1] + ac);
            float2 f[Q];
            f[0] = a0;
#pragma unroll
            for (int q = 1; q < Q; ++q) {
                const float *src = fa[1 - cx(q)] + ac - cy(q) * AZ - cz(q);
                float2 a;
                if (yz_fast || p.wall_mode != 1) {
                    a = (cz(q) & 1) ? make_float2(src[0], src[1]) : *reinterpret_cast<const float2 *>(src);
                } else {
                    const int skA = gz - cz(q), skB = gz + 1 - cz(q);
                    a.x = (skA < 3 || skA > p.dz - 4) ? a0.x : src[0];
                    a.y = (skB < 3 || skB > p.dz - 4) ? a0.y : src[1];
                }
                f[q] = fma(K(wgt<float>(q)), SP::tof(hv[q - 1]), mul(K(ratio0(q)), a));
            }
            const float2 ir = make_float2(1.0f / r.x, 1.0f / r.y);
            const float2 ux = mul(sub(sub(sub(sub(sub(add(add(add(add(f[1], f[7]), f[9]), f[11]), f[13]), f[2]), f[8]),
                                              f[10]), f[12]), f[14]), ir);
            const float2 uy = mul(sub(sub(sub(sub(sub(add(add(add(add(f[3], f[7]), f[8]), f[15]), f[17]), f[4]), f[9]),
                                              f[10]), f[16]), f[18]), ir);
            const float2 uz = mul(sub(sub(sub(sub(sub(add(add(add(add(f[5], f[11]), f[12]), f[15]), f[16]), f[6]),
                                                  f[13]), f[14]), f[17]), f[18]), ir);
            const float2 Fx = make_float2(FA[0], FB[0]), Fy = make_float2(FA[1], FB[1]), Fz = make_float2(FA[2], FB[2]);
            {   // MV = u + F / (2 rho) on the pair's fluid nodes
                const float2 hr = mul(K(0.5f), ir);
                const float2 vx = fma(Fx, hr, ux), vy = fma(Fy, hr, uy), vz = fma(Fz, hr, uz);
                const float2 v2 = fma(vx, vx, fma(vy, vy, mul(vz, vz)));
                if (inA) mv2 = fmaxf(mv2, v2.x);
                if (inB) mv2 = fmaxf(mv2, v2.y);
            }
            if (p.qp) {
                float qa[Q], qb[Q];
#pragma unroll
                for (int a = 0; a < Q; ++a) qa[a] = qb[a] = 0.f;
                auto fill = [&](const float gr[3], float qp[Q]) {
                    qp[1] = -19.f * (p.k1 + 3.f * p.k2) * (gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
                    qp[9] = -p.k1 * (2.f * gr[0] * gr[0] - gr[1] * gr[1] - gr[2] * gr[2]);
                    qp[11] = -p.k1 * (gr[1] * gr[1] - gr[2] * gr[2]);
                    qp[13] = -p.k1 * gr[0] * gr[1];
                    qp[14] = -p.k1 * gr[2] * gr[1];
                    qp[15] = -p.k1 * gr[0] * gr[2];
                };
                fill(grA, qa);
                fill(grB, qb);
                float2 qp2[Q];
#pragma unroll
                for (int a = 0; a < Q; ++a) qp2[a] = make_float2(qa[a], qb[a]);
                collide_mrt_edm_fused2(f, r, ir, ux, uy, uz, Fx, Fy, Fz, p.ts, p.omts, qp2);
            } else {
                collide_mrt_edm_fused2(f, r, ir, ux, uy, uz, Fx, Fy, Fz, p.ts, p.omts, nullptr);
            }

            // encode against the pair's new rest populations and stream
            const int gx = wrap_small(x, p.dx);
            const unsigned I = (unsigned)gx * plane + (unsigned)(gy * p.dz + gz);
            const float2 an = f[0];
            if (ev && both) {
                *reinterpret_cast<float2 *>(f0n + I) = an;
            } else {
                if (inA) f0n[I] = an.x;
                if (inB) f0n[I + 1] = an.y;
            }
            if (P == 0 && ev && both) {
#pragma unroll
                for (int q = 1; q < Q; ++q)
                    *reinterpret_cast<T *>(slot(opp(q) - 1, I)) =
                        SP::fromf(mul(fma(K(-ratio0(q)), an, f[q]), K(inv_w(q))));
            } else if (P == 0) {
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const T v = SP::fromf(mul(fma(K(-ratio0(q)), an, f[q]), K(inv_w(q))));
                    if (inA) *slot(opp(q) - 1, I) = SP::lo(v);
                    if (inB) *slot(opp(q) - 1, I + 1) = SP::hi(v);
                }
            } else if (yz_fast && gx >= 1 && gx + 1 < p.dx) {
                if (ev) {
#pragma unroll
                    for (int q = 1; q < Q; ++q) {
                        const T v = SP::fromf(mul(fma(K(-ratio0(q)), an, f[q]), K(inv_w(q))));
                        S *ptr = slot(q - 1, I + (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q)));
                        if (cz(q) & 1) {
                            ptr[0] = SP::lo(v);
                            ptr[1] = SP::hi(v);
                        } else {
                            *reinterpret_cast<T *>(ptr) = v;
                        }
                    }
                } else {
#pragma unroll
                    for (int q = 1; q < Q; ++q) {
                        const T v = SP::fromf(mul(fma(K(-ratio0(q)), an, f[q]), K(inv_w(q))));
                        S *ptr = slot(q - 1, I + (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q)));
                        ptr[0] = SP::lo(v);
                        ptr[1] = SP::hi(v);
                    }
                }
            } else if (p.wall_mode == 1 && gy >= 1 && gy + 1 < p.dy && gx >= 1 && gx + 1 < p.dx) {
                const bool loA = gz == 3, hiA = gz == p.dz - 4, loB = gz + 1 == 3, hiB = gz + 1 == p.dz - 4;
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const T v = SP::fromf(mul(fma(K(-ratio0(q)), an, f[q]), K(inv_w(q))));
                    const unsigned dst = I + (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q));
                    const bool sA = (cz(q) == -1 && loA) || (cz(q) == 1 && hiA);
                    const bool sB = (cz(q) == -1 && loB) || (cz(q) == 1 && hiB);
                    if (inA) *(sA ? slot(opp(q) - 1, I) : slot(q - 1, dst)) = SP::lo(v);
                    if (inB) *(sB ? slot(opp(q) - 1, I + 1) : slot(q - 1, dst + 1)) = SP::hi(v);
                }
            } else {
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const T v = SP::fromf(mul(fma(K(-ratio0(q)), an, f[q]), K(inv_w(q))));
                    if (inA) store_general(q, gx, gz, I, SP::lo(v));
                    if (inB) store_general(q, gx, gz + 1, I + 1, SP::hi(v));
                }
            }
        }
#pragma unroll
        for (int q = 0; q < Q - 1; ++q) hv[q] = hn[q];
    }
    cp_async_wait_all();
    mvmax_flush(p, P, mv2);
}

// Registers: at most 128 per thread for 4-byte storage pairs and the
// half-precision ones alike (two CTAs of 256 threads per SM).
template <int NT>
constexpr int fused2_min_blocks()
{
    return NT >= 512 ? 1 : 512 / NT;
}

template <class S, int TY, int TZ, int L>
__global__ void __launch_bounds__(TY *TZ / 2, fused2_min_blocks<TY * TZ / 2>())
    k_fused2_collide(KParams<float> p, int P, SlotTable<S> slots, const float *__restrict__ f0c,
                     float *__restrict__ f0n, const float *__restrict__ rho, int xl)
{
    extern __shared__ float4 smem4[];
    fused_tile2<S, TY, TZ, L>(p, P, slots, f0c, f0n, rho, blockIdx.x * TZ, blockIdx.y * TY, blockIdx.z * xl, xl,
                              smem4);
}

// Persistent batch form (see k_fused_collide_batch).
template <class S, int TY, int TZ, int L>
__global__ void __launch_bounds__(TY *TZ / 2, fused2_min_blocks<TY * TZ / 2>())
    k_fused2_collide_batch(const KParams<float> *__restrict__ params, const BatchBox *__restrict__ boxes,
                           int nbox, long long total_items, int P, int xl, unsigned int *counter)
{
    extern __shared__ float4 smem4[];
    __shared__ long long item_s;
    __shared__ int box_s;
    __shared__ S *slot_s[Q - 1];
    for (;;) {
        if (threadIdx.x == 0) {
            const long long it = (long long)atomicAdd(counter, 1u);
            int lo = 0, hi = nbox - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) / 2;
                if (boxes[mid].item0 <= it) lo = mid;
                else hi = mid - 1;
            }
            item_s = it;
            box_s = lo;
        }
        __syncthreads();
        const long long it = item_s;
        if (it >= total_items) break;
        const BatchBox &bx = boxes[box_s];
        const KParams<float> &p = params[box_s];
        const long long local = it - bx.item0;
        const int per_chunk = bx.tiles_z * bx.tiles_y;
        const int chunk = (int)(local / per_chunk), rem = (int)(local % per_chunk);
        const int ytile = rem / bx.tiles_z, ztile = rem % bx.tiles_z;
        if (threadIdx.x < Q - 1) slot_s[threadIdx.x] = (S *)bx.h + (size_t)p.n * threadIdx.x;
        fused_tile2<S, TY, TZ, L>(p, P, SlotShared<S>{slot_s}, bx.f0[P], bx.f0[1 - P], bx.rho[P], ztile * TZ,
                                  ytile * TY, chunk * xl, xl, smem4);
        __syncthreads();
    }
}

}  // namespace cpmp
