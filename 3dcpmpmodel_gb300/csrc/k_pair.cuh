// k_pair.cuh -- the FUSED collide with two z-adjacent nodes per thread and
// shared-memory rings filled by bulk copies.
//
// Storage, A-A addressing and arithmetic are those of fused_tile
// (k_fused.cuh); the collision, decode, encode and the chemical potential run
// as paired FP32 instructions (lane_math.cuh, Lane2), which give exactly the
// bits of the one-node kernel.  Requirements: DZ a multiple of 4, so that a
// thread's node pair (z, z + 1), z even, is one aligned 2-element access
// wherever the A-A offset keeps the parity, and every ring row of an x plane
// starts on a 16-byte boundary in global memory.
//
// A CTA owns a TY x TZ column tile of (y, z) (TY * TZ / 2 threads; a warp is
// one or two rows of pairs along z) and marches over x.  Per output plane x:
//   rho ring  (planes x+3-L .. x+4+L, rows y0-3-L .. y0+TY+2+L, z0-8 .. z0+TZ+7)
//   f0 ring   (planes x-1 .. x+2, rows y0-1 .. y0+TY, z0-4 .. z0+TZ+3)
// are filled one x plane at a time by cp.async.bulk row copies (one lane per
// row, a row split where it wraps around a periodic z edge) that complete on
// one mbarrier per ring slot; the (rho, mu) ring (planes x-3 .. x+4, rows
// y0-3 .. y0+TY+2, z0-4 .. z0+TZ+3) is computed in the CTA from the rho ring,
// two z-adjacent elements per thread.  The force of a node pair reads both
// nodes' (rho, mu) neighbours with one 16-byte shared load where the stencil
// offset along z is even.  Every wait on a copy is bounded in time: a CTA that
// gives up sets the error word and returns after a bounded wait for its other
// copies.
#pragma once

#include "k_fused.cuh"

namespace cpmp {

// ------------------------------------------------------ bulk copies ----
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase with the given parity to complete, for at most ~2 s.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    if (mbar_test(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_test(bar, parity))
        if (global_ns() - t0 > 2000000000ull) return false;
    return true;
}
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// orders this thread's (and, after a barrier, the CTA's) earlier shared-memory
// reads before the async-proxy writes of the copies it issues next
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// A node pair's two stored values as one 32-bit (FP16 / BF16) or 64-bit (FP32)
// register, and its conversion to and from a pair of floats.
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
};
template <>
struct SPair<__nv_bfloat16> {
    using T = __nv_bfloat162;
    static __device__ __forceinline__ float2 tof(T v) { return __bfloat1622float2(v); }
    static __device__ __forceinline__ T fromf(float2 v) { return __float22bfloat162_rn(v); }
    static __device__ __forceinline__ T make(__nv_bfloat16 a, __nv_bfloat16 b) { return __halves2bfloat162(a, b); }
    static __device__ __forceinline__ __nv_bfloat16 lo(T v) { return __low2bfloat16(v); }
    static __device__ __forceinline__ __nv_bfloat16 hi(T v) { return __high2bfloat16(v); }
};
template <>
struct SPair<float> {
    using T = float2;
    static __device__ __forceinline__ float2 tof(T v) { return v; }
    static __device__ __forceinline__ T fromf(float2 v) { return v; }
    static __device__ __forceinline__ T make(float a, float b) { return make_float2(a, b); }
    static __device__ __forceinline__ float lo(T v) { return v.x; }
    static __device__ __forceinline__ float hi(T v) { return v.y; }
};

template <int TY, int TZ, int L>
struct PairRings {
    static constexpr int NT = TY * TZ / 2, TH = TZ / 2;
    static constexpr int RH = 3 + L;
    static constexpr int RY = TY + 2 * RH, RZ = TZ + 16;  // rho ring rows, columns z0-8 ..
    static constexpr int NR = 2 * L + 2;                  // rho planes
    static constexpr int MY = TY + 6, MZ = TZ + 8, HM = MZ / 2;  // (rho, mu) ring, columns z0-4 ..
    static constexpr int NM = 8;
    static constexpr int AY = TY + 2, AZ = TZ + 8;  // f0 ring, columns z0-4 ..
    static constexpr int NF = 5;
    static constexpr int NPM = MY * HM;                  // (rho, mu) pairs per plane
    static constexpr int KM = (NPM + NT - 1) / NT;       // pairs per thread per plane
    static constexpr size_t RHO_BYTES = sizeof(float) * NR * RY * RZ;
    static constexpr size_t RM_BYTES = sizeof(float2) * NM * MY * MZ;
    static constexpr size_t F0_BYTES = sizeof(float) * NF * AY * AZ;
    static constexpr size_t BAR_BYTES = sizeof(unsigned long long) * (NR + NF);
    static constexpr size_t BYTES = RHO_BYTES + RM_BYTES + F0_BYTES + BAR_BYTES;
    static_assert(RY <= 32 && AY <= 32, "one lane per ring row");
    static_assert(TZ % 32 == 0, "tile height");
    static_assert(RHO_BYTES % 16 == 0 && RM_BYTES % 16 == 0 && F0_BYTES % 16 == 0, "16-byte ring slots");
};

// Row copies of one x plane of `field` into a ring slot (lane r copies row r):
// rows y_first + r (wrapped in y), columns [z_first, z_first + width) wrapped
// in z (periodic box) or clipped to [0, dz) (walled box; the clipped columns
// lie beyond the walls and are never read for a fluid node).
__device__ __forceinline__ void issue_plane(const KParams<float> &p, const float *field, int xlog, float *slot,
                                            int nrows, int y_first, int z_first, int width,
                                            unsigned long long *bar, int lane)
{
    const int gx = wrap_small(xlog, p.dx);
    const float *base = field + (size_t)((unsigned)gx * (unsigned)(p.dy * p.dz));
    unsigned bytes = 0;
    const bool mine = lane < nrows;
    int lo = z_first, hi = z_first + width;
    if (p.wall_mode == 1) {
        lo = max(lo, 0);
        hi = min(hi, p.dz);
    }
    if (mine && hi > lo) bytes = (unsigned)(hi - lo) * 4u;
    bytes = __reduce_add_sync(0xffffffffu, bytes);
    if (lane == 0) mbar_expect_tx(bar, bytes);
    __syncwarp();
    if (!mine || hi <= lo) return;
    const int y = wrap_small(y_first + lane, p.dy);
    const float *row = base + (size_t)y * p.dz;
    float *drow = slot + lane * width;
    fence_proxy_async();
    if (p.wall_mode == 1) {
        bulk_copy(drow + (lo - z_first), row + lo, (unsigned)(hi - lo) * 4u, bar);
        return;
    }
    int zz = z_first, done = 0;
    while (done < width) {
        const int zw = wrap_small(zz, p.dz);
        const int len = min(width - done, p.dz - zw);
        bulk_copy(drow + done, row + zw, (unsigned)len * 4u, bar);
        done += len;
        zz += len;
    }
}

template <class S, int TY, int TZ, int L, bool REF, class SL>
__device__ __forceinline__ void pair_tile(const KParams<float> &p, int P, const SL &slots,
                                          const float *__restrict__ f0c, float *__restrict__ f0n,
                                          const float *__restrict__ rho, const int z0, const int y0, const int x0,
                                          const int xl, float4 *smem4)
{
    using RG = PairRings<TY, TZ, L>;
    using SP = SPair<S>;
    using T = typename SP::T;
    using O = Lane2;
    constexpr int RY = RG::RY, RZ = RG::RZ, NR = RG::NR, MY = RG::MY, MZ = RG::MZ, HM = RG::HM;
    constexpr int AY = RG::AY, AZ = RG::AZ, NF = RG::NF, NT = RG::NT, TH = RG::TH;

    float *srho = reinterpret_cast<float *>(smem4);
    float2 *srm = reinterpret_cast<float2 *>(reinterpret_cast<char *>(smem4) + RG::RHO_BYTES);
    float *sf0 = reinterpret_cast<float *>(reinterpret_cast<char *>(smem4) + RG::RHO_BYTES + RG::RM_BYTES);
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(smem4) +
                                                                      RG::RHO_BYTES + RG::RM_BYTES + RG::F0_BYTES);
    unsigned long long *rbar = bars, *fbar = bars + NR;
    __shared__ int s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x1 = min(x0 + xl, p.dx);
    const unsigned plane = (unsigned)(p.dy * p.dz);
    const EosLane eos = make_eos_lane(p.eos, p.A, p.B, p.T);

    if (tid == 0) {
        for (int i = 0; i < NR + NF; ++i) mbar_init(bars + i, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    __syncthreads();

    // ring bookkeeping: rho planes are issued in order from x0-3-L, f0 planes from x0-1
    const int rp0 = x0 - 3 - L, fp0 = x0 - 1;
    auto rslot = [&](int pl) { return (pl - rp0) % NR; };
    auto rpar = [&](int pl) { return (unsigned)(((pl - rp0) / NR) & 1); };
    auto fslot = [&](int pl) { return (pl - fp0) % NF; };
    auto fpar = [&](int pl) { return (unsigned)(((pl - fp0) / NF) & 1); };
    auto rho_plane = [&](int pl) -> const float * { return srho + rslot(pl) * (RY * RZ); };
    auto f0_plane = [&](int pl) -> const float * { return sf0 + fslot(pl) * (AY * AZ); };
    auto rm_plane = [&](int pl) -> float2 * { return srm + (pl & 7) * (MY * MZ); };
    // warp 0 issues rho planes, the last warp f0 planes; planes issued so far
    // and planes whose copies this thread saw complete
    const int fwarp = NT / 32 - 1;
    int r_iss = rp0 - 1, f_iss = fp0 - 1, r_got = rp0 - 1, f_got = fp0 - 1;
    auto issue_rho = [&](int pl) {
        r_iss = pl;
        if (warp == 0)
            issue_plane(p, rho, pl, srho + rslot(pl) * (RY * RZ), RY, y0 - 3 - L, z0 - 8, RZ, rbar + rslot(pl), lane);
    };
    auto issue_f0 = [&](int pl) {
        f_iss = pl;
        if (warp == fwarp)
            issue_plane(p, f0c, pl, sf0 + fslot(pl) * (AY * AZ), AY, y0 - 1, z0 - 4, AZ, fbar + fslot(pl), lane);
    };
    bool ok = true;
    auto wait_rho = [&](int pl) {
        for (int q = r_got + 1; ok && q <= pl; ++q) {
            ok = mbar_wait(rbar + rslot(q), rpar(q));
            if (ok) r_got = q;
        }
    };
    auto wait_f0 = [&](int pl) {
        for (int q = f_got + 1; ok && q <= pl; ++q) {
            ok = mbar_wait(fbar + fslot(q), fpar(q));
            if (ok) f_got = q;
        }
    };

    // ---- the (rho, mu) elements this thread evaluates in every plane
    const bool walled = p.wall_mode == 1;
    const bool wall_tile = walled && (z0 - 4 < 3 || z0 + TZ + 4 > p.dz - 3);
    int roff[RG::KM], moff[RG::KM], wcol[RG::KM], wflag[RG::KM];
#pragma unroll
    for (int k = 0; k < RG::KM; ++k) {
        const int e = tid + k * NT;
        const int r = e / HM, c = e - (e / HM) * HM;
        roff[k] = (r + L) * RZ + 4 + 2 * c;
        moff[k] = r * MZ + 2 * c;
        const int z = z0 - 4 + 2 * c;
        // bit 0 / 1: element z / z + 1 is solid; bit 2: the top wall
        const int sa = walled && (z < 3 || z > p.dz - 4), sb = walled && (z + 1 < 3 || z + 1 > p.dz - 4);
        wflag[k] = (e < RG::NPM) ? (sa | (sb << 1) | ((z > p.dz / 2) << 2)) : 0;
        wcol[k] = wrap_small(y0 - 3 + r, p.dy);
    }
    auto comp_mu = [&](int pl) {
        const int gx = wrap_small(pl, p.dx);
        float2 *dst = rm_plane(pl);
        // planes pl-L .. pl+L: one slot computation, then consecutive slots
        const float *rpl[2 * L + 1];
        {
            int sl = rslot(pl - L);
#pragma unroll
            for (int k = 0; k <= 2 * L; ++k) {
                rpl[k] = srho + sl * (RY * RZ);
                sl = sl + 1 == NR ? 0 : sl + 1;
            }
        }
        const float *rc = rpl[L], *rm1 = rpl[L - 1], *rp1 = rpl[L + 1];
        const float *rm2 = rpl[L - 2], *rp2 = rpl[L + 2];
        const float *rm3 = L == 3 ? rpl[0] : rc, *rp3 = L == 3 ? rpl[2 * L] : rc;
        auto ld = [](const float *b, int i) { return *reinterpret_cast<const float2 *>(b + i); };
#pragma unroll
        for (int k = 0; k < RG::KM; ++k) {
            if (k * NT + tid >= RG::NPM) break;
            const int c = roff[k];
            const float2 r0 = ld(rc, c);
            const float2 lo = ld(rc, c - 2), hi = ld(rc, c + 2);
            // z neighbours of the pair (A = z, B = z + 1)
            const float2 zm1 = make_float2(lo.y, r0.x), zp1 = make_float2(r0.y, hi.x);
            const float2 n1 = axis_sum<O>(ld(rm1, c), ld(rp1, c), ld(rc, c - RZ), ld(rc, c + RZ), zm1, zp1);
            const float2 n2 = axis_sum<O>(ld(rm2, c), ld(rp2, c), ld(rc, c - 2 * RZ), ld(rc, c + 2 * RZ), lo, hi);
            float2 mu;
            if (L == 2) {
                mu = mu_lap5<O>(eos, p.kk, p.ka, r0, n1, n2);
            } else {
                const float2 lo3 = ld(rc, c - 4), hi3 = ld(rc, c + 4);
                const float2 n3 = axis_sum<O>(ld(rm3, c), ld(rp3, c), ld(rc, c - 3 * RZ), ld(rc, c + 3 * RZ),
                                              make_float2(lo3.y, lo.x), make_float2(hi.y, hi3.x));
                mu = mu_lap7<O>(eos, p.kk, p.ka, r0, n1, n2, n3);
            }
            if (wall_tile && (wflag[k] & 3)) {
                const float w = p.wall[((wflag[k] & 4) ? p.dx * p.dy : 0) + gx * p.dy + wcol[k]];
                if (wflag[k] & 1) mu.x = w;
                if (wflag[k] & 2) mu.y = w;
            }
            *reinterpret_cast<float4 *>(dst + moff[k]) = make_float4(r0.x, mu.x, r0.y, mu.y);
        }
    };

    // ---- this thread's node pair
    const int ty = tid / TH, tzp = tid - (tid / TH) * TH;
    const int gy = y0 + ty, gz = z0 + 2 * tzp;
    const bool dom = gy < p.dy && gz < p.dz;  // DZ even: z + 1 is inside too
    const bool fluA = dom && !solid_k(p.wall_mode, gz, p.dz), fluB = dom && !solid_k(p.wall_mode, gz + 1, p.dz);
    const bool act = fluA || fluB;
    // the pairs next to a wall: (2, 3) has its fluid node B on the bottom wall
    // layer, (dz-4, dz-3) its fluid node A under the top wall layer
    const bool botw = walled && gz == 2, topw = walled && gz == p.dz - 4;
    // a tile whose pairs need no wrap and have no solid neighbour
    const bool yz_plain = (walled ? (z0 >= 4 && z0 + TZ <= p.dz - 4) : (z0 >= 2 && z0 + TZ <= p.dz - 2)) &&
                          y0 >= 1 && y0 + TY <= p.dy - 1;
    // index corrections (mod 2^32) of sources across a periodic y / z edge;
    // a destination across the same edge takes the opposite correction
    const unsigned ysp = gy == 0 ? plane : 0u, ysm = gy == p.dy - 1 ? 0u - plane : 0u;  // cy = +1 / -1
    const unsigned zsA = (!walled && gz == 0) ? (unsigned)p.dz : 0u;          // node A, cz = +1
    const unsigned zsB = (!walled && gz + 1 == p.dz - 1) ? 0u - p.dz : 0u;    // node B, cz = -1
    auto slot = [&](int q, unsigned idx) -> S * { return slots(q, idx); };

    // moving populations of the pair in plane x (A-A read slots)
    auto fetch = [&](int x, T hv[Q - 1]) {
        if (!act) return;
        const int gx = wrap_small(x, p.dx);
        const unsigned I = (unsigned)gx * plane + (unsigned)(gy * p.dz + gz);
        if (P == 0) {
#pragma unroll
            for (int q = 1; q < Q; ++q) hv[q - 1] = *reinterpret_cast<const T *>(slot(q - 1, I));
            return;
        }
        const bool edge = !yz_plain || gx == 0 || gx == p.dx - 1;
        // source index I - off(q) + correction (mod 2^32): a source across a
        // periodic x / y edge lies dx * plane / plane further on
        const unsigned xsp = gx == 0 ? p.dx * plane : 0u, xsm = gx == p.dx - 1 ? 0u - p.dx * plane : 0u;
#pragma unroll
        for (int q = 1; q < Q; ++q) {
            unsigned src = I - (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q));
            if (edge) src += (cx(q) == 1 ? xsp : (cx(q) == -1 ? xsm : 0u)) + (cy(q) == 1 ? ysp : (cy(q) == -1 ? ysm : 0u));
            const S *b = slot(opp(q) - 1, 0);
            T v;
            if (cz(q) == 0) {
                v = *reinterpret_cast<const T *>(b + src);
            } else {
                const unsigned ca = (edge && cz(q) == 1) ? zsA : 0u, cb = (edge && cz(q) == -1) ? zsB : 0u;
                v = SP::make(b[src + ca], b[src + 1u + cb]);
                // a source on a wall layer: the node's own slot (half-way
                // bounce-back) -- node B of (2, 3) for cz = +1, node A of
                // (dz-4, dz-3) for cz = -1 (the other node of each is solid)
                if (cz(q) == 1 && botw) v = *reinterpret_cast<const T *>(slot(q - 1, I));
                if (cz(q) == -1 && topw) v = *reinterpret_cast<const T *>(slot(q - 1, I));
            }
            hv[q - 1] = v;
        }
    };

    // ---- prologue: mu of planes x0-3 .. x0+2, f0 of x0-1 .. x0+1
    for (int pl = rp0; pl <= rp0 + 2 * L; ++pl) issue_rho(pl);
    for (int pl = x0 - 1; pl <= x0 + 1; ++pl) issue_f0(pl);
    for (int y = x0 - 3; y <= x0 + 2; ++y) {
        wait_rho(y + L);
        comp_mu(y);
        __syncthreads();
        issue_rho(y + L + 1);
    }
    T hv[Q - 1];
    fetch(x0, hv);
    wait_f0(x0 - 1);
    wait_f0(x0);

    const int mc = (ty + 3) * MZ + 2 * tzp + 4;  // (rho, mu) ring element of node A (even)
    const int ac = (ty + 1) * AZ + 2 * tzp + 4;  // f0 ring element of node A (even)
    float mv2 = 0.f;
    for (int x = x0; x < x1; ++x) {
        wait_rho(x + 3 + L);
        wait_f0(x + 1);
        if (!ok) s_abort = 1;
        if (x + 1 < x1) {
            issue_rho(x + 4 + L);
            issue_f0(x + 2);
        }
        T hn[Q - 1];
        if (x + 1 < x1) fetch(x + 1, hn);
        comp_mu(x + 3);
        __syncthreads();
        if (s_abort) break;
        if (act) {
            // ---- force on both nodes from the (rho, mu) ring
            float2 la[9], lb[9];
#pragma unroll
            for (int l = 0; l < 9; ++l) {
                la[l] = lb[l] = make_float2(0.f, 0.f);
#pragma unroll
                for (int d = 1; d <= 3; ++d) {
                    const int ox = line_x(l) * d, oz = line_z(l) * d, mo = line_y(l) * d * MZ + oz;
                    const float2 *pa = rm_plane(x + ox), *pb = rm_plane(x - ox);
                    float2 aA, aB, bA, bB;
                    if ((oz & 1) == 0) {
                        const float4 a4 = *reinterpret_cast<const float4 *>(pa + mc + mo);
                        const float4 b4 = *reinterpret_cast<const float4 *>(pb + mc - mo);
                        aA = make_float2(a4.x, a4.y);
                        aB = make_float2(a4.z, a4.w);
                        bA = make_float2(b4.x, b4.y);
                        bB = make_float2(b4.z, b4.w);
                    } else {
                        aA = pa[mc + mo];
                        aB = pa[mc + mo + 1];
                        bA = pb[mc - mo];
                        bB = pb[mc - mo + 1];
                    }
                    la[l] = line_term(la[l], line_c(d), aA, bA);
                    lb[l] = line_term(lb[l], line_c(d), aB, bB);
                }
            }
            const float4 cen = *reinterpret_cast<const float4 *>(rm_plane(x) + mc);
            float FA[3], FB[3], grA[3], grB[3];
            force_from_lines<sizeof(S) == 4>(la, cen.x, FA, grA);  // exact scaling for FP32 storage
            force_from_lines<sizeof(S) == 4>(lb, cen.z, FB, grB);
            const float2 r = make_float2(cen.x, cen.z);

            // ---- decode with the sources' rest populations: g = h + 3 a
            const float *fa[3];
            {
                const int s0 = fslot(x - 1), s1 = s0 + 1 == NF ? 0 : s0 + 1, s2 = s1 + 1 == NF ? 0 : s1 + 1;
                fa[0] = sf0 + s0 * (AY * AZ);
                fa[1] = sf0 + s1 * (AY * AZ);
                fa[2] = sf0 + s2 * (AY * AZ);
            }
            auto col = [&](int ccx, int ccy, int dzo) -> float2 {
                return *reinterpret_cast<const float2 *>(fa[1 - ccx] + ac - ccy * AZ + dzo);
            };
            const float2 a0 = col(0, 0, 0);
            float2 g[Q];
            g[0] = a0;
#pragma unroll
            for (int q = 1; q < Q; ++q) {
                float2 a;
                if (cz(q) == 0) {
                    a = col(cx(q), cy(q), 0);
                } else if (cz(q) == 1) {  // sources z - 1, z
                    const float2 lo = col(cx(q), cy(q), -2), mid = col(cx(q), cy(q), 0);
                    a = botw ? a0 : make_float2(lo.y, mid.x);
                } else {                  // sources z + 1, z + 2
                    const float2 mid = col(cx(q), cy(q), 0), hi = col(cx(q), cy(q), 2);
                    a = topw ? a0 : make_float2(mid.y, hi.x);
                }
                g[q] = O::fma(O::k(3.f), a, SP::tof(hv[q - 1]));
            }
            float2 v2;
            if (p.qp) {
                float qa[Q], qb[Q];
                qp36_moments(p.k1, p.k2, grA, qa);
                qp36_moments(p.k1, p.k2, grB, qb);
                float2 qp[Q];
#pragma unroll
                for (int a = 0; a < Q; ++a) qp[a] = make_float2(qa[a], qb[a]);
                collide36<O, REF>(g, r, make_float2(FA[0], FB[0]), make_float2(FA[1], FB[1]), make_float2(FA[2], FB[2]),
                             p.ts, p.omts, qp, v2);
            } else {
                collide36<O, REF>(g, r, make_float2(FA[0], FB[0]), make_float2(FA[1], FB[1]), make_float2(FA[2], FB[2]),
                             p.ts, p.omts, nullptr, v2);
            }
            if (fluA) mv2 = fmaxf(mv2, v2.x);
            if (fluB) mv2 = fmaxf(mv2, v2.y);

            // ---- encode against the pair's new rest populations and stream
            const int gx = wrap_small(x, p.dx);
            const unsigned I = (unsigned)gx * plane + (unsigned)(gy * p.dz + gz);
            const float2 an = g[0];
            *reinterpret_cast<float2 *>(f0n + I) = an;
            if (P == 0) {
#pragma unroll
                for (int q = 1; q < Q; ++q)
                    *reinterpret_cast<T *>(slot(opp(q) - 1, I)) = SP::fromf(O::fma(O::k(-3.f), an, g[q]));
            } else {
                const bool edge = !yz_plain || gx == 0 || gx == p.dx - 1;
                const unsigned xsp = gx == 0 ? p.dx * plane : 0u, xsm = gx == p.dx - 1 ? 0u - p.dx * plane : 0u;
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const T v = SP::fromf(O::fma(O::k(-3.f), an, g[q]));
                    // destination I + off(q); across a periodic edge the
                    // source corrections of the opposite direction apply
                    unsigned dst = I + (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q));
                    if (edge) dst += (cx(q) == -1 ? xsp : (cx(q) == 1 ? xsm : 0u)) + (cy(q) == -1 ? ysp : (cy(q) == 1 ? ysm : 0u));
                    S *b = slot(q - 1, 0);
                    if (cz(q) == 0) {
                        *reinterpret_cast<T *>(b + dst) = v;
                    } else {
                        // node A's destination across the bottom periodic edge, node B's across the top;
                        // the solid node of a wall pair (A of (2, 3), B of (dz-4, dz-3)) stores
                        // nothing here: its z neighbour is the pair's fluid node
                        const unsigned ca = (edge && cz(q) == -1) ? zsA : 0u, cb = (edge && cz(q) == 1) ? zsB : 0u;
                        if (!botw) b[dst + ca] = SP::lo(v);
                        if (!topw) b[dst + 1u + cb] = SP::hi(v);
                        // half-way bounce-back: a destination on a wall layer returns to the node's own slot
                        if ((cz(q) == 1 && topw) || (cz(q) == -1 && botw))
                            *reinterpret_cast<T *>(slot(opp(q) - 1, I)) = v;
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < Q - 1; ++q) hv[q] = hn[q];
    }
    if (s_abort) {
        // a copy did not complete in time: report it; thread 0 waits (bounded)
        // for every copy the CTA issued and it has not seen complete, so the
        // CTA's shared memory outlives them
        if (tid == 0) {
            if (p.err) atomicOr(p.err, 1u);
            for (int q = r_got + 1; q <= r_iss; ++q) mbar_wait(rbar + rslot(q), rpar(q));
            for (int q = f_got + 1; q <= f_iss; ++q) mbar_wait(fbar + fslot(q), fpar(q));
        }
        return;
    }
    mvmax_flush(p, P, mv2);
}

// Registers: at most 128 per thread (two CTAs of 256 threads per SM).
template <int NT>
constexpr int pair_min_blocks()
{
    return NT >= 512 ? 1 : 512 / NT;
}

// REF: the MRT rates follow the reference's pattern (collide36)
template <class S, int TY, int TZ, int L, bool REF>
__global__ void __launch_bounds__(TY *TZ / 2, pair_min_blocks<TY * TZ / 2>())
    k_pair_collide(KParams<float> p, int P, SlotTable<S> slots, const float *__restrict__ f0c,
                   float *__restrict__ f0n, const float *__restrict__ rho, int xl)
{
    extern __shared__ __align__(128) float4 smem4[];
    pair_tile<S, TY, TZ, L, REF>(p, P, slots, f0c, f0n, rho, blockIdx.x * TZ, blockIdx.y * TY, blockIdx.z * xl, xl,
                            smem4);
}

}  // namespace cpmp
