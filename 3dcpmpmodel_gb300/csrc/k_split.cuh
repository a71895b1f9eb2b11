// k_split.cuh -- the FUSED step in two passes: a force pass (chemical
// potential and non-ideal force on a shared-memory tile) and a collide-stream
// pass with no shared memory.
//
// The one-pass kernels (k_pair.cuh, k_fused.cuh) evaluate mu, the force and
// the collision of a node in one CTA; the collision's registers then limit the
// stencil work to 16 warps per SM.  Here:
//
//   force pass   k_force_pass<TY, TZ, L>: a TY x TZ column tile marching over
//                x with the rho ring (cp.async.bulk rows on mbarriers) and the
//                (rho, mu) ring of the paired kernel; writes F = -rho grad(mu)
//                + grad(rho) / 3 of every node pair of the tile (and grad(rho)
//                when the K1/K2 term is on) to an FP32 field.  It has no
//                storage-type parameter: it reads only the density.
//   collide      k_node_collide<S, P, REF>: one z-adjacent node pair per
//                thread; reads its 18 moving populations (A-A addressing of
//                parity P), the rest populations of their sources, its density
//                and its force, collides and streams in place.  Loads come
//                straight from global memory (the source anchors of a block's
//                rows hit L1), so the kernel is bound by HBM bandwidth.
//
// The force is the paired kernel's line-sum stencil evaluated in the same
// order and passed through memory exactly, the decode, collision and encode
// are the same Lane2 code, so the two passes give exactly the bits of the
// one-pass kernels.  Requirements as for the paired kernel: DZ a multiple of 4.
#pragma once

#include "k_pair.cuh"

namespace cpmp {

// ------------------------------------------------------------ force pass ----
template <int TY, int TZ, int L>
struct ForceRings {
    static constexpr int NT = TY * TZ / 2, TH = TZ / 2;
    static constexpr int RH = 3 + L;
    static constexpr int RY = TY + 2 * RH, RZ = TZ + 16;  // rho ring rows, columns z0-8 ..
    static constexpr int NR = 2 * L + 2;                  // rho planes
    static constexpr int MY = TY + 6, MZ = TZ + 8, HM = MZ / 2;  // (rho, mu) ring, columns z0-4 ..
    static constexpr int NPM = MY * HM;                  // (rho, mu) pairs per plane
    static constexpr int KM = (NPM + NT - 1) / NT;       // pairs per thread per plane
    static constexpr size_t RHO_BYTES = sizeof(float) * NR * RY * RZ;
    static constexpr size_t RM_BYTES = sizeof(float2) * 8 * MY * MZ;
    static constexpr size_t BAR_BYTES = sizeof(unsigned long long) * NR;
    static constexpr size_t BYTES = RHO_BYTES + RM_BYTES + BAR_BYTES;
    static_assert(RY <= 32, "one lane per ring row");
    static_assert(TZ % 32 == 0, "tile height");
    static_assert(RHO_BYTES % 16 == 0 && RM_BYTES % 16 == 0, "16-byte ring slots");
};

// F field layout: component c of node I at F[c * n + I]; components 0-2 the
// force, 3-5 grad(rho) (written only with the K1/K2 term).
// EXACT: the force scaling for FP32 storage (force_from_lines).
template <int TY, int TZ, int L, bool EXACT>
__device__ __forceinline__ void force_tile(const KParams<float> &p, const float *__restrict__ rho,
                                           float *__restrict__ F, const int z0, const int y0, const int x0,
                                           const int xl, float4 *smem4)
{
    using RG = ForceRings<TY, TZ, L>;
    using O = Lane2;
    constexpr int RY = RG::RY, RZ = RG::RZ, NR = RG::NR, MY = RG::MY, MZ = RG::MZ, HM = RG::HM;
    constexpr int TH = RG::TH, NT = RG::NT;

    float *srho = reinterpret_cast<float *>(smem4);
    float2 *srm = reinterpret_cast<float2 *>(reinterpret_cast<char *>(smem4) + RG::RHO_BYTES);
    unsigned long long *rbar =
        reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(smem4) + RG::RHO_BYTES + RG::RM_BYTES);
    __shared__ int s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x1 = min(x0 + xl, p.dx);
    const unsigned plane = (unsigned)(p.dy * p.dz);
    const EosLane eos = make_eos_lane(p.eos, p.A, p.B, p.T);

    if (tid == 0) {
        for (int i = 0; i < NR; ++i) mbar_init(rbar + i, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    __syncthreads();

    // rho planes are issued in order from x0-3-L by warp 0
    const int rp0 = x0 - 3 - L;
    auto rslot = [&](int pl) { return (pl - rp0) % NR; };
    auto rpar = [&](int pl) { return (unsigned)(((pl - rp0) / NR) & 1); };
    auto rm_plane = [&](int pl) -> float2 * { return srm + (pl & 7) * (MY * MZ); };
    int r_iss = rp0 - 1, r_got = rp0 - 1;
    auto issue_rho = [&](int pl) {
        r_iss = pl;
        if (warp == 0)
            issue_plane(p, rho, pl, srho + rslot(pl) * (RY * RZ), RY, y0 - 3 - L, z0 - 8, RZ, rbar + rslot(pl), lane);
    };
    bool ok = true;
    auto wait_rho = [&](int pl) {
        for (int q = r_got + 1; ok && q <= pl; ++q) {
            ok = mbar_wait(rbar + rslot(q), rpar(q));
            if (ok) r_got = q;
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
    const bool dom = gy < p.dy && gz < p.dz;
    const bool act = dom && (!solid_k(p.wall_mode, gz, p.dz) || !solid_k(p.wall_mode, gz + 1, p.dz));
    const size_t n = (size_t)p.n;

    // ---- prologue: mu of planes x0-3 .. x0+2
    for (int pl = rp0; pl <= rp0 + 2 * L; ++pl) issue_rho(pl);
    for (int y = x0 - 3; y <= x0 + 2; ++y) {
        wait_rho(y + L);
        comp_mu(y);
        __syncthreads();
        issue_rho(y + L + 1);
    }

    const int mc = (ty + 3) * MZ + 2 * tzp + 4;  // (rho, mu) ring element of node A (even)
    for (int x = x0; x < x1; ++x) {
        wait_rho(x + 3 + L);
        if (!ok) s_abort = 1;
        if (x + 1 < x1) issue_rho(x + 4 + L);
        comp_mu(x + 3);
        __syncthreads();
        if (s_abort) break;
        if (act) {
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
            force_from_lines<EXACT>(la, cen.x, FA, grA);
            force_from_lines<EXACT>(lb, cen.z, FB, grB);
            const int gx = wrap_small(x, p.dx);
            float *out = F + ((size_t)gx * plane + (size_t)(gy * p.dz + gz));
#pragma unroll
            for (int c = 0; c < 3; ++c) *reinterpret_cast<float2 *>(out + c * n) = make_float2(FA[c], FB[c]);
            if (p.qp) {
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    *reinterpret_cast<float2 *>(out + (3 + c) * n) = make_float2(grA[c], grB[c]);
            }
        }
    }
    if (s_abort) {
        // a copy did not complete in time: report it; thread 0 waits (bounded)
        // for every copy the CTA issued and it has not seen complete, so the
        // CTA's shared memory outlives them
        if (tid == 0) {
            if (p.err) atomicOr(p.err, 1u);
            for (int q = r_got + 1; q <= r_iss; ++q) mbar_wait(rbar + rslot(q), rpar(q));
        }
    }
}

// Registers: at most 128 per thread with 256 threads; shared memory decides
// how many CTAs share an SM.
template <int TY, int TZ, int L, bool EXACT>
__global__ void __launch_bounds__(TY *TZ / 2, pair_min_blocks<TY * TZ / 2>())
    k_force_pass(KParams<float> p, const float *__restrict__ rho, float *__restrict__ F, int xl)
{
    extern __shared__ __align__(128) float4 smem4[];
    force_tile<TY, TZ, L, EXACT>(p, rho, F, blockIdx.x * TZ, blockIdx.y * TY, blockIdx.z * xl, xl, smem4);
}

// --------------------------------------------------------- collide pass ----
// Block: NCZ node pairs along z (one warp per row) x NCY rows of y; grid
// (pair blocks, row blocks, dx).  The rest populations of a node pair's
// sources lie in the nine columns (x - cx, y - cy); a block's rows share most
// of them, so those loads hit L1.
constexpr int NCZ = 32, NCY = 8;

template <class S, int P, bool REF>
__global__ void __launch_bounds__(NCZ *NCY, 2)
    k_node_collide(KParams<float> p, SlotTable<S> slots, const float *__restrict__ f0c, float *__restrict__ f0n,
                   const float *__restrict__ rho, const float *__restrict__ F)
{
    using SP = SPair<S>;
    using T = typename SP::T;
    using O = Lane2;
    const int gz = 2 * (int)(blockIdx.x * NCZ + threadIdx.x);
    const int gy = (int)(blockIdx.y * NCY + threadIdx.y), gx = (int)blockIdx.z;
    const bool walled = p.wall_mode == 1;
    const bool dom = gy < p.dy && gz < p.dz;  // DZ even: z + 1 is inside too
    const bool fluA = dom && !solid_k(p.wall_mode, gz, p.dz), fluB = dom && !solid_k(p.wall_mode, gz + 1, p.dz);
    const bool act = fluA || fluB;
    float mv2 = 0.f;
    if (act) {
        const int dy = p.dy, dz = p.dz;
        const unsigned plane = (unsigned)(dy * dz);
        const size_t n = (size_t)p.n;
        const unsigned I = (unsigned)gx * plane + (unsigned)(gy * dz + gz);
        // the pairs next to a wall: (2, 3) has its fluid node B on the bottom
        // wall layer, (dz-4, dz-3) its fluid node A under the top wall layer
        const bool botw = walled && gz == 2, topw = walled && gz == dz - 4;
        // column (x - a, y - b) of the box, periodic in x and y: index of its z = 0
        const int xm = gx == 0 ? p.dx - 1 : gx - 1, xp = gx == p.dx - 1 ? 0 : gx + 1;
        const int ym = gy == 0 ? dy - 1 : gy - 1, yp = gy == dy - 1 ? 0 : gy + 1;
        auto col = [&](int a, int b) -> unsigned {
            const int xs = a == 1 ? xm : (a == -1 ? xp : gx), ys = b == 1 ? ym : (b == -1 ? yp : gy);
            return (unsigned)xs * plane + (unsigned)(ys * dz);
        };
        // z of the source / destination one node away (periodic boxes wrap;
        // in a walled box an active pair never reaches past z = 0 or dz - 1)
        const int zA_m = gz == 0 ? dz - 1 : gz - 1;     // node A, z - 1
        const int zB_p = gz + 2 == dz ? 0 : gz + 2;     // node B, z + 1
        const int zlo = gz == 0 ? dz - 2 : gz - 2;      // anchor pair below
        const int zhi = gz + 2 == dz ? 0 : gz + 2;      // anchor pair above

        // ---- moving populations (A-A read slots) and the sources' rest populations
        T hv[Q - 1];
#pragma unroll
        for (int q = 1; q < Q; ++q) {
            if (P == 0) {
                hv[q - 1] = *reinterpret_cast<const T *>(slots(q - 1, I));
                continue;
            }
            const unsigned c = col(cx(q), cy(q));
            const S *b = slots(opp(q) - 1, 0);
            T v;
            if (cz(q) == 0) {
                v = *reinterpret_cast<const T *>(b + c + gz);
            } else if (cz(q) == 1) {  // sources z - 1, z
                v = SP::make(b[c + zA_m], b[c + gz]);
                // a source on a wall layer: the node's own slot (half-way bounce-back)
                if (botw) v = *reinterpret_cast<const T *>(slots(q - 1, I));
            } else {                  // sources z + 1, z + 2
                v = SP::make(b[c + gz + 1], b[c + zB_p]);
                if (topw) v = *reinterpret_cast<const T *>(slots(q - 1, I));
            }
            hv[q - 1] = v;
        }
        const float2 a0 = *reinterpret_cast<const float2 *>(f0c + I);
        float2 an[Q];
#pragma unroll
        for (int q = 1; q < Q; ++q) {
            if (cz(q) != 0 || (cx(q) == 0 && cy(q) == 0)) continue;
            // column (cx, cy): mid serves cz = 0, with lo / hi also cz = +1 / -1
            const unsigned c = col(cx(q), cy(q));
            const float2 mid = *reinterpret_cast<const float2 *>(f0c + c + gz);
            const bool axis = cx(q) == 0 || cy(q) == 0;
            float2 lo = mid, hi = mid;
            if (axis) {
                lo = *reinterpret_cast<const float2 *>(f0c + c + zlo);
                hi = *reinterpret_cast<const float2 *>(f0c + c + zhi);
            }
#pragma unroll
            for (int r = 1; r < Q; ++r) {
                if (cx(r) != cx(q) || cy(r) != cy(q)) continue;
                an[r] = cz(r) == 0 ? mid : (cz(r) == 1 ? make_float2(lo.y, mid.x) : make_float2(mid.y, hi.x));
            }
        }
        {   // the pair's own column: cz = +1 / -1
            const float2 lo = *reinterpret_cast<const float2 *>(f0c + col(0, 0) + zlo);
            const float2 hi = *reinterpret_cast<const float2 *>(f0c + col(0, 0) + zhi);
            an[5] = make_float2(lo.y, a0.x);
            an[6] = make_float2(a0.y, hi.x);
        }
        const float2 r = *reinterpret_cast<const float2 *>(rho + I);
        const float2 Fx = *reinterpret_cast<const float2 *>(F + I);
        const float2 Fy = *reinterpret_cast<const float2 *>(F + n + I);
        const float2 Fz = *reinterpret_cast<const float2 *>(F + 2 * n + I);

        // ---- decode with the sources' rest populations: g = h + 3 a
        float2 g[Q];
        g[0] = a0;
#pragma unroll
        for (int q = 1; q < Q; ++q) {
            float2 a = an[q];
            if (cz(q) == 1 && botw) a = a0;
            if (cz(q) == -1 && topw) a = a0;
            g[q] = O::fma(O::k(3.f), a, SP::tof(hv[q - 1]));
        }
        float2 v2;
        if (p.qp) {
            float grA[3], grB[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 gr = *reinterpret_cast<const float2 *>(F + (3 + c) * n + I);
                grA[c] = gr.x;
                grB[c] = gr.y;
            }
            float qa[Q], qb[Q];
            qp36_moments(p.k1, p.k2, grA, qa);
            qp36_moments(p.k1, p.k2, grB, qb);
            float2 qp[Q];
#pragma unroll
            for (int a = 0; a < Q; ++a) qp[a] = make_float2(qa[a], qb[a]);
            collide36<O, REF>(g, r, Fx, Fy, Fz, p.ts, p.omts, qp, v2);
        } else {
            collide36<O, REF>(g, r, Fx, Fy, Fz, p.ts, p.omts, nullptr, v2);
        }
        if (fluA) mv2 = fmaxf(mv2, v2.x);
        if (fluB) mv2 = fmaxf(mv2, v2.y);

        // ---- encode against the pair's new rest populations and stream
        const float2 a1 = g[0];
        *reinterpret_cast<float2 *>(f0n + I) = a1;
#pragma unroll
        for (int q = 1; q < Q; ++q) {
            const T v = SP::fromf(O::fma(O::k(-3.f), a1, g[q]));
            if (P == 0) {
                *reinterpret_cast<T *>(slots(opp(q) - 1, I)) = v;
                continue;
            }
            // destination column (x + cx, y + cy)
            const unsigned c = col(-cx(q), -cy(q));
            S *b = slots(q - 1, 0);
            if (cz(q) == 0) {
                *reinterpret_cast<T *>(b + c + gz) = v;
            } else {
                // node A's destination z + cz, node B's z + 1 + cz; the solid
                // node of a wall pair (A of (2, 3), B of (dz-4, dz-3)) stores
                // nothing here: its z neighbour is the pair's fluid node
                const unsigned da = cz(q) == 1 ? (unsigned)(gz + 1) : (unsigned)zA_m;
                const unsigned db = cz(q) == 1 ? (unsigned)zB_p : (unsigned)gz;
                if (!botw) b[c + da] = SP::lo(v);
                if (!topw) b[c + db] = SP::hi(v);
                // half-way bounce-back: a destination on a wall layer returns to the node's own slot
                if ((cz(q) == 1 && topw) || (cz(q) == -1 && botw))
                    *reinterpret_cast<T *>(slots(opp(q) - 1, I)) = v;
            }
        }
    }
    mvmax_flush(p, P, mv2);
}

}  // namespace cpmp
