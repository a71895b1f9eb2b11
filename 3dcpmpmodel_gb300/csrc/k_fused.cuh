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

#include "lane_math.cuh"
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

// The 18 moving-population arrays (slot k holds direction k + 1 of the A-A
// addressing): as base pointers in the launch's parameter space, so that an
// access is one multiply-add on a constant operand, in shared memory (the
// items and the density blocks of a batch, whose boxes differ).
template <class S>
struct SlotTable {
    S *q[Q - 1];
    __device__ __forceinline__ S *operator()(int k, unsigned idx) const { return q[k] + idx; }
};
template <class S>
struct SlotShared {
    S *const *q;  // shared-memory copy of the item's box pointers
    __device__ __forceinline__ S *operator()(int k, unsigned idx) const { return q[k] + idx; }
};


// w_q / w_0 and 1 / w_q
__host__ __device__ __forceinline__ constexpr float ratio0(int q) { return q <= 6 ? 1.0f / 6.0f : 1.0f / 12.0f; }
__host__ __device__ __forceinline__ constexpr float inv_w(int q) { return q <= 6 ? 18.0f : 36.0f; }

// Decoded population: f = w_q h + (w_q / w_0) a, evaluated with explicit
// rounding (no FMA contraction) so every kernel that decodes the same stored
// value gets the same float.
template <class S>
__device__ __forceinline__ float decode_pop(int q, S hv, float a)
{
    return __fadd_rn(__fmul_rn(wgt<float>(q), s2f<S>(hv)), __fmul_rn(ratio0(q), a));
}

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
        f[q] = __fadd_rn(__fmul_rn(wgt<float>(q), hv), __fmul_rn(ratio0(q), a));
    }
}

// ------------------------------------------------------------ density ----
// Is every node of the z-range [z0, z0+tz) and all its +-1 neighbours a fluid
// node that needs no z wrap?
__device__ __forceinline__ bool z_interior(const KParams<float> &p, int z0, int tz)
{
    return p.wall_mode == 1 ? (z0 >= 4 && z0 + tz <= p.dz - 4) : (z0 >= 1 && z0 + tz <= p.dz - 1);
}

// rho = sum of the post-stream populations (MacroCalculate's density,
// FluidCuda.cu:357-361) on fluid nodes, in the collision's scaled form: each
// population decoded as g = h + 3 a (the collide's decode), rho = f_0 +
// (2 ES + DS) / 36 (mass_sums, correctly rounded division).  The general path,
// for nodes next to a wall or a periodic edge.
template <class S>
__device__ __forceinline__ void density_node(const KParams<float> &p, int P, const S *__restrict__ h,
                                             const float *__restrict__ f0, float *__restrict__ rho, int i, int j,
                                             int k)
{
    if (solid_k(p.wall_mode, k, p.dz)) return;
    const long long I = ((long long)i * p.dy + j) * p.dz + k;
    const long long n = p.n;
    const float a0 = f0[I];
    float g[Q];
#pragma unroll
    for (int q = 1; q < Q; ++q) {
        const int si = wrap1(i - cx(q), p.dx), sj = wrap1(j - cy(q), p.dy), sk = wrap1(k - cz(q), p.dz);
        const bool ss = solid_k(p.wall_mode, sk, p.dz);
        const long long src = ((long long)si * p.dy + sj) * p.dz + sk;
        const float a = ss ? a0 : __ldg(f0 + src);
        const float hv = s2f<S>((P == 0 || ss) ? h[(long long)(q - 1) * n + I] : h[(long long)(opp(q) - 1) * n + src]);
        g[q] = fmaf(3.f, a, hv);
    }
    float ES, DS;
    mass_sums<Lane1>(g, ES, DS);
    rho[I] = a0 + div36(fmaf(2.f, ES, DS));
}

// Two stored values of consecutive nodes as a float pair: one vector load
// when the first index is even, two scalar loads otherwise.
template <class S>
__device__ __forceinline__ float2 load_pair(const S *__restrict__ ptr, bool even);
template <>
__device__ __forceinline__ float2 load_pair<float>(const float *__restrict__ ptr, bool even)
{
    return even ? *reinterpret_cast<const float2 *>(ptr) : make_float2(ptr[0], ptr[1]);
}
template <>
__device__ __forceinline__ float2 load_pair<__half>(const __half *__restrict__ ptr, bool even)
{
    return even ? __half22float2(*reinterpret_cast<const __half2 *>(ptr))
                : make_float2(__half2float(ptr[0]), __half2float(ptr[1]));
}
template <>
__device__ __forceinline__ float2 load_pair<__nv_bfloat16>(const __nv_bfloat16 *__restrict__ ptr, bool even)
{
    return even ? __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(ptr))
                : make_float2(__bfloat162float(ptr[0]), __bfloat162float(ptr[1]));
}

// Two stored values of consecutive nodes kept packed (one register for FP16
// and BF16) from the load until the decode, and their conversion to floats
// (exact, the same floats as load_pair's).
template <class S>
struct Packed;
template <>
struct Packed<__half> {
    using T = __half2;
    static __device__ __forceinline__ T load(const __half *p, bool even)
    {
        return even ? *reinterpret_cast<const __half2 *>(p) : __halves2half2(p[0], p[1]);
    }
    static __device__ __forceinline__ float2 tof(T v) { return __half22float2(v); }
};
template <>
struct Packed<__nv_bfloat16> {
    using T = __nv_bfloat162;
    static __device__ __forceinline__ T load(const __nv_bfloat16 *p, bool even)
    {
        return even ? *reinterpret_cast<const __nv_bfloat162 *>(p) : __halves2bfloat162(p[0], p[1]);
    }
    static __device__ __forceinline__ float2 tof(T v) { return __bfloat1622float2(v); }
};
template <>
struct Packed<float> {
    using T = float2;
    static __device__ __forceinline__ T load(const float *p, bool even)
    {
        return even ? *reinterpret_cast<const float2 *>(p) : make_float2(p[0], p[1]);
    }
    static __device__ __forceinline__ float2 tof(T v) { return v; }
};

// Is node k of a column one whose 18 sources are fluid nodes with no z wrap?
__device__ __forceinline__ bool z_plain(const KParams<float> &p, int k)
{
    return p.wall_mode == 1 ? (k >= 4 && k <= p.dz - 5) : (k >= 1 && k <= p.dz - 2);
}

// Paired density of nodes I and I + 1 (I even, both with plain sources), in
// paired FP32 (the sums of density_node).  With
// an even DZ every pair of loads has a parity known at compile time (node
// index and N even, so it is that of cz(q)) and aligned pairs are vector
// loads; otherwise all moving-population and anchor loads are scalar (vector
// loads where a pair's address happens to be aligned, chosen at run time,
// measured slower: the two load paths cost more than the loads they save).
// Every load is issued before the first add so their latencies overlap.
// botw / topw (even DZ only): the pair is (2, 3) / (dz-4, dz-3) of an x/y-
// interior column of a walled box: its fluid node's sources across the wall
// layer are its own slots and rest population (density_wall_node's sums, by
// selects instead of a per-node path), and only the fluid node is written.
template <class S, int P, bool EVEN, class SL>
__device__ __forceinline__ void density_pair_fast(const KParams<float> &p, const SL &slots,
                                                  const float *__restrict__ f0, float *__restrict__ rho,
                                                  unsigned I, bool botw = false, bool topw = false)
{
    // node indices are 32-bit (the FUSED scheme keeps N below 2^32); the
    // neighbour offsets are applied as signed pointer offsets from the node's
    // own addresses, so the nine in-plane parts are shared and the z part is
    // an immediate
    const int plane = p.dy * p.dz;
    const float *fI = f0 + I;
    // the moving populations stay packed until the decode, so the 18 pairs and
    // the anchors fit the register budget without reloads
    typename Packed<S>::T hv[Q - 1];
    float2 a[Q - 1];
#pragma unroll
    for (int q = 1; q < Q; ++q) {
        const int off = cx(q) * plane + cy(q) * p.dz + cz(q);
        const S *hp = P == 0 ? slots(q - 1, I) : slots(opp(q) - 1, I) - off;
        const bool odd_off = (cz(q) & 1) != 0;
        hv[q - 1] = Packed<S>::load(hp, EVEN && (P == 0 || !odd_off));
        // a source on a wall layer: the node's own slot (half-way bounce-back)
        if (EVEN && P == 1 && cz(q) == 1 && botw) hv[q - 1] = Packed<S>::load(slots(q - 1, I), true);
        if (EVEN && P == 1 && cz(q) == -1 && topw) hv[q - 1] = Packed<S>::load(slots(q - 1, I), true);
        if (!EVEN) a[q - 1] = load_pair<float>(fI - off, false);
    }
    if (EVEN) {
        // anchors: in the source column (cx, cy) of the pair, direction cz
        // needs the rest populations at z = k0 - cz and k0 + 1 - cz; the
        // aligned pairs below k0, at k0 and above k0 + 1 hold all of them
        auto column = [&](int ccx, int ccy, float2 &lo, float2 &mid, float2 &hi) {
            const float *b = fI - (ccx * plane + ccy * p.dz);
            lo = *reinterpret_cast<const float2 *>(b - 2);
            mid = *reinterpret_cast<const float2 *>(b);
            hi = *reinterpret_cast<const float2 *>(b + 2);
        };
#pragma unroll
        for (int q = 1; q < Q; ++q) {
            if (cz(q) != 0 || (cx(q) != 0 && cy(q) != 0)) continue;  // diagonal in-plane: below
            if (cx(q) == 0 && cy(q) == 0) continue;
            float2 lo, mid, hi;
            column(cx(q), cy(q), lo, mid, hi);
            // every q' sharing this column: cz' = 0 (this q), +1, -1
#pragma unroll
            for (int r2 = 1; r2 < Q; ++r2) {
                if (cx(r2) != cx(q) || cy(r2) != cy(q)) continue;
                a[r2 - 1] = cz(r2) == 0 ? mid : (cz(r2) == 1 ? make_float2(lo.y, mid.x) : make_float2(mid.y, hi.x));
            }
        }
        {   // the pair's own column (cz = +1, -1)
            const float2 lo = *reinterpret_cast<const float2 *>(fI - 2), hi = *reinterpret_cast<const float2 *>(fI + 2);
            const float2 mid = *reinterpret_cast<const float2 *>(fI);
#pragma unroll
            for (int r2 = 1; r2 < Q; ++r2)
                if (cx(r2) == 0 && cy(r2) == 0)
                    a[r2 - 1] = cz(r2) == 1 ? make_float2(lo.y, mid.x) : make_float2(mid.y, hi.x);
        }
#pragma unroll
        for (int q = 1; q < Q; ++q)  // in-plane diagonals: cz = 0 only
            if (cz(q) == 0 && cx(q) != 0 && cy(q) != 0)
                a[q - 1] = *reinterpret_cast<const float2 *>(fI - (cx(q) * plane + cy(q) * p.dz));
        // a source on a wall layer: the node's own rest population
        const float2 own = *reinterpret_cast<const float2 *>(fI);
#pragma unroll
        for (int q = 1; q < Q; ++q) {
            if (cz(q) == 1 && botw) a[q - 1] = own;
            if (cz(q) == -1 && topw) a[q - 1] = own;
        }
    }
    float2 g[Q];
#pragma unroll
    for (int q = 1; q < Q; ++q) g[q] = Lane2::fma(Lane2::k(3.f), a[q - 1], Packed<S>::tof(hv[q - 1]));
    float2 ES, DS;
    mass_sums<Lane2>(g, ES, DS);
    const float2 a0 = *reinterpret_cast<const float2 *>(f0 + I);
    const float2 r = Lane2::add(a0, Lane2::div36(Lane2::fma(Lane2::k(2.f), ES, DS)));
    if (botw) rho[I + 1] = r.y;       // node I is on the bottom wall layer
    else if (topw) rho[I] = r.x;      // node I + 1 is on the top wall layer
    else *reinterpret_cast<float2 *>(rho + I) = r;
}

// Density of one fluid node k of an x/y-interior column of a walled box
// (wall_mode 1): the sums of density_node with each source across the wall
// layer (k = 3 or dz - 4) replaced by the node's own slot and rest population.
template <class S, class SL>
__device__ __forceinline__ void density_wall_node(const KParams<float> &p, int P, const SL &slots,
                                                  const float *__restrict__ f0, float *__restrict__ rho,
                                                  unsigned I, int k)
{
    const int plane = p.dy * p.dz;
    const bool lo = k == 3, hi = k == p.dz - 4;
    const float a0 = f0[I];
    float hv[Q - 1], a[Q - 1];
#pragma unroll
    for (int q = 1; q < Q; ++q) {
        const unsigned src = I - (unsigned)(cx(q) * plane + cy(q) * p.dz + cz(q));
        const bool ss = (cz(q) == 1 && lo) || (cz(q) == -1 && hi);
        hv[q - 1] = s2f<S>(*((P == 0 || ss) ? slots(q - 1, I) : slots(opp(q) - 1, src)));
        a[q - 1] = ss ? a0 : f0[src];
    }
    float g[Q];
#pragma unroll
    for (int q = 1; q < Q; ++q) g[q] = fmaf(3.f, a[q - 1], hv[q - 1]);
    float ES, DS;
    mass_sums<Lane1>(g, ES, DS);
    rho[I] = a0 + div36(fmaf(2.f, ES, DS));
}

// density_wall_node for a fluid node of an x or y edge column of a walled
// box: the sources wrap in x and y (periodic), never in z.
template <class S, class SL>
__device__ __forceinline__ void density_edge_node(const KParams<float> &p, int P, const SL &slots,
                                                  const float *__restrict__ f0, float *__restrict__ rho, int i,
                                                  int j, int k, unsigned I)
{
    const bool lo = k == 3, hi = k == p.dz - 4;
    const float a0 = f0[I];
    float hv[Q - 1], a[Q - 1];
#pragma unroll
    for (int q = 1; q < Q; ++q) {
        const int si = wrap1(i - cx(q), p.dx), sj = wrap1(j - cy(q), p.dy);
        const unsigned src = ((unsigned)si * p.dy + sj) * p.dz + (k - cz(q));
        const bool ss = (cz(q) == 1 && lo) || (cz(q) == -1 && hi);
        hv[q - 1] = s2f<S>(*((P == 0 || ss) ? slots(q - 1, I) : slots(opp(q) - 1, src)));
        a[q - 1] = ss ? a0 : f0[src];
    }
    float g[Q];
#pragma unroll
    for (int q = 1; q < Q; ++q) g[q] = fmaf(3.f, a[q - 1], hv[q - 1]);
    float ES, DS;
    mass_sums<Lane1>(g, ES, DS);
    rho[I] = a0 + div36(fmaf(2.f, ES, DS));
}

// Density of the nodes k0 and k0 + 1 of column (i, j) (either may lie
// outside [0, dz)); the node index of k0 is even (see pair_k0).  Pairs next
// to a z wall in an x/y-interior column take density_wall_node, pairs in an
// x or y edge column of a walled box density_edge_node, pairs at a periodic
// z edge the general per-node path.
template <class S, class SL>
__device__ __forceinline__ void density_pair(const KParams<float> &p, int P, const S *__restrict__ h,
                                             const SL &slots, const float *__restrict__ f0,
                                             float *__restrict__ rho, int i, int j, int k0)
{
    const bool in0 = k0 >= 0 && k0 < p.dz, in1 = k0 + 1 >= 0 && k0 + 1 < p.dz;
    const bool xy = i >= 1 && i + 1 < p.dx && j >= 1 && j + 1 < p.dy;
    if ((p.dz & 1) == 0 && p.wall_mode == 1 && xy) {
        // every pair of an x/y-interior column of a walled box with even DZ
        // (k0 even): the wall-adjacent pairs take the paired path with selects
        if (k0 < 2 || k0 > p.dz - 4) return;  // both nodes on wall layers
        const unsigned I = ((unsigned)i * p.dy + j) * p.dz + k0;
        const bool botw = k0 == 2, topw = k0 == p.dz - 4;
        if (P == 0) density_pair_fast<S, 0, true>(p, slots, f0, rho, I, botw, topw);
        else density_pair_fast<S, 1, true>(p, slots, f0, rho, I, botw, topw);
        return;
    }
    const bool fast = in0 && in1 && xy && z_plain(p, k0) && z_plain(p, k0 + 1);
    if (!fast) {
        const unsigned I = ((unsigned)i * p.dy + j) * p.dz + k0;
        if (xy && p.wall_mode == 1) {
            if (in0 && !solid_k(1, k0, p.dz)) density_wall_node<S>(p, P, slots, f0, rho, I, k0);
            if (in1 && !solid_k(1, k0 + 1, p.dz)) density_wall_node<S>(p, P, slots, f0, rho, I + 1, k0 + 1);
            return;
        }
        if (p.wall_mode == 1) {
            if (in0 && !solid_k(1, k0, p.dz)) density_edge_node<S>(p, P, slots, f0, rho, i, j, k0, I);
            if (in1 && !solid_k(1, k0 + 1, p.dz)) density_edge_node<S>(p, P, slots, f0, rho, i, j, k0 + 1, I + 1);
            return;
        }
        if (in0) density_node<S>(p, P, h, f0, rho, i, j, k0);
        if (in1) density_node<S>(p, P, h, f0, rho, i, j, k0 + 1);
        return;
    }
    const unsigned I = ((unsigned)i * p.dy + j) * p.dz + k0;
    if ((p.dz & 1) == 0) {
        if (P == 0) density_pair_fast<S, 0, true>(p, slots, f0, rho, I);
        else density_pair_fast<S, 1, true>(p, slots, f0, rho, I);
    } else {
        if (P == 0) density_pair_fast<S, 0, false>(p, slots, f0, rho, I);
        else density_pair_fast<S, 1, false>(p, slots, f0, rho, I);
    }
}

// First node of the pair thread t of column (i, j) handles: pairs start on
// even node indices, so a column whose first index is odd begins with a lone
// node (k0 = -1).  An even DZ makes every column start on an even index
// (DZ / 2 pairs); an odd one needs (DZ + 1) / 2 pairs whichever the parity.
__device__ __forceinline__ int pair_k0(const KParams<float> &p, int i, int j, int t)
{
    const long long base = ((long long)i * p.dy + j) * p.dz;
    return 2 * t - (int)(base & 1);
}

// The box of block g of a batch's flattened grid: the last box whose first
// block (first(box)) is at most g; boxes with no blocks share the next box's
// first block and are skipped.
template <class F>
__device__ __forceinline__ int batch_box_of(const BatchBox *__restrict__ boxes, int nbox, long long g, F first)
{
    int lo = 0, hi = nbox - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first(boxes[mid]) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}


// Block: 32 pairs of a column x 4 columns (y); grid (pair blocks, y blocks,
// dx).  The anchors of the y +- 1 neighbours of a block's nodes are mostly
// rows that the same block reads, so they come from L1.
template <class S>
__global__ void __launch_bounds__(DENSITY_BZ *DENSITY_BY, 8) k_density(KParams<float> p, int P,
                                                                     const S *__restrict__ h,
                                                                     SlotTable<const S> slots,
                                                                     const float *__restrict__ f0,
                                                                     float *__restrict__ rho)
{
    const int ppc = pairs_per_column(p.dz);
    const int t = blockIdx.x * DENSITY_BZ + threadIdx.x, j = blockIdx.y * DENSITY_BY + threadIdx.y;
    if (t >= ppc || j >= p.dy) return;
    const int i = blockIdx.z;
    // pairs rotated by two: the two wall-adjacent pairs of a walled column
    // (1 and ppc - 2) land in the column's last warp, the only one whose
    // lanes then take two paths
    const int tr = (t + 2) % ppc;
    density_pair<S>(p, P, h, slots, f0, rho, i, j, pair_k0(p, i, j, tr));
}

// --------------------------------------------------------- fused step ----
__device__ __forceinline__ int wrap_small(int a, int n)
{
    while (a < 0) a += n;
    while (a >= n) a -= n;
    return a;
}

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// The shared-memory rings of a fused-collide CTA that owns a TY x TZ column
// tile of (y, z) and marches over x with NT threads:
//   rho : planes x+3-L .. x+4+L, halo 3+L (L = 2: five-point Laplacian, 3: seven-point)
//   (rho, mu) pairs: planes x-3 .. x+3, halo 3 (the force stencil's support)
//   f0  : planes x-1 .. x+2, halo 1 in y and AZH in z (anchors of the moving
//         populations; AZH = 2 keeps node pairs on even indices)
// Ring sizes are powers of two so a plane's slot is (x & (size - 1)), also for
// the negative x of the prologue.  Per-tile element tables (built once,
// fixed for the whole march) give each ring element its offset in an x plane
// and each (rho, mu) element its centre in the rho plane, solid flag and wall
// offset, so the per-plane loops run a fixed trip count without division.
template <int TY, int TZ, int L, int NT, int AZH>
struct FusedRings {
    static constexpr int RH = 3 + L;
    static constexpr int RY = TY + 2 * RH, RZ = TZ + 2 * RH;
    static constexpr int NR = 8;
    static_assert(2 * L + 2 <= NR, "rho ring too small");
    static constexpr int MY = TY + 6, MZ = TZ + 6;
    static constexpr int AY = TY + 2, AZ = TZ + 2 * AZH;
    static constexpr int RHO_FLOATS = ((NR * RY * RZ + 3) / 4) * 4;
    static constexpr int RM_PAIRS = 8 * MY * MZ;
    static constexpr int F0_FLOATS = ((4 * AY * AZ + 3) / 4) * 4;
    static constexpr int MTAB_INT2 = MY * MZ;
    static constexpr int TAB_INTS = 2 * RY + RZ + RY * RZ + AY * AZ;
    static constexpr size_t BYTES = ((sizeof(float) * RHO_FLOATS + sizeof(float2) * RM_PAIRS +
                                      sizeof(float) * F0_FLOATS + sizeof(int2) * MTAB_INT2 +
                                      sizeof(int) * TAB_INTS + 15) / 16) * 16;
    static constexpr int KR = (RY * RZ + NT - 1) / NT, KA = (AY * AZ + NT - 1) / NT;
    static constexpr int KM = (MY * MZ + NT - 1) / NT;

    const KParams<float> &p;
    const float *rho, *f0c;
    unsigned plane;
    EosLane eos;
    float *srho;
    float2 *srm;
    float *sf0;
    int2 *mtab;
    int *tabY, *tabZ, *tabYdz, *offR, *offA;

    __device__ __forceinline__ FusedRings(const KParams<float> &p_, const float *rho_, const float *f0c_,
                                          float4 *smem4)
        : p(p_), rho(rho_), f0c(f0c_), plane((unsigned)(p_.dy * p_.dz)),
          eos(make_eos_lane(p_.eos, p_.A, p_.B, p_.T))
    {
        srho = reinterpret_cast<float *>(smem4);
        srm = reinterpret_cast<float2 *>(srho + RHO_FLOATS);
        sf0 = reinterpret_cast<float *>(srm + RM_PAIRS);
        mtab = reinterpret_cast<int2 *>(sf0 + F0_FLOATS);
        tabY = reinterpret_cast<int *>(mtab + MTAB_INT2);
        tabZ = tabY + RY;
        tabYdz = tabZ + RZ;    // wrapped y row times dz
        offR = tabYdz + RY;    // rho ring element -> offset in its x plane
        offA = offR + RY * RZ; // anchor ring element -> offset in its x plane
    }

    // wrapped y / z coordinates of the halo rows and columns, then the element tables
    __device__ __forceinline__ void setup(int y0, int z0)
    {
        for (int e = threadIdx.x; e < RY + RZ; e += NT) {
            if (e < RY) {
                tabY[e] = wrap_small(y0 - RH + e, p.dy);
                tabYdz[e] = tabY[e] * p.dz;
            } else {
                tabZ[e - RY] = wrap_small(z0 - RH + (e - RY), p.dz);
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < RY * RZ; e += NT) {
            const int ly = e / RZ, lz = e - ly * RZ;
            offR[e] = tabYdz[ly] + tabZ[lz];
        }
        for (int e = threadIdx.x; e < AY * AZ; e += NT) {
            const int ly = e / AZ, lz = e - ly * AZ;
            offA[e] = tabYdz[ly + RH - 1] + tabZ[lz + RH - AZH];
        }
        for (int e = threadIdx.x; e < MY * MZ; e += NT) {
            const int my = e / MZ, mz = e - my * MZ;
            const int c = (my + L) * RZ + (mz + L), gz = tabZ[mz + L];
            const int woff = (gz < 3 ? 0 : p.dx * p.dy) + tabY[my + L];
            mtab[e] = make_int2(solid_k(p.wall_mode, gz, p.dz) ? (int)((unsigned)c | 0x80000000u) : c, woff);
        }
        __syncthreads();
    }

    __device__ __forceinline__ void issue_rho(int xlog)
    {
        const float *src = rho + (size_t)((unsigned)wrap_small(xlog, p.dx) * plane);
        float *dst = srho + (xlog & (NR - 1)) * (RY * RZ);
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int e = threadIdx.x + k * NT;
            if ((k + 1) * NT <= RY * RZ || e < RY * RZ) cp_async4(dst + e, src + (unsigned)offR[e]);
        }
    }
    __device__ __forceinline__ void issue_f0(int xlog)
    {
        const float *src = f0c + (size_t)((unsigned)wrap_small(xlog, p.dx) * plane);
        float *dst = sf0 + (xlog & 3) * (AY * AZ);
#pragma unroll
        for (int k = 0; k < KA; ++k) {
            const int e = threadIdx.x + k * NT;
            if ((k + 1) * NT <= AY * AZ || e < AY * AZ) cp_async4(dst + e, src + (unsigned)offA[e]);
        }
    }
    // mu of plane xlog: EOS + Laplacian on fluid nodes, the wall potential on solid ones
    __device__ __forceinline__ void comp_mu(int xlog)
    {
        const int gx = wrap_small(xlog, p.dx);
        float2 *dst = srm + (xlog & 7) * (MY * MZ);
        auto rpl = [&](int xx) -> const float * { return srho + (xx & (NR - 1)) * (RY * RZ); };
        const float *rc = rpl(xlog), *rm1 = rpl(xlog - 1), *rp1 = rpl(xlog + 1);
        const float *rm2 = rpl(xlog - 2), *rp2 = rpl(xlog + 2);
        const float *rm3 = L == 3 ? rpl(xlog - 3) : rc;
        const float *rp3 = L == 3 ? rpl(xlog + 3) : rc;
        const int wx = gx * p.dy;
#pragma unroll
        for (int k = 0; k < KM; ++k) {
            const int e = threadIdx.x + k * NT;
            if (!((k + 1) * NT <= MY * MZ || e < MY * MZ)) break;
            const int2 t = mtab[e];
            const int c = t.x & 0x7fffffff;
            const float r0 = rc[c];
            if (t.x < 0) {
                dst[e] = make_float2(r0, p.wall[t.y + wx]);
                continue;
            }
            float mu;
            if (L == 2) {
                const float n1 = axis_sum<Lane1>(rm1[c], rp1[c], rc[c - RZ], rc[c + RZ], rc[c - 1], rc[c + 1]);
                const float n2 = axis_sum<Lane1>(rm2[c], rp2[c], rc[c - 2 * RZ], rc[c + 2 * RZ], rc[c - 2], rc[c + 2]);
                mu = mu_lap5<Lane1>(eos, p.kk, p.ka, r0, n1, n2);
            } else {
                const float n1 = axis_sum<Lane1>(rm1[c], rp1[c], rc[c - RZ], rc[c + RZ], rc[c - 1], rc[c + 1]);
                const float n2 = axis_sum<Lane1>(rm2[c], rp2[c], rc[c - 2 * RZ], rc[c + 2 * RZ], rc[c - 2], rc[c + 2]);
                const float n3 = axis_sum<Lane1>(rm3[c], rp3[c], rc[c - 3 * RZ], rc[c + 3 * RZ], rc[c - 3], rc[c + 3]);
                mu = mu_lap7<Lane1>(eos, p.kk, p.ka, r0, n1, n2, n3);
            }
            dst[e] = make_float2(r0, mu);
        }
    }
    // mu(x0-3 .. x0+2) evaluated; f0(x0-1 .. x0+1) and rho(x0+3+L) in flight
    __device__ __forceinline__ void prologue(int x0)
    {
        for (int x = x0 - 3 - L; x <= x0 - 3 + L; ++x) issue_rho(x);
        issue_f0(x0 - 1);
        issue_f0(x0);
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
        comp_mu(x0 - 3);
        for (int x = x0 - 2; x <= x0 + 2; ++x) {
            __syncthreads();
            issue_rho(x + L);
            cp_async_commit();
            cp_async_wait_all();
            __syncthreads();
            comp_mu(x);
        }
        __syncthreads();
        issue_rho(x0 + 3 + L);
        issue_f0(x0 + 1);
        cp_async_commit();
    }
    // start of output plane x: rho(x+3+L) and f0(x+1) landed, plane x-1 done
    // by every thread; the next planes' copies go out (unless x is the last)
    __device__ __forceinline__ void begin_plane(int x, bool more)
    {
        cp_async_wait_all();
        __syncthreads();
        if (more) {
            issue_rho(x + 4 + L);
            issue_f0(x + 2);
        }
        cp_async_commit();
    }
    __device__ __forceinline__ const float2 *rm_plane(int x) const { return srm + (x & 7) * (MY * MZ); }
    __device__ __forceinline__ const float *f0_plane(int x) const { return sf0 + (x & 3) * (AY * AZ); }
};

// Warp maximum of the threads' max |MV|^2, one atomicMax per warp (the bits
// of a non-negative float order as unsigned integers).
__device__ __forceinline__ void mvmax_flush(const KParams<float> &p, int P, float mv2)
{
    if (!p.mvmax) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mv2 = fmaxf(mv2, __shfl_xor_sync(0xffffffffu, mv2, o));
    if ((threadIdx.x & 31) == 0) atomicMax(p.mvmax + P * p.mvmax_stride, __float_as_uint(mv2));
}

// One CTA owns a TY x TZ column tile of (y, z) (one node per thread) and
// marches over xl planes of x with the rings of FusedRings.  The next plane's
// rho and f0 are copied in with cp.async while the current plane is computed,
// and the next plane's moving populations are loaded into registers, so
// global-memory latency overlaps the stencil and collision work.  For output
// plane x: mu(x+3) is evaluated (EOS + Laplacian; wall potential on solid
// nodes), then every fluid node of plane x computes
// F = -rho grad7(mu) + grad7(rho)/3, decodes its populations, collides (MRT +
// exact-difference forcing) and streams A-A in place.
template <int TY, int TZ, int L>
using Rings1 = FusedRings<TY, TZ, L, TY * TZ, 1>;

// REF: the rates follow the reference's pattern (collide36's compile-time case).
template <class S, int TY, int TZ, int L, bool REF = false, class SL>
__device__ __forceinline__ void fused_tile(const KParams<float> &p, int P, const SL &slots,
                                           const float *__restrict__ f0c, float *__restrict__ f0n,
                                           const float *__restrict__ rho, const int z0, const int y0,
                                           const int x0, const int xl, float4 *smem4)
{
    using RG = Rings1<TY, TZ, L>;
    constexpr int MZ = RG::MZ, AZ = RG::AZ;
    const int tz = threadIdx.x % TZ, ty = threadIdx.x / TZ;
    const int x1 = min(x0 + xl, p.dx);
    // node indices are 32-bit (the FUSED scheme keeps N below 2^32)
    const unsigned plane = (unsigned)(p.dy * p.dz);
    auto slot = [&](int q, unsigned idx) -> S * { return slots(q, idx); };
    const bool yz_fast = z_interior(p, z0, TZ) && y0 >= 1 && y0 + TY <= p.dy - 1;
    RG R(p, rho, f0c, smem4);
    R.setup(y0, z0);

    const int gy = y0 + ty, gz = z0 + tz;
    const bool active = gy < p.dy && gz < p.dz && !solid_k(p.wall_mode, gz, p.dz);

    // moving populations of one node of plane x into registers (A-A read slots)
    auto fetch = [&](int x, S hv[Q - 1]) {
        if (!active) return;
        const int gx = wrap_small(x, p.dx);
        const unsigned I = (unsigned)gx * plane + (unsigned)(gy * p.dz + gz);
        if (P == 0) {
#pragma unroll
            for (int q = 1; q < Q; ++q) hv[q - 1] = *slot(q - 1, I);
        } else if (yz_fast && gx >= 1 && gx + 1 < p.dx) {
#pragma unroll
            for (int q = 1; q < Q; ++q)
                hv[q - 1] = *slot(opp(q) - 1, I - (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q)));
        } else if (p.wall_mode == 1 && gy >= 1 && gy + 1 < p.dy && gx >= 1 && gx + 1 < p.dx) {
            // no wrap: only the sources across a wall layer (z = 3 or dz - 4) are solid
            const bool lo = gz == 3, hi = gz == p.dz - 4;
#pragma unroll
            for (int q = 1; q < Q; ++q) {
                const bool ss = (cz(q) == 1 && lo) || (cz(q) == -1 && hi);
                hv[q - 1] = *(ss ? slot(q - 1, I)
                                 : slot(opp(q) - 1, I - (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q))));
            }
        } else if (p.wall_mode == 1) {
            // walls at a periodic x or y edge: x and y wrap, z does not
            const bool lo = gz == 3, hi = gz == p.dz - 4;
#pragma unroll
            for (int q = 1; q < Q; ++q) {
                const bool ss = (cz(q) == 1 && lo) || (cz(q) == -1 && hi);
                const int si = wrap1(gx - cx(q), p.dx), sj = wrap1(gy - cy(q), p.dy);
                hv[q - 1] = *(ss ? slot(q - 1, I)
                                 : slot(opp(q) - 1, (unsigned)si * plane + (unsigned)(sj * p.dz + gz - cz(q))));
            }
        } else {
#pragma unroll
            for (int q = 1; q < Q; ++q) {
                const int si = wrap1(gx - cx(q), p.dx), sj = wrap1(gy - cy(q), p.dy), sk = wrap1(gz - cz(q), p.dz);
                if (solid_k(p.wall_mode, sk, p.dz))
                    hv[q - 1] = *slot(q - 1, I);
                else
                    hv[q - 1] = *slot(opp(q) - 1, (unsigned)si * plane + (unsigned)(sj * p.dz + sk));
            }
        }
    };

    S hv[Q - 1];
    R.prologue(x0);
    fetch(x0, hv);

    const int mc = (ty + 3) * MZ + (tz + 3);
    const int ac = (ty + 1) * AZ + (tz + 1);
    float mv2 = 0.f;  // max |MV|^2 of this thread's nodes
    for (int x = x0; x < x1; ++x) {
        R.begin_plane(x, x + 1 < x1);
        S hn[Q - 1];
        if (x + 1 < x1) fetch(x + 1, hn);
        R.comp_mu(x + 3);
        __syncthreads();
        if (active) {
            // force from the (rho, mu) ring
            const float2 *pl[7];
#pragma unroll
            for (int d = -3; d <= 3; ++d) pl[d + 3] = R.rm_plane(x + d);
            float2 lines[9];
#pragma unroll
            for (int l = 0; l < 9; ++l) {
                float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                for (int d = 1; d <= 3; ++d) {
                    const int mo = line_y(l) * d * MZ + line_z(l) * d;
                    acc = line_term(acc, line_c(d), pl[3 + line_x(l) * d][mc + mo], pl[3 - line_x(l) * d][mc - mo]);
                }
                lines[l] = acc;
            }
            const float r = pl[3][mc].x;
            float F[3], gr[3];
            force_from_lines<sizeof(S) == 4>(lines, r, F, gr);  // exact scaling for FP32 storage

            // decode with the sources' rest populations as anchors: g = h + 3 a
            const float *fa[3] = {R.f0_plane(x - 1), R.f0_plane(x), R.f0_plane(x + 1)};
            const float a0 = fa[1][ac];
            float f[Q];
            f[0] = a0;
#pragma unroll
            for (int q = 1; q < Q; ++q) {
                const int sk = gz - cz(q);
                const bool ss = !yz_fast && p.wall_mode == 1 && (sk < 3 || sk > p.dz - 4);
                const float a = ss ? a0 : fa[1 - cx(q)][ac - cy(q) * AZ - cz(q)];
                f[q] = fmaf(3.f, a, s2f<S>(hv[q - 1]));
            }
            float v2;
            if (p.qp) {
                float qp[Q];
                qp36_moments(p.k1, p.k2, gr, qp);
                collide36<Lane1, REF>(f, r, F[0], F[1], F[2], p.ts, p.omts, qp, v2);
            } else {
                collide36<Lane1, REF>(f, r, F[0], F[1], F[2], p.ts, p.omts, nullptr, v2);
            }
            mv2 = fmaxf(mv2, v2);

            // encode against this node's new rest population and stream
            const int gx = wrap_small(x, p.dx);
            const unsigned I = (unsigned)gx * plane + (unsigned)(gy * p.dz + gz);
            const float an = f[0];
            f0n[I] = an;
            if (P == 0) {
#pragma unroll
                for (int q = 1; q < Q; ++q) *slot(opp(q) - 1, I) = f2s<S>(fmaf(-3.f, an, f[q]));
            } else if (yz_fast && gx >= 1 && gx + 1 < p.dx) {
#pragma unroll
                for (int q = 1; q < Q; ++q)
                    *slot(q - 1, I + (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q))) =
                        f2s<S>(fmaf(-3.f, an, f[q]));
            } else if (p.wall_mode == 1 && gy >= 1 && gy + 1 < p.dy && gx >= 1 && gx + 1 < p.dx) {
                const bool lo = gz == 3, hi = gz == p.dz - 4;
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const bool ss = (cz(q) == -1 && lo) || (cz(q) == 1 && hi);
                    *(ss ? slot(opp(q) - 1, I) : slot(q - 1, I + (unsigned)(cx(q) * (int)plane + cy(q) * p.dz + cz(q)))) =
                        f2s<S>(fmaf(-3.f, an, f[q]));
                }
            } else if (p.wall_mode == 1) {
                const bool lo = gz == 3, hi = gz == p.dz - 4;
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const bool ss = (cz(q) == -1 && lo) || (cz(q) == 1 && hi);
                    const int di = wrap1(gx + cx(q), p.dx), dj = wrap1(gy + cy(q), p.dy);
                    *(ss ? slot(opp(q) - 1, I) : slot(q - 1, (unsigned)di * plane + (unsigned)(dj * p.dz + gz + cz(q)))) =
                        f2s<S>(fmaf(-3.f, an, f[q]));
                }
            } else {
#pragma unroll
                for (int q = 1; q < Q; ++q) {
                    const S v = f2s<S>(fmaf(-3.f, an, f[q]));
                    const int di = wrap1(gx + cx(q), p.dx), dj = wrap1(gy + cy(q), p.dy), dk = wrap1(gz + cz(q), p.dz);
                    if (solid_k(p.wall_mode, dk, p.dz))
                        *slot(opp(q) - 1, I) = v;
                    else
                        *slot(q - 1, (unsigned)di * plane + (unsigned)(dj * p.dz + dk)) = v;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < Q - 1; ++q) hv[q] = hn[q];
    }
    cp_async_wait_all();
    mvmax_flush(p, P, mv2);
}

// One box: CTA (bx, by, bz) owns z tile bx, y tile by and x chunk bz.
template <class S, int TY, int TZ, int L>
__global__ void __launch_bounds__(TY *TZ, 768 / (TY * TZ))
    k_fused_collide(KParams<float> p, int P, SlotTable<S> slots, const float *__restrict__ f0c,
                    float *__restrict__ f0n, const float *__restrict__ rho, int xl)
{
    extern __shared__ float4 smem4[];
    fused_tile<S, TY, TZ, L>(p, P, slots, f0c, f0n, rho, blockIdx.x * TZ, blockIdx.y * TY, blockIdx.z * xl, xl,
                             smem4);
}

// Many boxes in one persistent launch: each CTA takes (box, z tile, y tile,
// x chunk) work items from an atomic counter until none are left.  Uneven
// box sizes balance themselves; every box shares the tile shape and march.
// The boxes' parameters are read from global memory (REF: every box's rates
// follow the reference's pattern, so the collision reads two of them).
template <class S, int TY, int TZ, int L, bool REF>
__global__ void __launch_bounds__(TY *TZ, 768 / (TY * TZ))
    k_fused_collide_batch(const KParams<float> *__restrict__ params, const BatchBox *__restrict__ boxes,
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
            while (lo < hi) {  // last box with item0 <= it
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
        // read first after the tile's own barriers
        if (threadIdx.x < Q - 1) slot_s[threadIdx.x] = (S *)bx.h + (size_t)p.n * threadIdx.x;
        const long long local = it - bx.item0;
        const int per_chunk = bx.tiles_z * bx.tiles_y;
        const int chunk = (int)(local / per_chunk), rem = (int)(local % per_chunk);
        const int ytile = rem / bx.tiles_z, ztile = rem % bx.tiles_z;
        fused_tile<S, TY, TZ, L, REF>(p, P, SlotShared<S>{slot_s}, bx.f0[P], bx.f0[1 - P], bx.rho[P],
                                      ztile * TZ, ytile * TY, chunk * xl, xl, smem4);
        __syncthreads();
    }
}

// Batched density pass, one node pair per thread (the pairing of
// k_density): blockIdx.z is the box, blockIdx.y the x plane, blockIdx.x the
// plane's pairs (numbered column by column) in blocks of 128; blocks past a
// box's extent exit at once.
template <class S>
__global__ void __launch_bounds__(BATCH_DENSITY_BLOCK, 8) k_density_batch(const KParams<float> *__restrict__ params,
                                                                        const BatchBox *__restrict__ boxes, int nbox,
                                                                        int P)
{
    // flattened grid: box b owns the blocks from boxes[b].dblk0 on, for each
    // x plane ceil(dy * pairs per column / BATCH_DENSITY_BLOCK) of them; the
    // pairs of a plane are numbered column by column, so a block's threads
    // cover consecutive pairs of one or more columns (no idle lanes on short
    // columns)
    const long long g = blockIdx.x;
    const int b = batch_box_of(boxes, nbox, g, [](const BatchBox &x) { return x.dblk0; });
    const KParams<float> &p = params[b];
    const BatchBox &bx = boxes[b];
    // a block's threads all belong to box b: its 18 slot pointers once per
    // block, in shared memory (computed per thread they crowd the registers)
    __shared__ const S *slot_s[Q - 1];
    if (threadIdx.x < Q - 1) slot_s[threadIdx.x] = (const S *)bx.h + (size_t)p.n * threadIdx.x;
    __syncthreads();
    const int ppc = pairs_per_column(p.dz);
    const int per_plane = (int)(((long long)p.dy * ppc + BATCH_DENSITY_BLOCK - 1) / BATCH_DENSITY_BLOCK);
    const long long local = g - bx.dblk0;
    const int i = (int)(local / per_plane);
    const int e = (int)(local - (long long)i * per_plane) * BATCH_DENSITY_BLOCK + threadIdx.x;
    if (e >= p.dy * ppc) return;
    const int j = e / ppc, t = e - j * ppc;
    density_pair<S>(p, P, (const S *)bx.h, SlotShared<const S>{slot_s}, bx.f0[P], bx.rho[P], i, j,
                    pair_k0(p, i, j, t));
}

template <class S, int TY, int TZ, int L>
constexpr size_t fused_smem_bytes()
{
    return Rings1<TY, TZ, L>::BYTES;
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
