// lane_math.cuh -- FP32 arithmetic of the FUSED collide, written once for one
// node per thread (Lane1, scalar instructions) and for two nodes per thread
// (Lane2, the paired FP32 instructions FADD2 / FMUL2 / FFMA2).  Every function
// performs the same IEEE operations in the same order on each lane, so a pair
// gives exactly the bits of two single-node evaluations; the FUSED translation
// units are compiled without implicit multiply-add contraction so no
// instantiation rounds differently.
//
// Populations in the collision are carried as g_q = f_q / w_q (q >= 1) and the
// rest population f_0 itself.  A stored deviation h = f_q / w_q - a / w_0
// (a = the rest population of the node that wrote it) decodes with one
// multiply-add, g = h + 3 a, and encodes with one, h = g - 3 a.
//
// The MRT collision of the reference (LocalCollideMrt + GlobalCollide,
// FluidCuda.cu:245-347) is evaluated in moment space on m~ = 36 m, m = M f with
// the reference's moment basis (Common.h:104-146): the relaxation
// m* = m - S (m - meq(u)) + (meq(u + F/rho) - meq(u)) (exact-difference forcing,
// M feq(rho, v) = meq(rho, v) for this basis) is diagonal, so a common scale of
// the moments commutes with it, and 36 = lcm(18, 36) turns the weights of the
// axis (1/18) and diagonal (1/36) directions into small integers.  The inverse
// transform M^-1 = M^T diag(1/|row|^2) produces g* = f* / w_q directly.
#pragma once

#include "lbm_core.cuh"

namespace cpmp {

// x / d for the constant divisors of the FUSED arithmetic, as x Ch + RN(x Cl)
// with Ch = RN(1/d) and Cl = RN(1/d - Ch): one multiply and one fused
// multiply-add (the double-word constant multiplication of Brisebarre and
// Muller, "Correctly rounded multiplication by arbitrary precision constants",
// IEEE Trans. Computers 57(2), 2008).  For d = 3, 36 and 360 it gives the
// correctly rounded quotient of every FP32 x with |x| >= 2^-93 (where x Cl
// stays normal): tests/test_scaling_constants.py checks the constants and the
// method with exact integer arithmetic over every eighth mantissa of a binade
// (the rounding does not depend on the binade), and a sweep of every mantissa
// found no difference either.
__device__ __forceinline__ float div3(float x) { return __fmaf_rn(x, 0x1.555556p-2f, __fmul_rn(x, -0x1.555556p-27f)); }
__device__ __forceinline__ float div36(float x) { return __fmaf_rn(x, 0x1.c71c72p-6f, __fmul_rn(x, -0x1.c71c72p-33f)); }
__device__ __forceinline__ float div360(float x)
{
    return __fmaf_rn(x, 0x1.6c16c2p-9f, __fmul_rn(x, -0x1.27d27ep-34f));
}

struct Lane1 {
    using V = float;
    static __device__ __forceinline__ V k(float c) { return c; }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ V max(V a, V b) { return fmaxf(a, b); }
    static __device__ __forceinline__ V gt(V a, float t, V x, V y) { return a > t ? x : y; }
    // approximate reciprocal and base-2 logarithm, and the correctly rounded
    // reciprocal, per lane
    static __device__ __forceinline__ V rcp(V a) { return __fdividef(1.0f, a); }
    static __device__ __forceinline__ V lg2(V a) { return __log2f(a); }
    static __device__ __forceinline__ V rcp_rn(V a) { return __frcp_rn(a); }
    static __device__ __forceinline__ V div36(V a) { return cpmp::div36(a); }
};

struct Lane2 {
    using V = float2;
    static __device__ __forceinline__ V k(float c) { return make_float2(c, c); }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd2_rn(a, b); }
    // a - b as one fused multiply-add: b * (-1) + a rounds once, as a - b does
    static __device__ __forceinline__ V sub(V a, V b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __ffma2_rn(a, b, c); }
    static __device__ __forceinline__ V max(V a, V b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
    static __device__ __forceinline__ V gt(V a, float t, V x, V y)
    {
        return make_float2(a.x > t ? x.x : y.x, a.y > t ? x.y : y.y);
    }
    static __device__ __forceinline__ V rcp(V a) { return make_float2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }
    static __device__ __forceinline__ V lg2(V a) { return make_float2(__log2f(a.x), __log2f(a.y)); }
    static __device__ __forceinline__ V rcp_rn(V a) { return make_float2(__frcp_rn(a.x), __frcp_rn(a.y)); }
    static __device__ __forceinline__ V div36(V a)
    {
        return __ffma2_rn(a, make_float2(0x1.c71c72p-6f, 0x1.c71c72p-6f),
                          __fmul2_rn(a, make_float2(-0x1.c71c72p-33f, -0x1.c71c72p-33f)));
    }
};

// ---------------------------------------------------------------- EOS ----
// Bulk chemical potential mu0(rho) in FP32 with the reference's density soft
// cap (FluidCuda.cu:450-451): the forms of mu0() in lbm_core.cuh with one
// approximate reciprocal per distinct denominator and ln x = log2(x) ln 2 from
// the hardware base-2 logarithm; mu is a sum of O(0.1) terms, so this stays at
// FP32 rounding level.
struct EosLane {
    int eos;
    float A, B, T, TA;  // TA: T ln 2 (VdW, PR, RK) ; c: A/(2 sqrt2 B) (PR), A/B (RK)
    float c, cln2;      // cln2 = c ln 2
};
__device__ __forceinline__ EosLane make_eos_lane(int eos, float A, float B, float T)
{
    const float ln2 = 0.693147180559945309f;
    EosLane e{eos, A, B, T, T * ln2, 0.f, 0.f};
    if (eos == 0) e.c = A / (1.41421356237f * 2.0f * B);
    if (eos == 3) e.c = A / B;
    e.cln2 = e.c * ln2;
    return e;
}

template <class O>
__device__ __forceinline__ typename O::V mu0_lane(const EosLane &e, typename O::V rho)
{
    using V = typename O::V;
    const float R0 = 9.7f, W0 = 1.5f;
    // soft cap above R0: d = R0 + (rho - R0) / (1 + (rho - R0) W0)
    const V ex = O::sub(rho, O::k(R0));
    const V capped = O::fma(ex, O::rcp(O::fma(ex, O::k(W0), O::k(1.f))), O::k(R0));
    const V d = O::gt(rho, R0, capped, rho);
    const V bd = O::mul(O::k(e.B), d);
    const V ir = O::rcp(O::sub(O::k(1.f), bd));
    if (e.eos == 2) {
        // T ln d + T + T (8 bd - 9 bd^2 + 3 bd^3) / (1 - bd)^3 - 2 A d
        const V om3 = O::mul(O::mul(ir, ir), ir);
        const V poly = O::mul(bd, O::fma(bd, O::fma(O::k(3.f), bd, O::k(-9.f)), O::k(8.f)));
        const V t = O::fma(O::k(e.T), O::mul(poly, om3), O::fma(O::k(e.TA), O::lg2(d), O::k(e.T)));
        return O::fma(O::k(-2.f * e.A), d, t);
    }
    // T ln(d / (1 - bd)) + T / (1 - bd)
    const V base = O::fma(O::k(e.TA), O::lg2(O::mul(d, ir)), O::mul(O::k(e.T), ir));
    if (e.eos == 1) return O::fma(O::k(-2.f * e.A), d, base);
    if (e.eos == 3) {
        // - (A/B) ln(1 + bd) - A d / (1 + bd)
        const V op = O::add(O::k(1.f), bd);
        const V t = O::fma(O::k(-e.cln2), O::lg2(op), base);
        return O::fma(O::mul(O::k(-e.A), d), O::rcp(op), t);
    }
    // PR (FluidCuda.cu:453): - A/(2 sqrt2 B) ln((sqrt2 - 1 + bd) / (sqrt2 + 1 - bd))
    //                        - A d / (1 + 2 bd - bd^2)
    const float s2 = 1.41421356237f;
    const V ratio = O::mul(O::add(O::k(s2 - 1.0f), bd), O::rcp(O::sub(O::k(s2 + 1.0f), bd)));
    const V t = O::fma(O::k(-e.cln2), O::lg2(ratio), base);
    const V den = O::fma(bd, O::sub(O::k(2.f), bd), O::k(1.f));
    return O::fma(O::mul(O::k(-e.A), d), O::rcp(den), t);
}

// mu = K^2 mu0(rho) - kappa lap(rho) on a fluid node.  Five-point Laplacian
// (GradD5, Common.h:189-206): n1 / n2 = sums of the six neighbours at distance
// 1 / 2 along the axes, lap = (16 n1 - 90 rho - n2) / 12.  Seven-point
// (GradD7): lap = (270 n1 - 27 n2 + 2 n3 - 1470 rho) / 180.  Each axis sum adds
// the x pair, the y pair and the z pair in that order.
template <class O>
__device__ __forceinline__ typename O::V mu_lap5(const EosLane &e, float kk, float ka, typename O::V r0,
                                                 typename O::V n1, typename O::V n2)
{
    const typename O::V lap =
        O::mul(O::fma(O::k(16.f), n1, O::fma(O::k(-90.f), r0, O::mul(O::k(-1.f), n2))), O::k(1.f / 12.f));
    return O::fma(O::k(kk), mu0_lane<O>(e, r0), O::mul(O::k(-ka), lap));
}
template <class O>
__device__ __forceinline__ typename O::V mu_lap7(const EosLane &e, float kk, float ka, typename O::V r0,
                                                 typename O::V n1, typename O::V n2, typename O::V n3)
{
    const typename O::V lap = O::mul(
        O::fma(O::k(270.f), n1, O::fma(O::k(-27.f), n2, O::fma(O::k(2.f), n3, O::mul(O::k(-1470.f), r0)))),
        O::k(1.f / 180.f));
    return O::fma(O::k(kk), mu0_lane<O>(e, r0), O::mul(O::k(-ka), lap));
}
template <class O>
__device__ __forceinline__ typename O::V axis_sum(typename O::V xm, typename O::V xp, typename O::V ym,
                                                  typename O::V yp, typename O::V zm, typename O::V zp)
{
    return O::add(O::add(O::add(xm, xp), O::add(ym, yp)), O::add(zm, zp));
}

// -------------------------------------------------------------- force ----
// F = -rho grad(mu) + grad(rho) / 3 with the Gradx7 stencil (Common.h:207-246)
// on (rho, mu) pairs.  line[l] holds, for the nine lattice lines in the order
// x, y, z, (1,1,0), (1,-1,0), (1,0,1), (1,0,-1), (0,1,1), (0,1,-1), the sum over
// d = 1..3 of c_d (v(+d) - v(-d)), c = 45, -9, 1, accumulated with line_term;
// the axis lines count twice and the whole stencil is divided by 360.
__device__ __forceinline__ float2 line_term(float2 acc, float c, float2 a, float2 b)
{
    return __ffma2_rn(make_float2(c, c), __fadd2_rn(a, make_float2(-b.x, -b.y)), acc);
}
// EXACT (FP32 storage): the stencil sums are divided by 360 and grad(rho) by
// 3 with correct rounding (div360, div3).  Multiplying by the rounded
// reciprocals instead scales both gradients by 360 fl(1/360) = 1 + 2.4e-8 and
// the ideal term by 3 fl(1/3) = 1 + 3.0e-8 in FP32: a bias of one sign on every
// node, which moves the steady state (with it the FP32 density settled 2.9e-5
// from the FP64 reference on a walled droplet box, without it within 2.3e-6).
// FP16 / BF16 storage round the populations to 4.9e-4 / 3.9e-3 every step and
// keep the single multiplications.
template <bool EXACT = false>
__device__ __forceinline__ void force_from_lines(const float2 l[9], float r, float F[3], float gr[3])
{
    const float2 two = make_float2(2.f, 2.f), z = make_float2(0.f, 0.f);
    auto neg = [](float2 v) { return make_float2(-v.x, -v.y); };
    float2 g0 = __ffma2_rn(two, l[0], z), g1 = __ffma2_rn(two, l[1], z), g2 = __ffma2_rn(two, l[2], z);
    g0 = __fadd2_rn(g0, l[3]);
    g1 = __fadd2_rn(g1, l[3]);
    g0 = __fadd2_rn(g0, l[4]);
    g1 = __fadd2_rn(g1, neg(l[4]));
    g0 = __fadd2_rn(g0, l[5]);
    g2 = __fadd2_rn(g2, l[5]);
    g0 = __fadd2_rn(g0, l[6]);
    g2 = __fadd2_rn(g2, neg(l[6]));
    g1 = __fadd2_rn(g1, l[7]);
    g2 = __fadd2_rn(g2, l[7]);
    g1 = __fadd2_rn(g1, l[8]);
    g2 = __fadd2_rn(g2, neg(l[8]));
    if (EXACT) {
        gr[0] = div360(g0.x);
        gr[1] = div360(g1.x);
        gr[2] = div360(g2.x);
        F[0] = fmaf(-div360(g0.y), r, div3(gr[0]));
        F[1] = fmaf(-div360(g1.y), r, div3(gr[1]));
        F[2] = fmaf(-div360(g2.y), r, div3(gr[2]));
        return;
    }
    const float inv360 = 1.0f / 360.0f;
    gr[0] = g0.x * inv360;
    gr[1] = g1.x * inv360;
    gr[2] = g2.x * inv360;
    F[0] = fmaf(-(g0.y * inv360), r, gr[0] * (1.0f / 3.0f));
    F[1] = fmaf(-(g1.y * inv360), r, gr[1] * (1.0f / 3.0f));
    F[2] = fmaf(-(g2.y * inv360), r, gr[2] * (1.0f / 3.0f));
}
// lattice direction of line l
__host__ __device__ __forceinline__ constexpr int line_x(int l) { return (l == 0 || (l >= 3 && l <= 6)) ? 1 : 0; }
__host__ __device__ __forceinline__ constexpr int line_y(int l)
{
    return l == 1 ? 1 : (l == 3 || l == 7 || l == 8) ? 1 : (l == 4 ? -1 : 0);
}
__host__ __device__ __forceinline__ constexpr int line_z(int l)
{
    return l == 2 ? 1 : (l == 5 || l == 7) ? 1 : ((l == 6 || l == 8) ? -1 : 0);
}
__host__ __device__ __forceinline__ constexpr float line_c(int d) { return d == 1 ? 45.f : (d == 2 ? -9.f : 1.f); }

// ---------------------------------------------------------- moments ----
// m~ = 36 M f from g (g[0] = f_0, g[q] = f_q / w_q).
template <class O>
__device__ __forceinline__ void moments36(const typename O::V g[Q], typename O::V m[Q])
{
    using V = typename O::V;
    const V A1 = O::add(g[1], g[2]), A2 = O::add(g[3], g[4]), A3 = O::add(g[5], g[6]);
    const V D1 = O::sub(g[1], g[2]), D2 = O::sub(g[3], g[4]), D3 = O::sub(g[5], g[6]);
    // xy plane: 7(+,+) 8(-,+) 9(+,-) 10(-,-)
    const V p710 = O::add(g[7], g[10]), m710 = O::sub(g[7], g[10]);
    const V p89 = O::add(g[8], g[9]), m89 = O::sub(g[8], g[9]);
    const V SXY = O::add(p710, p89), KXY = O::sub(p710, p89), XXY = O::sub(m710, m89), YXY = O::add(m710, m89);
    // xz plane: 11(+,+) 12(-,+) 13(+,-) 14(-,-)
    const V p1114 = O::add(g[11], g[14]), m1114 = O::sub(g[11], g[14]);
    const V p1213 = O::add(g[12], g[13]), m1213 = O::sub(g[12], g[13]);
    const V SXZ = O::add(p1114, p1213), KXZ = O::sub(p1114, p1213), XXZ = O::sub(m1114, m1213),
            ZXZ = O::add(m1114, m1213);
    // yz plane: 15(+,+) 16(-,+) 17(+,-) 18(-,-)
    const V p1518 = O::add(g[15], g[18]), m1518 = O::sub(g[15], g[18]);
    const V p1617 = O::add(g[16], g[17]), m1617 = O::sub(g[16], g[17]);
    const V SYZ = O::add(p1518, p1617), KYZ = O::sub(p1518, p1617), YYZ = O::sub(m1518, m1617),
            ZYZ = O::add(m1518, m1617);
    const V ES = O::add(O::add(A1, A2), A3), DS = O::add(O::add(SXY, SXZ), SYZ);
    m[0] = O::fma(O::k(36.f), g[0], O::fma(O::k(2.f), ES, DS));
    m[1] = O::fma(O::k(-1080.f), g[0], O::fma(O::k(-22.f), ES, O::mul(O::k(8.f), DS)));
    m[2] = O::fma(O::k(432.f), g[0], O::fma(O::k(-8.f), ES, DS));
    const V SX = O::add(XXY, XXZ), SY = O::add(YXY, YYZ), SZ = O::add(ZXZ, ZYZ);
    m[3] = O::fma(O::k(2.f), D1, SX);
    m[4] = O::fma(O::k(-8.f), D1, SX);
    m[5] = O::fma(O::k(2.f), D2, SY);
    m[6] = O::fma(O::k(-8.f), D2, SY);
    m[7] = O::fma(O::k(2.f), D3, SZ);
    m[8] = O::fma(O::k(-8.f), D3, SZ);
    const V T9 = O::fma(O::k(-2.f), SYZ, O::add(SXY, SXZ));
    const V A23 = O::add(A2, A3);
    m[9] = O::fma(O::k(4.f), A1, O::fma(O::k(-2.f), A23, T9));
    m[10] = O::fma(O::k(-8.f), A1, O::fma(O::k(4.f), A23, T9));
    const V D23 = O::sub(A2, A3), S23 = O::sub(SXY, SXZ);
    m[11] = O::fma(O::k(2.f), D23, S23);
    m[12] = O::fma(O::k(-4.f), D23, S23);
    m[13] = KXY;
    m[14] = KYZ;
    m[15] = KXZ;
    m[16] = O::sub(XXY, XXZ);
    m[17] = O::sub(YYZ, YXY);
    m[18] = O::sub(ZXZ, ZYZ);
}

// Mass of a node's populations in the scaled form: sum_q f_q = f_0 + (2 ES +
// DS) / 36 with ES the sum of g over the six axis directions and DS over the
// twelve diagonal ones.  Both the collision (the rest population as the
// remainder of the new mass) and the density pass use these sums and a
// correctly rounded division by 36, so no rounded weight enters the mass
// balance: the lattice mass then changes only by unbiased roundings.
template <class O>
__device__ __forceinline__ void mass_sums(const typename O::V g[Q], typename O::V &ES, typename O::V &DS)
{
    ES = O::add(O::add(O::add(g[1], g[2]), O::add(g[3], g[4])), O::add(g[5], g[6]));
    DS = O::add(O::add(O::add(O::add(g[7], g[8]), O::add(g[9], g[10])),
                       O::add(O::add(g[11], g[12]), O::add(g[13], g[14]))),
                O::add(O::add(g[15], g[16]), O::add(g[17], g[18])));
}

// 36 meq(rho, u) given r36 = 36 rho (moments 16..18 vanish)
template <class O>
__device__ __forceinline__ void meq36(typename O::V r36, typename O::V ux, typename O::V uy, typename O::V uz,
                                      typename O::V me[16])
{
    using V = typename O::V;
    const V uxx = O::mul(ux, ux), uyy = O::mul(uy, uy), uzz = O::mul(uz, uz);
    const V u2 = O::add(O::add(uxx, uyy), uzz);
    const V jx = O::mul(r36, ux), jy = O::mul(r36, uy), jz = O::mul(r36, uz);
    me[0] = r36;
    me[1] = O::mul(r36, O::fma(O::k(19.f), u2, O::k(-11.f)));
    me[2] = O::mul(r36, O::fma(O::k(-5.5f), u2, O::k(3.f)));
    me[3] = jx;
    me[4] = O::mul(jx, O::k(-2.f / 3.f));
    me[5] = jy;
    me[6] = O::mul(jy, O::k(-2.f / 3.f));
    me[7] = jz;
    me[8] = O::mul(jz, O::k(-2.f / 3.f));
    const V pxx = O::mul(r36, O::sub(O::mul(O::k(2.f), uxx), O::add(uyy, uzz)));
    const V pww = O::mul(r36, O::sub(uyy, uzz));
    me[9] = pxx;
    me[10] = O::mul(pxx, O::k(-0.5f));
    me[11] = pww;
    me[12] = O::mul(pww, O::k(-0.5f));
    me[13] = O::mul(jx, uy);
    me[14] = O::mul(jy, uz);
    me[15] = O::mul(jx, uz);
}

// g* = f* / w_q (q >= 1) and g*[0] = f*_0 from m~* = 36 m*:
// f* = M^T diag(1 / |row|^2) m*, with the row norms 19, 2394, 252, 10, 40, 10,
// 40, 10, 40, 36, 72, 12, 24, 4, 4, 4, 8, 8, 8 of the reference's basis.
template <class O>
__device__ __forceinline__ void inverse36(const typename O::V m[Q], typename O::V g[Q])
{
    using V = typename O::V;
    g[0] = O::fma(O::k(1.f / 684.f), m[0], O::fma(O::k(-5.f / 14364.f), m[1], O::mul(O::k(1.f / 756.f), m[2])));
    const V BE = O::fma(O::k(1.f / 38.f), m[0], O::fma(O::k(-11.f / 4788.f), m[1], O::mul(O::k(-1.f / 126.f), m[2])));
    const V BD = O::fma(O::k(1.f / 19.f), m[0], O::fma(O::k(8.f / 2394.f), m[1], O::mul(O::k(1.f / 252.f), m[2])));
    const V JX = O::mul(O::sub(m[3], m[4]), O::k(0.05f)), JY = O::mul(O::sub(m[5], m[6]), O::k(0.05f)),
            JZ = O::mul(O::sub(m[7], m[8]), O::k(0.05f));
    const V GX = O::fma(m[3], O::k(0.1f), O::mul(m[4], O::k(0.025f)));
    const V GY = O::fma(m[5], O::k(0.1f), O::mul(m[6], O::k(0.025f)));
    const V GZ = O::fma(m[7], O::k(0.1f), O::mul(m[8], O::k(0.025f)));
    const V PXA = O::mul(O::sub(m[9], m[10]), O::k(1.f / 36.f));
    const V PYZ = O::mul(PXA, O::k(-0.5f));
    const V QW = O::mul(O::sub(m[11], m[12]), O::k(1.f / 24.f));
    const V S910 = O::fma(m[9], O::k(1.f / 36.f), O::mul(m[10], O::k(1.f / 72.f)));
    const V S1112 = O::fma(m[11], O::k(1.f / 12.f), O::mul(m[12], O::k(1.f / 24.f)));
    const V N13 = O::mul(m[13], O::k(0.25f)), N14 = O::mul(m[14], O::k(0.25f)), N15 = O::mul(m[15], O::k(0.25f));
    const V N16 = O::mul(m[16], O::k(0.125f)), N17 = O::mul(m[17], O::k(0.125f)), N18 = O::mul(m[18], O::k(0.125f));
    // axis directions
    const V t12 = O::add(BE, PXA);
    g[1] = O::add(t12, JX);
    g[2] = O::sub(t12, JX);
    const V u = O::add(BE, PYZ);
    const V t34 = O::add(u, QW), t56 = O::sub(u, QW);
    g[3] = O::add(t34, JY);
    g[4] = O::sub(t34, JY);
    g[5] = O::add(t56, JZ);
    g[6] = O::sub(t56, JZ);
    // diagonal directions, plane by plane
    const V BS = O::add(BD, S910);
    const V PXY = O::add(BS, S1112), PXZ = O::sub(BS, S1112), PYZD = O::fma(O::k(-2.f), S910, BD);
    {   // xy: 7 = PXY + GX + GY + N13 + N16 - N17, 8, 9, 10 by the signs of (x, y)
        const V Pp = O::add(PXY, N13), Pm = O::sub(PXY, N13);
        const V a = O::add(GX, N16), b = O::sub(GY, N17);
        const V s = O::add(a, b), d = O::sub(a, b);
        g[7] = O::add(Pp, s);
        g[10] = O::sub(Pp, s);
        g[8] = O::sub(Pm, d);
        g[9] = O::add(Pm, d);
    }
    {   // xz: 11 = PXZ + GX + GZ + N15 - N16 + N18, 12, 13, 14
        const V Pp = O::add(PXZ, N15), Pm = O::sub(PXZ, N15);
        const V a = O::sub(GX, N16), b = O::add(GZ, N18);
        const V s = O::add(a, b), d = O::sub(a, b);
        g[11] = O::add(Pp, s);
        g[14] = O::sub(Pp, s);
        g[12] = O::sub(Pm, d);
        g[13] = O::add(Pm, d);
    }
    {   // yz: 15 = PYZD + GY + GZ + N14 + N17 - N18, 16, 17, 18
        const V Pp = O::add(PYZD, N14), Pm = O::sub(PYZD, N14);
        const V a = O::add(GY, N17), b = O::sub(GZ, N18);
        const V s = O::add(a, b), d = O::sub(a, b);
        g[15] = O::add(Pp, s);
        g[18] = O::sub(Pp, s);
        g[16] = O::sub(Pm, d);
        g[17] = O::add(Pm, d);
    }
}

// The collision of one (Lane1) or two (Lane2) fluid nodes: in g = decoded
// post-stream populations, rho from the density field, F the non-ideal force,
// qp36 = 36 x the K1/K2 pressure-tensor moments (FluidCuda.cu:260-266) or null;
// out g = post-collision populations (same form), mv2 = |u + F / (2 rho)|^2 of
// the colliding state, u = (jx, jy, jz) / rho from the moments of g.
//
// REF: the rates follow the reference's pattern (FluidCuda.cu:154-157, what
// ts_from_tau builds): s = 1 for moments 0, 1, 3, 5, 7, 10, 12, 16, 17, 18, one
// rate for 2, 4, 6, 8 and one for 9, 11, 13, 14, 15.  A unit rate makes the
// relaxed moment its forced equilibrium (1 - s = 0), so those moments need no
// relaxation and 16-18 vanish; the compiler then drops what only they used.
// The results are those of the general form (the zero terms it adds can only
// change the sign of a zero).
template <class O, bool REF = false>
__device__ __forceinline__ void collide36(typename O::V g[Q], typename O::V rho, typename O::V Fx,
                                          typename O::V Fy, typename O::V Fz, const float ts[Q],
                                          const float omts[Q], const typename O::V *qp36, typename O::V &mv2)
{
    using V = typename O::V;
    V m[Q];
    moments36<O>(g, m);
    // 1 / rho and 1 / (36 rho), correctly rounded: u = (36 j) / (36 rho)
    const V r36 = O::mul(O::k(36.f), rho);
    const V ir = O::rcp_rn(rho), ir36 = O::rcp_rn(r36);
    const V ux = O::mul(m[3], ir36), uy = O::mul(m[5], ir36), uz = O::mul(m[7], ir36);
    {   // MV = u + F / (2 rho), the reference's MacroCalculate velocity
        const V hr = O::mul(O::k(0.5f), ir);
        const V vx = O::fma(Fx, hr, ux), vy = O::fma(Fy, hr, uy), vz = O::fma(Fz, hr, uz);
        mv2 = O::fma(vx, vx, O::fma(vy, vy, O::mul(vz, vz)));
    }
    V me[16], me1[16];
    meq36<O>(r36, ux, uy, uz, me);
    meq36<O>(r36, O::fma(Fx, ir, ux), O::fma(Fy, ir, uy), O::fma(Fz, ir, uz), me1);
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        V v;
        if (!REF) {
            v = a >= 16 ? O::mul(O::k(omts[a]), m[a]) : O::fma(O::k(omts[a]), O::sub(m[a], me[a]), me1[a]);
        } else if (a == 2 || a == 4 || a == 6 || a == 8) {
            v = O::fma(O::k(omts[2]), O::sub(m[a], me[a]), me1[a]);
        } else if (a == 9 || a == 11 || a == 13 || a == 14 || a == 15) {
            v = O::fma(O::k(omts[9]), O::sub(m[a], me[a]), me1[a]);
        } else {
            v = a >= 16 ? O::k(0.f) : me1[a];
        }
        if (qp36) v = O::fma(qp36[a], O::k(ts[a]), v);
        m[a] = v;
    }
    inverse36<O>(m, g);
    // rest population: the remainder of the relaxed mass moment 36 rho*, so the
    // node emits exactly (up to the last rounding) the mass it keeps
    V ES, DS;
    mass_sums<O>(g, ES, DS);
    g[0] = O::div36(O::sub(m[0], O::fma(O::k(2.f), ES, DS)));
}

// 36 x the K1/K2 pressure-tensor moments Qp (FluidCuda.cu:260-266) from
// grad(rho) of one node; the other moments are zero.
__device__ __forceinline__ void qp36_moments(float k1, float k2, const float gr[3], float qp[Q])
{
#pragma unroll
    for (int a = 0; a < Q; ++a) qp[a] = 0.f;
    qp[1] = -36.f * 19.f * (k1 + 3.f * k2) * (gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
    qp[9] = -36.f * k1 * (2.f * gr[0] * gr[0] - gr[1] * gr[1] - gr[2] * gr[2]);
    qp[11] = -36.f * k1 * (gr[1] * gr[1] - gr[2] * gr[2]);
    qp[13] = -36.f * k1 * gr[0] * gr[1];
    qp[14] = -36.f * k1 * gr[2] * gr[1];
    qp[15] = -36.f * k1 * gr[0] * gr[2];
}

}  // namespace cpmp
