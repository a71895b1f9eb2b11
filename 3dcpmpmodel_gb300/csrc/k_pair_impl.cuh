// k_pair_impl.cuh -- launchers of the paired FUSED collide (k_pair.cuh) for
// one storage type; each k_pair_<storage>.cu instantiates them for its type so
// the three compile in parallel.
#pragma once

#include "k_pair.cuh"
#include "kernels.h"

namespace cpmp {
namespace pair_detail {

template <int TY, int TZ, int L>
constexpr size_t smem_bytes() { return PairRings<TY, TZ, L>::BYTES; }

template <class S, int TY, int TZ, int L>
void launch_t(const KParams<float> &p, int P, int xl, S *h, const float *f0c, float *f0n, const float *rho,
              cudaStream_t st)
{
    const dim3 grid((p.dz + TZ - 1) / TZ, (p.dy + TY - 1) / TY, (p.dx + xl - 1) / xl);
    SlotTable<S> slots;
    for (int k = 0; k < Q - 1; ++k) slots.q[k] = h + (size_t)p.n * k;
    constexpr size_t sm = smem_bytes<TY, TZ, L>();
    if (reference_rates(p))
        k_pair_collide<S, TY, TZ, L, true><<<grid, TY * TZ / 2, sm, st>>>(p, P, slots, f0c, f0n, rho, xl);
    else
        k_pair_collide<S, TY, TZ, L, false><<<grid, TY * TZ / 2, sm, st>>>(p, P, slots, f0c, f0n, rho, xl);
}

template <class S, int TY, int TZ, int L>
bool set_attr_t(int max_smem)
{
    const size_t b = smem_bytes<TY, TZ, L>();
    if ((int)b > max_smem) return false;
    const bool ok =
        cudaFuncSetAttribute(k_pair_collide<S, TY, TZ, L, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)b) == cudaSuccess &&
        cudaFuncSetAttribute(k_pair_collide<S, TY, TZ, L, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)b) == cudaSuccess;
    cudaGetLastError();
    return ok;
}

// the paired tile shapes (nodes): 8x32, 16x32, 8x64, 4x64, 16x64
template <class S, int L, class F>
bool by_shape(int ty, int tz, F f)
{
    if (ty == 8 && tz == 32) return f.template operator()<S, 8, 32, L>();
    if (ty == 16 && tz == 32) return f.template operator()<S, 16, 32, L>();
    if (ty == 8 && tz == 64) return f.template operator()<S, 8, 64, L>();
    if (ty == 4 && tz == 64) return f.template operator()<S, 4, 64, L>();
    if (ty == 16 && tz == 64) return f.template operator()<S, 16, 64, L>();
    return false;
}

struct SetAttr {
    int max_smem;
    template <class S, int TY, int TZ, int L>
    bool operator()() { return set_attr_t<S, TY, TZ, L>(max_smem); }
};
struct Launch {
    const KParams<float> *p;
    int P, xl;
    void *h;
    const float *f0c;
    float *f0n;
    const float *rho;
    cudaStream_t st;
    template <class S, int TY, int TZ, int L>
    bool operator()()
    {
        launch_t<S, TY, TZ, L>(*p, P, xl, (S *)h, f0c, f0n, rho, st);
        return true;
    }
};

template <class S>
bool set_attr(int lap_order, int ty, int tz, int max_smem)
{
    SetAttr f{max_smem};
    return lap_order == 7 ? by_shape<S, 3>(ty, tz, f) : by_shape<S, 2>(ty, tz, f);
}
template <class S>
bool launch(const KParams<float> &p, int P, const FusedTile &t, void *h, const float *f0c, float *f0n,
            const float *rho, cudaStream_t st)
{
    Launch f{&p, P, t.xl, h, f0c, f0n, rho, st};
    return p.lap_order == 7 ? by_shape<S, 3>(t.ty, t.tz, f) : by_shape<S, 2>(t.ty, t.tz, f);
}

}  // namespace pair_detail
}  // namespace cpmp

// Defines the storage's entry points (declared in kernels.h).
#define CPMP_PAIR_UNIT(SUFFIX, STYPE)                                                                            \
    namespace cpmp {                                                                                             \
    bool pair_set_attr_##SUFFIX(int lap_order, int ty, int tz, int max_smem)                                     \
    {                                                                                                            \
        return pair_detail::set_attr<STYPE>(lap_order, ty, tz, max_smem);                                       \
    }                                                                                                            \
    bool pair_launch_##SUFFIX(const KParams<float> &p, int P, const FusedTile &t, void *h, const float *f0c,     \
                              float *f0n, const float *rho, cudaStream_t st)                                     \
    {                                                                                                            \
        return pair_detail::launch<STYPE>(p, P, t, h, f0c, f0n, rho, st);                                        \
    }                                                                                                            \
    }
