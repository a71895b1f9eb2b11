// k_batch_impl.cuh -- launchers of the batches' persistent one-node collide
// (k_fused_collide_batch, k_fused.cuh) for one storage type; each
// k_batch_<storage>.cu instantiates them for its type so the three compile in
// parallel.
#pragma once

#include <algorithm>

#include "k_fused.cuh"
#include "kernels.h"

namespace cpmp {
namespace batch_detail {

// One CTA per resident slot of every SM (the kernel takes work items from a
// device counter until none are left), at most one per item.
template <class S, int TY, int TZ, int L, bool REF>
void launch_t(const KParams<float> *params, const BatchBox *boxes, int nbox, long long total, int P, int xl,
              unsigned *counter, cudaStream_t st)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_collide_batch<S, TY, TZ, L, REF>, TY * TZ,
                                                  fused_smem_bytes<S, TY, TZ, L>());
    long long grid = (long long)sms * std::max(per_sm, 1);
    if (grid > total) grid = total;
    if (grid < 1) grid = 1;
    k_fused_collide_batch<S, TY, TZ, L, REF><<<(unsigned)grid, TY * TZ, fused_smem_bytes<S, TY, TZ, L>(), st>>>(
        params, boxes, nbox, total, P, xl, counter);
}

template <class S, int TY, int TZ, int L>
bool set_attr_t(int max_smem)
{
    const size_t b = fused_smem_bytes<S, TY, TZ, L>();
    if ((int)b > max_smem) return false;
    const bool ok = cudaFuncSetAttribute(k_fused_collide_batch<S, TY, TZ, L, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b) == cudaSuccess &&
                    cudaFuncSetAttribute(k_fused_collide_batch<S, TY, TZ, L, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b) == cudaSuccess;
    cudaGetLastError();
    return ok;
}

// the one-node tile shapes (nodes): 4x32, 8x32, 16x32, 16x16, 8x16
template <class S, int L, class F>
bool by_shape(int ty, int tz, F f)
{
    if (ty == 4 && tz == 32) return f.template operator()<S, 4, 32, L>();
    if (ty == 8 && tz == 32) return f.template operator()<S, 8, 32, L>();
    if (ty == 16 && tz == 32) return f.template operator()<S, 16, 32, L>();
    if (ty == 16 && tz == 16) return f.template operator()<S, 16, 16, L>();
    if (ty == 8 && tz == 16) return f.template operator()<S, 8, 16, L>();
    return false;
}

struct SetAttr {
    int max_smem;
    template <class S, int TY, int TZ, int L>
    bool operator()() { return set_attr_t<S, TY, TZ, L>(max_smem); }
};
struct Launch {
    const KParams<float> *params;
    const BatchBox *boxes;
    int nbox;
    long long total;
    int P, xl;
    unsigned *counter;
    bool ref;
    cudaStream_t st;
    template <class S, int TY, int TZ, int L>
    bool operator()()
    {
        if (ref)
            launch_t<S, TY, TZ, L, true>(params, boxes, nbox, total, P, xl, counter, st);
        else
            launch_t<S, TY, TZ, L, false>(params, boxes, nbox, total, P, xl, counter, st);
        return true;
    }
};

}  // namespace batch_detail
}  // namespace cpmp

// Defines the storage's entry points (declared in kernels.h).
#define CPMP_BATCH_UNIT(SUFFIX, STYPE)                                                                           \
    namespace cpmp {                                                                                             \
    bool batch_set_attr_##SUFFIX(int lap_order, int ty, int tz, int max_smem)                                    \
    {                                                                                                            \
        batch_detail::SetAttr f{max_smem};                                                                       \
        return lap_order == 7 ? batch_detail::by_shape<STYPE, 3>(ty, tz, f)                                      \
                              : batch_detail::by_shape<STYPE, 2>(ty, tz, f);                                     \
    }                                                                                                            \
    void batch_collide_launch_##SUFFIX(int lap_order, const FusedTile &t, const KParams<float> *params,          \
                                       const BatchBox *boxes, int nbox, long long total, int P,                  \
                                       unsigned *counter, bool ref, cudaStream_t st)                             \
    {                                                                                                            \
        batch_detail::Launch f{params, boxes, nbox, total, P, t.xl, counter, ref, st};                           \
        if (lap_order == 7)                                                                                      \
            batch_detail::by_shape<STYPE, 3>(t.ty, t.tz, f);                                                     \
        else                                                                                                     \
            batch_detail::by_shape<STYPE, 2>(t.ty, t.tz, f);                                                     \
    }                                                                                                            \
    }
