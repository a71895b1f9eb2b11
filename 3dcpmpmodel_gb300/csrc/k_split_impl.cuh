// k_split_impl.cuh -- launchers of the two-pass FUSED step (k_split.cuh): the
// force pass (one unit, it reads only the FP32 density) and the collide pass
// for one storage type (one unit per type, so the three compile in parallel).
#pragma once

#include "k_pair_impl.cuh"
#include "k_split.cuh"

namespace cpmp {
namespace split_detail {

template <class S, int P>
void collide_t(const KParams<float> &p, S *h, const float *f0c, float *f0n, const float *rho, const float *F,
               cudaStream_t st)
{
    const dim3 grid((unsigned)((p.dz / 2 + NCZ - 1) / NCZ), (unsigned)((p.dy + NCY - 1) / NCY), (unsigned)p.dx);
    SlotTable<S> slots;
    for (int k = 0; k < Q - 1; ++k) slots.q[k] = h + (size_t)p.n * k;
    if (reference_rates(p))
        k_node_collide<S, P, true><<<grid, dim3(NCZ, NCY), 0, st>>>(p, slots, f0c, f0n, rho, F);
    else
        k_node_collide<S, P, false><<<grid, dim3(NCZ, NCY), 0, st>>>(p, slots, f0c, f0n, rho, F);
}

template <class S>
void collide(const KParams<float> &p, int P, void *h, const float *f0c, float *f0n, const float *rho,
             const float *F, cudaStream_t st)
{
    if (P == 0) collide_t<S, 0>(p, (S *)h, f0c, f0n, rho, F, st);
    else collide_t<S, 1>(p, (S *)h, f0c, f0n, rho, F, st);
}

}  // namespace split_detail
}  // namespace cpmp

// Defines the storage's collide-pass entry point (declared in kernels.h).
#define CPMP_SPLIT_UNIT(SUFFIX, STYPE)                                                                           \
    namespace cpmp {                                                                                             \
    void split_collide_launch_##SUFFIX(const KParams<float> &p, int P, void *h, const float *f0c, float *f0n,   \
                                       const float *rho, const float *F, cudaStream_t st)                        \
    {                                                                                                            \
        split_detail::collide<STYPE>(p, P, h, f0c, f0n, rho, F, st);                                             \
    }                                                                                                            \
    }
