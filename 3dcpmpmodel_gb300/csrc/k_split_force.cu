// k_split_force.cu -- the two-pass FUSED step's force pass (k_split.cuh):
// launchers and shared-memory attributes for every column tile (compiled
// without implicit FMA contraction, as the one-pass kernels).
#include "k_split_impl.cuh"

namespace cpmp {
namespace {

template <int TY, int TZ, int L>
constexpr size_t force_smem() { return ForceRings<TY, TZ, L>::BYTES; }

struct ForceAttr {
    int max_smem;
    template <class S, int TY, int TZ, int L>
    bool operator()()
    {
        const size_t b = force_smem<TY, TZ, L>();
        if ((int)b > max_smem) return false;
        const bool ok = cudaFuncSetAttribute(k_force_pass<TY, TZ, L, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b) == cudaSuccess &&
                        cudaFuncSetAttribute(k_force_pass<TY, TZ, L, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b) == cudaSuccess;
        cudaGetLastError();
        return ok;
    }
};
struct ForceLaunch {
    const KParams<float> *p;
    int xl;
    const float *rho;
    float *F;
    bool exact;
    cudaStream_t st;
    template <class S, int TY, int TZ, int L>
    bool operator()()
    {
        const dim3 grid((p->dz + TZ - 1) / TZ, (p->dy + TY - 1) / TY, (p->dx + xl - 1) / xl);
        if (exact)
            k_force_pass<TY, TZ, L, true><<<grid, TY * TZ / 2, force_smem<TY, TZ, L>(), st>>>(*p, rho, F, xl);
        else
            k_force_pass<TY, TZ, L, false><<<grid, TY * TZ / 2, force_smem<TY, TZ, L>(), st>>>(*p, rho, F, xl);
        return true;
    }
};

}  // namespace

bool split_force_set_attr(int lap_order, int ty, int tz, int max_smem)
{
    ForceAttr f{max_smem};
    return lap_order == 7 ? pair_detail::by_shape<float, 3>(ty, tz, f) : pair_detail::by_shape<float, 2>(ty, tz, f);
}

bool split_force_launch(const KParams<float> &p, const FusedTile &t, const float *rho, float *F, bool exact,
                        cudaStream_t st)
{
    ForceLaunch f{&p, t.xl, rho, F, exact, st};
    return p.lap_order == 7 ? pair_detail::by_shape<float, 3>(t.ty, t.tz, f)
                            : pair_detail::by_shape<float, 2>(t.ty, t.tz, f);
}

}  // namespace cpmp
