// kernels.h -- host-side declarations of every kernel launcher.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "launch.h"
#include "lbm_core.cuh"

// Sets the calling thread's cpmp_last_error() message (api.cpp).
extern "C" void cpmp_internal_set_error(const char *msg);

namespace cpmp {

// ---- PLAIN scheme (k_plain_f32.cu, k_plain_f64.cu) ------------------------
template <class R, class S>
void plain_launch_init(const KParams<R> &p, const DropletDev &d, uint8_t *type, R *rho, R *mu, R *u,
                       S *f, cudaStream_t st);
template <class R, class S>
void plain_launch_step(const KParams<R> &p, const uint8_t *type, R *rho, R *mu, R *u, R *F, R *mv,
                       const S *fc, S *fn, cudaStream_t st, LaunchHook *hook);
template <class R, class S>
void plain_launch_macro(const KParams<R> &p, const uint8_t *type, const S *f, R *rho, R *u,
                        cudaStream_t st);
template <class R>
void plain_launch_mu_force(const KParams<R> &p, const uint8_t *type, R *rho, R *mu, R *F,
                           cudaStream_t st, R *gm_out);
template <class R, class S>
void plain_launch_step_split(const KParams<R> &p, const uint8_t *type, R *rho, R *mu, const R *u, R *F, R *mv,
                             const S *fc, S *fn, R *rho_out, R *u_out, R *gm_out, cudaStream_t st,
                             LaunchHook *hook);
extern template void plain_launch_step_split<float, float>(const KParams<float> &, const uint8_t *, float *, float *, const float *, float *, float *, const float *, float *, float *, float *, float *, cudaStream_t, LaunchHook *);
extern template void plain_launch_step_split<double, double>(const KParams<double> &, const uint8_t *, double *, double *, const double *, double *, double *, const double *, double *, double *, double *, double *, cudaStream_t, LaunchHook *);

template <class R>
void plain_launch_wall(const KParams<R> &p, R *rho, cudaStream_t st);
extern template void plain_launch_wall<float>(const KParams<float> &, float *, cudaStream_t);
extern template void plain_launch_wall<double>(const KParams<double> &, double *, cudaStream_t);
extern template void plain_launch_init<float, float>(const KParams<float> &, const DropletDev &, uint8_t *, float *, float *, float *, float *, cudaStream_t);
extern template void plain_launch_step<float, float>(const KParams<float> &, const uint8_t *, float *, float *, float *, float *, float *, const float *, float *, cudaStream_t, LaunchHook *);
extern template void plain_launch_macro<float, float>(const KParams<float> &, const uint8_t *, const float *, float *, float *, cudaStream_t);
extern template void plain_launch_mu_force<float>(const KParams<float> &, const uint8_t *, float *, float *, float *, cudaStream_t, float *);
extern template void plain_launch_init<double, double>(const KParams<double> &, const DropletDev &, uint8_t *, double *, double *, double *, double *, cudaStream_t);
extern template void plain_launch_step<double, double>(const KParams<double> &, const uint8_t *, double *, double *, double *, double *, double *, const double *, double *, cudaStream_t, LaunchHook *);
extern template void plain_launch_macro<double, double>(const KParams<double> &, const uint8_t *, const double *, double *, double *, cudaStream_t);
extern template void plain_launch_mu_force<double>(const KParams<double> &, const uint8_t *, double *, double *, double *, cudaStream_t, double *);

// ---- FUSED scheme (k_fused.cu) --------------------------------------------
// storage: CPMP_STORE_F32 / F16 / BF16
// ty x tz nodes per CTA, an x march of xl planes, np nodes per thread (1, or
// 2 for the paired kernel of k_pair.cuh)
struct FusedTile {
    int ty, tz, xl;
    int np = 1;
    // 0: one pass (mu, force, collision and streaming in one kernel);
    // 1: two passes (k_split.cuh: force pass with this column tile, then the
    //    shared-memory-free collide pass), np = 2
    int form = 0;
};
// Tile shapes instantiated for the fused kernel; the autotuner picks among
// them per grid.
int fused_tile_count();
FusedTile fused_tile(int idx, int xl);
// The (storage, Laplacian, tile) instantiation fits this device's shared memory.
bool fused_tile_usable(int storage, int lap_order, int ty, int tz, int np = 1, int form = 0);
// The rates follow the reference's pattern: 1 except one value for moments
// 2, 4, 6, 8 and one for 9, 11, 13, 14, 15 (FluidCuda.cu:154-157); the
// collide kernels then take their compile-time case (collide36's REF).
inline bool reference_rates(const KParams<float> &p)
{
    for (int a : {0, 1, 3, 5, 7, 10, 12, 16, 17, 18})
        if (p.ts[a] != 1.0f) return false;
    for (int a : {4, 6, 8})
        if (p.ts[a] != p.ts[2] || p.omts[a] != p.omts[2]) return false;
    for (int a : {11, 13, 14, 15})
        if (p.ts[a] != p.ts[9] || p.omts[a] != p.omts[9]) return false;
    return true;
}
// The paired kernel's grid requirement: DZ a multiple of 4.
inline bool pair_grid_ok(int dz) { return dz % 4 == 0; }
// Paired kernel (k_pair_<storage>.cu, one unit per storage type): each
// returns false when (ty, tz) is not one of its shapes.
#define CPMP_PAIR_DECL(SUFFIX)                                                                                   \
    bool pair_set_attr_##SUFFIX(int lap_order, int ty, int tz, int max_smem);                                    \
    bool pair_launch_##SUFFIX(const KParams<float> &p, int P, const FusedTile &t, void *h, const float *f0c,     \
                              float *f0n, const float *rho, cudaStream_t st);
CPMP_PAIR_DECL(f16)
CPMP_PAIR_DECL(bf16)
CPMP_PAIR_DECL(f32)
#undef CPMP_PAIR_DECL
// Two-pass form (k_split_force.cu, k_split_<storage>.cu).  The force pass
// writes F[c * n + I] (c = 0..2; 3..5 grad(rho) with the K1/K2 term) with the
// paired column tile (ty, tz) and march xl; false when (ty, tz) is not one of
// its shapes.
bool split_force_set_attr(int lap_order, int ty, int tz, int max_smem);
// exact: the force scaling for FP32 storage (force_from_lines).
bool split_force_launch(const KParams<float> &p, const FusedTile &t, const float *rho, float *F, bool exact,
                        cudaStream_t st);
#define CPMP_SPLIT_DECL(SUFFIX)                                                                                  \
    void split_collide_launch_##SUFFIX(const KParams<float> &p, int P, void *h, const float *f0c, float *f0n,   \
                                       const float *rho, const float *F, cudaStream_t st);
CPMP_SPLIT_DECL(f16)
CPMP_SPLIT_DECL(bf16)
CPMP_SPLIT_DECL(f32)
#undef CPMP_SPLIT_DECL
// The batches' persistent one-node collide (k_batch_<storage>.cu): the
// dynamic shared memory attribute of a tile, and one launch over every box
// (ref: every box's rates follow the reference's pattern).
#define CPMP_BATCH_DECL(SUFFIX)                                                                                  \
    bool batch_set_attr_##SUFFIX(int lap_order, int ty, int tz, int max_smem);                                   \
    void batch_collide_launch_##SUFFIX(int lap_order, const FusedTile &t, const KParams<float> *params,          \
                                       const BatchBox *boxes, int nbox, long long total, int P,                  \
                                       unsigned *counter, bool ref, cudaStream_t st);
CPMP_BATCH_DECL(f16)
CPMP_BATCH_DECL(bf16)
CPMP_BATCH_DECL(f32)
#undef CPMP_BATCH_DECL

cudaError_t fused_setup_attributes();
void fused_launch_init(int storage, const KParams<float> &p, const DropletDev &d, uint8_t *type,
                       float *rho, float *f0, void *h, cudaStream_t st);
// Wall extrapolation on rho; every value written is mirrored into
// rho_mirror when it is non-null (the other density buffer).
void fused_launch_wall(const KParams<float> &p, float *rho, float *rho_mirror, cudaStream_t st, LaunchHook *hook);
// The fused collide reads rho, this step's density (wall layers included).
// F: the two-pass form's force field (3 n floats, 6 n with the K1/K2 term;
// unused by the one-pass form).
void fused_launch_collide(int storage, const KParams<float> &p, int P, const FusedTile &t, void *h,
                          const float *f0c, float *f0n, const float *rho, float *F, cudaStream_t st,
                          LaunchHook *hook);
// Density of the post-stream populations at parity P, every fluid node.
void fused_launch_density(int storage, const KParams<float> &p, int P, const void *h,
                          const float *f0, float *rho, cudaStream_t st, LaunchHook *hook);
// One time step of every box of a batch: batched wall passes, the persistent
// fused collide over all (box, tile, chunk) work items, the batched density
// pass.  params/boxes are device arrays of nbox entries; counter is one
// device unsigned (reset here); wall_blocks / density_blocks are the sizes of
// the flattened wall and density grids (each box's first block in
// BatchBox::wblk0 / dblk0); ref_rates: every box's rates follow the
// reference's pattern (reference_rates).
void fused_batch_step(int storage, int lap_order, int wall_mode, int complex_bc, const FusedTile &t,
                      const KParams<float> *params, const BatchBox *boxes, int nbox, long long total_items,
                      long long wall_blocks, long long density_blocks, int P, unsigned *counter, bool ref_rates,
                      cudaStream_t st, LaunchHook *hook);
// Natural-order populations (post-stream at each node) to/from device
// buffers of FP32 or FP64 (dst_is_f64).
void fused_launch_decode(int storage, const KParams<float> &p, int P, const void *h, const float *f0,
                         void *dst, bool dst_is_f64, cudaStream_t st);
void fused_launch_encode(int storage, const KParams<float> &p, int P, void *h, float *f0,
                         const void *src, bool src_is_f64, cudaStream_t st);
// Bare velocity of the current state.
void fused_launch_velocity(int storage, const KParams<float> &p, int P, const void *h,
                           const float *f0, const float *rho, float *u, cudaStream_t st);

// ---- adjoint (k_adjoint_f32.cu, k_adjoint_f64.cu) ---------------------------
// Four reals loaded or stored as one vector.
template <class R>
struct alignas(4 * sizeof(R)) Pack4 {
    R x, y, z, w;
};
template <class R>
struct alignas(2 * sizeof(R)) Pack2 {
    R x, y;
};
// CTAs of the adjoint's tiled force and chemical-potential launches (the
// length of AdjBufs::ka_acc).
long long adj_tiled_blocks(int dx, int dy, int dz);
template <class R>
struct AdjBufs {
    // dJ/df^n_q(x) = lamp_q(x) + lamrho(x) on fluid nodes, 0 on solid ones;
    // the *_next pair holds step n+1 while step n is being formed
    R *lamp, *lamp_next, *lamrho, *lamrho_next, *lammu;
    Pack2<R> *lmr;  // (lammu on fluid nodes, 0 on solid ones; rho) per node
    R *lamF;  // 4N: (dJ/dF_x, dJ/dF_y, dJ/dF_z, rho) per node
    double *ka_part;  // per-block partials of one reduction
    double *ka_acc;   // per-block dJ/dka sums over all reverse steps
    double *gka, *gwall, *loss;
};
template <class R>
void adj_launch_loss(const KParams<R> &p, const uint8_t *type, const R *rho, const double *target, AdjBufs<R> &b,
                     cudaStream_t st);
template <class R>
void adj_launch_finish(const KParams<R> &p, AdjBufs<R> &b, cudaStream_t st);
extern template void adj_launch_finish<float>(const KParams<float> &, AdjBufs<float> &, cudaStream_t);
extern template void adj_launch_finish<double>(const KParams<double> &, AdjBufs<double> &, cudaStream_t);
template <class R>
void adj_launch_step(const KParams<R> &p, const uint8_t *type, const R *rho, const R *u, const R *gm, const R *F,
                     AdjBufs<R> &b, cudaStream_t st, LaunchHook *hook);
extern template void adj_launch_loss<float>(const KParams<float> &, const uint8_t *, const float *, const double *, AdjBufs<float> &, cudaStream_t);
extern template void adj_launch_step<float>(const KParams<float> &, const uint8_t *, const float *, const float *, const float *, const float *, AdjBufs<float> &, cudaStream_t, LaunchHook *);
extern template void adj_launch_loss<double>(const KParams<double> &, const uint8_t *, const double *, const double *, AdjBufs<double> &, cudaStream_t);
extern template void adj_launch_step<double>(const KParams<double> &, const uint8_t *, const double *, const double *, const double *, const double *, AdjBufs<double> &, cudaStream_t, LaunchHook *);

// ---- diagnostics (k_diag.cu) ----------------------------------------------
// Results of one box's diagnostics, kDiagStride doubles: [0] sum rho over the
// fluid nodes, [1] max |MV|^2, [2] non-finite flag, [4..10] the contact angle
// (CaLeft, CaRight, CaCap, XLeft, XRight, H, L), [12..14] the Laplace probe
// (R, dp, sigma).
constexpr int kDiagStride = 16;
// One box of a batched diagnostics pass (FUSED boxes: FP32 density, no MV).
struct DiagBox {
    const uint8_t *type;
    const float *rho[2];  // the density after an even / odd number of steps
    double *part;         // the box's 3 * nb mass partials
    long long n, blk0;    // nodes; the box's first block in the flattened mass grid
    int nb, vec;          // diag_partial_blocks(n); diag_mass_vec_flags of type and both rho
    int dx, dy, dz, tier, angle, eos;  // angle: dx >= 8 and dz >= 8 (the slice search runs)
    double mid, A, B, T, kk;           // (den_g + den_l) / 2; EOS constants, K^2
};
// The diagnostics of nbox boxes: out[kDiagStride * b + ...] as above (the
// max |MV|^2 slot stays 0); mass_blocks = sum of the boxes' nb; par = the
// step count's parity, which selects rho[par].
void diag_launch_batch(const DiagBox *boxes, int nbox, long long mass_blocks, int par, double *out,
                       cudaStream_t st);
int diag_mass_vec_flags(const void *type, const void *rho, const void *mv, long long n);
// Deterministic FP64 reduction: out[0] = sum rho (fluid), out[1] = max |mv|^2,
// out[2] = non-finite flag.  `partials` holds 3 * diag_partial_blocks(n)
// doubles.
int diag_partial_blocks(long long n);
template <class R>
void diag_launch_mass(const uint8_t *type, const R *rho, const R *mv, long long n, double *partials,
                      double *out, cudaStream_t st);
// Contact angle on the x-z slice j = tier: out[7] = CaLeft, CaRight, CaCap,
// XLeft, XRight, H, L (ContactAngle, FluidCuda.cu:557-734).
template <class R>
void diag_launch_contact_angle(const R *rho, int dx, int dy, int dz, int tier, double den_g,
                               double den_l, double *out, cudaStream_t st);
// Laplace probe along y through (DX/2, ., DZ/2): out[3] = R, dp, sigma.
template <class R>
void diag_launch_laplace(const R *rho, int dx, int dy, int dz, int eos, double A, double B, double T,
                         double kk, double *out, cudaStream_t st);
// mv = u + F / (2 rho) on fluid nodes.
void diag_launch_mv(const uint8_t *type, const float *rho, const float *u, const float *F, float *mv,
                    long long n, cudaStream_t st);

// Droplet-impact sums (ComputeEnergy, Computetangential_velocity,
// SaveSpreadtime): out[13] in the order of cpmp_impact; `partials` holds
// diag_impact_quantities() * diag_partial_blocks(n) doubles.
int diag_impact_quantities();
template <class R>
void diag_launch_impact(const uint8_t *type, const R *rho, const R *mv, int dx, int dy, int dz, double mid,
                        double *partials, double *out, cudaStream_t st);
extern template void diag_launch_impact<float>(const uint8_t *, const float *, const float *, int, int, int, double, double *, double *, cudaStream_t);
extern template void diag_launch_impact<double>(const uint8_t *, const double *, const double *, int, int, int, double, double *, double *, cudaStream_t);
extern template void diag_launch_mass<float>(const uint8_t *, const float *, const float *, long long, double *, double *, cudaStream_t);
extern template void diag_launch_mass<double>(const uint8_t *, const double *, const double *, long long, double *, double *, cudaStream_t);
extern template void diag_launch_contact_angle<float>(const float *, int, int, int, int, double, double, double *, cudaStream_t);
extern template void diag_launch_contact_angle<double>(const double *, int, int, int, int, double, double, double *, cudaStream_t);
extern template void diag_launch_laplace<float>(const float *, int, int, int, int, double, double, double, double, double *, cudaStream_t);
extern template void diag_launch_laplace<double>(const double *, int, int, int, int, double, double, double, double, double *, cudaStream_t);

}  // namespace cpmp
