// k_fused.cu -- FUSED scheme instantiations and launchers.
#include <algorithm>

#include "k_fused.cuh"
#include "k_plain.cuh"  // k_wall_pass
#include "kernels.h"
#include "cpmp.h"

namespace cpmp {

__global__ void k_init_fused_a(KParams<float> p, DropletDev d, uint8_t *type, float *rho, float *f0)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    const int k = (int)(I % p.dz), j = (int)((I / p.dz) % p.dy), i = (int)(I / p.dz / p.dy);
    if (solid_k(p.wall_mode, k, p.dz)) {
        type[I] = SOLID;
        const float w = p.wall[(k < 3 ? 0 : (long long)p.dx * p.dy) + (long long)i * p.dy + j];
        rho[I] = w;
        f0[I] = w * wgt<float>(0);
    } else {
        type[I] = FLUID;
        const double r0 = droplet_density(d, i, j, k, p.dx, p.dy);
        rho[I] = (float)r0;
        f0[I] = (float)(r0 * wgt<double>(0));
    }
}

template <class S>
__global__ void __launch_bounds__(256) k_decode(KParams<float> p, int P, const S *__restrict__ h,
                                                const float *__restrict__ f0, void *dst, int as_f64)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    const int k = (int)(I % p.dz);
    if (solid_k(p.wall_mode, k, p.dz)) return;
    const int j = (int)((I / p.dz) % p.dy), i = (int)(I / p.dz / p.dy);
    float f[Q];
    gather_pops<S>(p, P, h, f0, i, j, k, I, f);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (as_f64)
            ((double *)dst)[q * p.n + I] = f[q];
        else
            ((float *)dst)[q * p.n + I] = f[q];
    }
}

// Encode natural-order populations: rest populations first (anchors) ...
__global__ void k_encode_a(KParams<float> p, float *f0, const void *src, int as_f64)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    if (solid_k(p.wall_mode, (int)(I % p.dz), p.dz)) return;
    f0[I] = as_f64 ? (float)((const double *)src)[I] : ((const float *)src)[I];
}
// ... then the moving populations into the slots parity P reads them from.
template <class S>
__global__ void k_encode_b(KParams<float> p, int P, S *h, const float *f0, const void *src, int as_f64)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    const int k = (int)(I % p.dz);
    if (solid_k(p.wall_mode, k, p.dz)) return;
    const int j = (int)((I / p.dz) % p.dy), i = (int)(I / p.dz / p.dy);
    for (int q = 1; q < Q; ++q) {
        const float fq = as_f64 ? (float)((const double *)src)[q * p.n + I] : ((const float *)src)[q * p.n + I];
        const int si = wrap1(i - cx(q), p.dx), sj = wrap1(j - cy(q), p.dy), sk = wrap1(k - cz(q), p.dz);
        const bool ss = solid_k(p.wall_mode, sk, p.dz);
        const long long s = ((long long)si * p.dy + sj) * p.dz + sk;
        const float a = ss ? f0[I] : f0[s];
        const S hv = f2s<S>((fq - ratio0(q) * a) * inv_w(q));
        if (P == 0 || ss)
            h[(long long)(q - 1) * p.n + I] = hv;
        else
            h[(long long)(opp(q) - 1) * p.n + s] = hv;
    }
}

template <class S>
__global__ void __launch_bounds__(256) k_velocity(KParams<float> p, int P, const S *__restrict__ h,
                                                  const float *__restrict__ f0, const float *__restrict__ rho,
                                                  float *__restrict__ u)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= p.n) return;
    const int k = (int)(I % p.dz);
    if (solid_k(p.wall_mode, k, p.dz)) return;
    const int j = (int)((I / p.dz) % p.dy), i = (int)(I / p.dz / p.dy);
    float f[Q];
    gather_pops<S>(p, P, h, f0, i, j, k, I, f);
    const float r = rho[I];
    u[I] = (f[1] + f[7] + f[9] + f[11] + f[13] - f[2] - f[8] - f[10] - f[12] - f[14]) / r;
    u[I + p.n] = (f[3] + f[7] + f[8] + f[15] + f[17] - f[4] - f[9] - f[10] - f[16] - f[18]) / r;
    u[I + 2 * p.n] = (f[5] + f[11] + f[12] + f[15] + f[16] - f[6] - f[13] - f[14] - f[17] - f[18]) / r;
}

// The layered wall passes of wall_column (pass 0: layers 0-2 <- E(layer 3);
// pass 1: layer 1 <- E(layer 2); pass 2: layer 0 <- E(layer 1), the same at
// the top wall) in one launch: E at a column reads layer 3 at the column and
// its four xy-diagonal neighbours, so the second layer of a column needs E at
// 5 columns and the third at 13, within a radius-3 diagonal neighbourhood.
// Every value is the expression of wall_extrap on the same inputs, so the
// result is that of the three launches bit for bit.  FUSED scheme: density
// only, mirrored into the other density buffer.  Used by the batches (many
// small boxes: one launch instead of three is faster there).
__device__ __forceinline__ float wall_mix(float c, float mm, float mp, float pm, float pp)
{
    // wall_extrap's sum order: centre x 2, then (-,-), (-,+), (+,-), (+,+)
    return (c * 2.f + mm + mp + pm + pp) / 6.f;
}
__device__ __forceinline__ void wall_column_all(const KParams<float> &p, long long c, float *rho, float *mirror)
{
    const int i = (int)(c / p.dy), j = (int)(c - (c / p.dy) * p.dy);
    const int D = p.dz;
    auto wr = [](int a, int n) { a %= n; return a < 0 ? a + n : a; };
    for (int top = 0; top < 2; ++top) {
        const int k3 = top ? D - 4 : 3, step = top ? 1 : -1;  // layers k3 + step, + 2 step, + 3 step
        auto E = [&](int a, int b) { return wall_extrap<float>(p, rho, wr(i + a, p.dx), wr(j + b, p.dy), k3); };
        const float e00 = E(0, 0);
        float l1 = e00, l0 = e00;
        if (p.complex_bc) {
            const float emm = E(-1, -1), emp = E(-1, 1), epm = E(1, -1), epp = E(1, 1);
            const float e2mm = E(-2, -2), e2m0 = E(-2, 0), e0m2 = E(0, -2), e2mp = E(-2, 2), e0p2 = E(0, 2);
            const float e2pm = E(2, -2), e2p0 = E(2, 0), e2pp = E(2, 2);
            l1 = wall_mix(e00, emm, emp, epm, epp);
            const float lmm = wall_mix(emm, e2mm, e2m0, e0m2, e00);
            const float lmp = wall_mix(emp, e2m0, e2mp, e00, e0p2);
            const float lpm = wall_mix(epm, e0m2, e00, e2pm, e2p0);
            const float lpp = wall_mix(epp, e00, e0p2, e2p0, e2pp);
            l0 = wall_mix(l1, lmm, lmp, lpm, lpp);
        }
        const long long col = ((long long)i * p.dy + j) * D;
        const long long k_e = col + k3 + step, k_1 = col + k3 + 2 * step, k_0 = col + k3 + 3 * step;
        rho[k_e] = e00;
        rho[k_1] = l1;
        rho[k_0] = l0;
        if (mirror) {
            mirror[k_e] = e00;
            mirror[k_1] = l1;
            mirror[k_0] = l0;
        }
    }
}
// All boxes of a batch on one flattened grid (box b owns the blocks from
// boxes[b].wblk0 on, none for a periodic box); the wall of box b at parity P is
// computed on rho[P] and mirrored into rho[1-P].
__global__ void k_wall_pass_batch(const KParams<float> *__restrict__ params, const BatchBox *__restrict__ boxes,
                                  int nbox, int P)
{
    const long long g = blockIdx.x;
    const int bi = batch_box_of(boxes, nbox, g, [](const BatchBox &x) { return x.wblk0; });
    const KParams<float> &p = params[bi];
    if (p.wall_mode != 1) return;
    const BatchBox &b = boxes[bi];
    const long long c = (g - b.wblk0) * blockDim.x + threadIdx.x;
    if (c >= (long long)p.dx * p.dy) return;
    wall_column_all(p, c, b.rho[P], b.rho[1 - P]);
}

// ------------------------------------------------------------- dispatch ----
namespace {
// (ty, tz, nodes per thread, form): form 1 is the two-pass step, whose
// column tile is the force pass's
constexpr int kTiles[][4] = {{4, 32, 1, 0},  {8, 32, 1, 0},  {16, 32, 1, 0}, {16, 16, 1, 0}, {8, 16, 1, 0},
                             {8, 32, 2, 0},  {16, 32, 2, 0}, {8, 64, 2, 0},  {4, 64, 2, 0},  {16, 64, 2, 0},
                             {8, 32, 2, 1},  {16, 32, 2, 1}, {8, 64, 2, 1},  {4, 64, 2, 1},  {16, 64, 2, 1}};
constexpr int kNumTiles = sizeof(kTiles) / sizeof(kTiles[0]);

template <class F>
void with_storage(int storage, F &&f)
{
    if (storage == CPMP_STORE_F16)
        f(__half{});
    else if (storage == CPMP_STORE_BF16)
        f(__nv_bfloat16{});
    else
        f(float{});
}

template <class S, int TY, int TZ, int L>
void launch_collide_t(const KParams<float> &p, int P, const FusedTile &t, S *h, const float *f0c,
                      float *f0n, const float *rho, cudaStream_t st)
{
    const dim3 grid((p.dz + TZ - 1) / TZ, (p.dy + TY - 1) / TY, (p.dx + t.xl - 1) / t.xl);
    SlotTable<S> slots;
    for (int k = 0; k < Q - 1; ++k) slots.q[k] = h + (size_t)p.n * k;
    k_fused_collide<S, TY, TZ, L><<<grid, TY * TZ, fused_smem_bytes<S, TY, TZ, L>(), st>>>(
        p, P, slots, f0c, f0n, rho, t.xl);
}

template <class S, int L>
void launch_collide_l(const KParams<float> &p, int P, const FusedTile &t, S *h, const float *f0c,
                      float *f0n, const float *rho, cudaStream_t st)
{
    if (t.ty == 4 && t.tz == 32) launch_collide_t<S, 4, 32, L>(p, P, t, h, f0c, f0n, rho, st);
    else if (t.ty == 8 && t.tz == 32) launch_collide_t<S, 8, 32, L>(p, P, t, h, f0c, f0n, rho, st);
    else if (t.ty == 16 && t.tz == 32) launch_collide_t<S, 16, 32, L>(p, P, t, h, f0c, f0n, rho, st);
    else if (t.ty == 16 && t.tz == 16) launch_collide_t<S, 16, 16, L>(p, P, t, h, f0c, f0n, rho, st);
    else launch_collide_t<S, 8, 16, L>(p, P, t, h, f0c, f0n, rho, st);
}

bool pair_set_attr(int storage, int lap_order, int ty, int tz, int max_smem)
{
    if (storage == CPMP_STORE_F16) return pair_set_attr_f16(lap_order, ty, tz, max_smem);
    if (storage == CPMP_STORE_BF16) return pair_set_attr_bf16(lap_order, ty, tz, max_smem);
    return pair_set_attr_f32(lap_order, ty, tz, max_smem);
}

// usable[storage index][L - 2][tile index]: the instantiation's shared
// memory fits the device's opt-in limit
bool g_usable[3][2][kNumTiles];
int storage_index(int storage) { return storage == CPMP_STORE_F16 ? 0 : (storage == CPMP_STORE_BF16 ? 1 : 2); }
int tile_index(int ty, int tz, int np = 1, int form = 0)
{
    for (int i = 0; i < kNumTiles; ++i)
        if (kTiles[i][0] == ty && kTiles[i][1] == tz && kTiles[i][2] == np && kTiles[i][3] == form) return i;
    return -1;
}

template <class S, int TY, int TZ, int L>
void set_attr_t(int si, int max_smem)
{
    const size_t b = fused_smem_bytes<S, TY, TZ, L>();
    bool ok = (int)b <= max_smem;
    if (ok)
        ok = cudaFuncSetAttribute(k_fused_collide<S, TY, TZ, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)b) == cudaSuccess;
    cudaGetLastError();
    // the batches' collide of the same tile (its own unit per storage)
    if (ok)
        ok = si == 0   ? batch_set_attr_f16(L == 3 ? 7 : 5, TY, TZ, max_smem)
             : si == 1 ? batch_set_attr_bf16(L == 3 ? 7 : 5, TY, TZ, max_smem)
                       : batch_set_attr_f32(L == 3 ? 7 : 5, TY, TZ, max_smem);
    g_usable[si][L - 2][tile_index(TY, TZ)] = ok;
}
template <class S, int L>
void set_attr_l(int si, int max_smem)
{
    set_attr_t<S, 4, 32, L>(si, max_smem);
    set_attr_t<S, 8, 32, L>(si, max_smem);
    set_attr_t<S, 16, 32, L>(si, max_smem);
    set_attr_t<S, 16, 16, L>(si, max_smem);
    set_attr_t<S, 8, 16, L>(si, max_smem);
}
}  // namespace

bool fused_tile_usable(int storage, int lap_order, int ty, int tz, int np, int form)
{
    const int t = tile_index(ty, tz, np, form);
    return t >= 0 && g_usable[storage_index(storage)][lap_order == 7 ? 1 : 0][t];
}

int fused_tile_count() { return kNumTiles; }
FusedTile fused_tile(int idx, int xl)
{
    return FusedTile{kTiles[idx][0], kTiles[idx][1], xl, kTiles[idx][2], kTiles[idx][3]};
}

cudaError_t fused_setup_attributes()
{
    int dev = 0, max_smem = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
    set_attr_l<__half, 2>(0, max_smem);
    set_attr_l<__half, 3>(0, max_smem);
    set_attr_l<__nv_bfloat16, 2>(1, max_smem);
    set_attr_l<__nv_bfloat16, 3>(1, max_smem);
    set_attr_l<float, 2>(2, max_smem);
    set_attr_l<float, 3>(2, max_smem);
    const int storages[3] = {CPMP_STORE_F16, CPMP_STORE_BF16, CPMP_STORE_F32};
    for (int i = 0; i < kNumTiles; ++i) {
        if (kTiles[i][2] != 2) continue;
        for (int si = 0; si < 3; ++si)
            for (int l = 0; l < 2; ++l)
                g_usable[si][l][i] = kTiles[i][3] == 1
                                         ? split_force_set_attr(l ? 7 : 5, kTiles[i][0], kTiles[i][1], max_smem)
                                         : pair_set_attr(storages[si], l ? 7 : 5, kTiles[i][0], kTiles[i][1], max_smem);
    }
    return cudaSuccess;
}

void fused_launch_init(int storage, const KParams<float> &p, const DropletDev &d, uint8_t *type,
                       float *rho, float *f0, void *h, cudaStream_t st)
{
    const unsigned g = (unsigned)((p.n + 255) / 256);
    k_init_fused_a<<<g, 256, 0, st>>>(p, d, type, rho, f0);
    with_storage(storage, [&](auto tag) {
        using S = decltype(tag);
        k_init_fused_b<S><<<g, 256, 0, st>>>(p, rho, f0, (S *)h);
    });
}

void fused_launch_wall(const KParams<float> &p, float *rho, float *rho_mirror, cudaStream_t st, LaunchHook *hook)
{
    if (p.wall_mode != 1) return;
    // one launch per layer pass: at 512^3 the single-launch form (k_wall_pass_batch's
    // wall_column_all) is slower, its redundant layer-3 reads cost more than two launches
    const long long np = (long long)p.dx * p.dy;
    const unsigned gw = (unsigned)((np + 127) / 128);
    for (int s = 0; s < (p.complex_bc ? 3 : 1); ++s) {
        hook_begin(hook, K_WALL, st);
        k_wall_pass<float><<<gw, 128, 0, st>>>(p, s, rho, nullptr, rho_mirror);
        hook_end(hook, K_WALL, st);
    }
}

void fused_launch_collide(int storage, const KParams<float> &p, int P, const FusedTile &t, void *h,
                          const float *f0c, float *f0n, const float *rho, float *F, cudaStream_t st,
                          LaunchHook *hook)
{
    if (t.form == 1) {
        hook_begin(hook, K_FORCE, st);
        split_force_launch(p, t, rho, F, storage == CPMP_STORE_F32, st);
        hook_end(hook, K_FORCE, st);
        hook_begin(hook, K_FUSED, st);
        if (storage == CPMP_STORE_F16)
            split_collide_launch_f16(p, P, h, f0c, f0n, rho, F, st);
        else if (storage == CPMP_STORE_BF16)
            split_collide_launch_bf16(p, P, h, f0c, f0n, rho, F, st);
        else
            split_collide_launch_f32(p, P, h, f0c, f0n, rho, F, st);
        hook_end(hook, K_FUSED, st);
        return;
    }
    hook_begin(hook, K_FUSED, st);
    if (t.np == 2 && storage == CPMP_STORE_F16)
        pair_launch_f16(p, P, t, h, f0c, f0n, rho, st);
    else if (t.np == 2 && storage == CPMP_STORE_BF16)
        pair_launch_bf16(p, P, t, h, f0c, f0n, rho, st);
    else if (t.np == 2)
        pair_launch_f32(p, P, t, h, f0c, f0n, rho, st);
    else
        with_storage(storage, [&](auto tag) {
            using S = decltype(tag);
            if (p.lap_order == 7)
                launch_collide_l<S, 3>(p, P, t, (S *)h, f0c, f0n, rho, st);
            else
                launch_collide_l<S, 2>(p, P, t, (S *)h, f0c, f0n, rho, st);
        });
    hook_end(hook, K_FUSED, st);
}

void fused_launch_density(int storage, const KParams<float> &p, int P, const void *h,
                          const float *f0, float *rho, cudaStream_t st, LaunchHook *hook)
{
    const dim3 g((unsigned)((pairs_per_column(p.dz) + DENSITY_BZ - 1) / DENSITY_BZ),
                 (unsigned)((p.dy + DENSITY_BY - 1) / DENSITY_BY), (unsigned)p.dx);
    hook_begin(hook, K_DENSITY, st);
    with_storage(storage, [&](auto tag) {
        using S = decltype(tag);
        SlotTable<const S> slots;
        for (int k = 0; k < Q - 1; ++k) slots.q[k] = (const S *)h + (size_t)p.n * k;
        k_density<S><<<g, dim3(DENSITY_BZ, DENSITY_BY), 0, st>>>(p, P, (const S *)h, slots, f0, rho);
    });
    hook_end(hook, K_DENSITY, st);
}

// ------------------------------------------------------------- batches ----

void fused_batch_step(int storage, int lap_order, int wall_mode, int complex_bc, const FusedTile &t,
                      const KParams<float> *params, const BatchBox *boxes, int nbox, long long total_items,
                      long long wall_blocks, long long density_blocks, int P, unsigned *counter, bool ref_rates,
                      cudaStream_t st, LaunchHook *hook)
{
    if (wall_mode == 1 && wall_blocks > 0) {
        hook_begin(hook, K_WALL, st);
        k_wall_pass_batch<<<(unsigned)wall_blocks, BATCH_WALL_BLOCK, 0, st>>>(params, boxes, nbox, P);
        hook_end(hook, K_WALL, st);
    }
    hook_begin(hook, K_FUSED, st);
    cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
    if (storage == CPMP_STORE_F16)
        batch_collide_launch_f16(lap_order, t, params, boxes, nbox, total_items, P, counter, ref_rates, st);
    else if (storage == CPMP_STORE_BF16)
        batch_collide_launch_bf16(lap_order, t, params, boxes, nbox, total_items, P, counter, ref_rates, st);
    else
        batch_collide_launch_f32(lap_order, t, params, boxes, nbox, total_items, P, counter, ref_rates, st);
    hook_end(hook, K_FUSED, st);
    hook_begin(hook, K_DENSITY, st);
    with_storage(storage, [&](auto tag) {
        using S = decltype(tag);
        k_density_batch<S><<<(unsigned)density_blocks, BATCH_DENSITY_BLOCK, 0, st>>>(params, boxes, nbox, 1 - P);
    });
    hook_end(hook, K_DENSITY, st);
}

void fused_launch_decode(int storage, const KParams<float> &p, int P, const void *h, const float *f0,
                         void *dst, bool dst_is_f64, cudaStream_t st)
{
    const unsigned g = (unsigned)((p.n + 255) / 256);
    with_storage(storage, [&](auto tag) {
        using S = decltype(tag);
        k_decode<S><<<g, 256, 0, st>>>(p, P, (const S *)h, f0, dst, dst_is_f64 ? 1 : 0);
    });
}

void fused_launch_encode(int storage, const KParams<float> &p, int P, void *h, float *f0,
                         const void *src, bool src_is_f64, cudaStream_t st)
{
    const unsigned g = (unsigned)((p.n + 255) / 256);
    k_encode_a<<<g, 256, 0, st>>>(p, f0, src, src_is_f64 ? 1 : 0);
    with_storage(storage, [&](auto tag) {
        using S = decltype(tag);
        k_encode_b<S><<<g, 256, 0, st>>>(p, P, (S *)h, f0, src, src_is_f64 ? 1 : 0);
    });
}

void fused_launch_velocity(int storage, const KParams<float> &p, int P, const void *h,
                           const float *f0, const float *rho, float *u, cudaStream_t st)
{
    const unsigned g = (unsigned)((p.n + 255) / 256);
    with_storage(storage, [&](auto tag) {
        using S = decltype(tag);
        k_velocity<S><<<g, 256, 0, st>>>(p, P, (const S *)h, f0, rho, u);
    });
}

}  // namespace cpmp
