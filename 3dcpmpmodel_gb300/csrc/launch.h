// launch.h -- launch-side helpers shared by the kernel files and the host
// API: droplet description, per-kernel timing hook, kernel class ids.
#pragma once

#include <cuda_runtime.h>
#include <cmath>
#include <vector>

namespace cpmp {

// Kernel classes reported by cpmp_kernel_times().
enum KernelClass {
    K_WALL = 0,     // wall-layer extrapolation (ChemBoundary)
    K_MU = 1,       // chemical potential (ChemPotential)
    K_FORCE = 2,    // non-ideal force (NonidealForce)
    K_COLLIDE = 3,  // collide + stream (GlobalCollide), PLAIN scheme
    K_MACRO = 4,    // density / velocity moments (MacroCalculate)
    K_FUSED = 5,    // fused mu + force + MRT + forcing + A-A stream
    K_DENSITY = 6,  // FUSED scheme density pass
    K_ADJ_COLLIDE = 7,  // adjoint: collision + streaming (R2)
    K_ADJ_FORCE = 8,    // adjoint: non-ideal force (R3)
    K_ADJ_MU = 9,       // adjoint: chemical potential + kappa partials (R4)
    K_ADJ_WALL = 10,    // adjoint: wall layers + wall gradient (R5)
    K_ADJ_SUM = 11,     // adjoint: loss and kappa reductions
    K_CLASSES = 12
};

inline const char *kernel_class_name(int c)
{
    static const char *names[K_CLASSES] = {"wall",          "chem_potential", "force",       "collide_stream",
                                           "macro",         "fused_collide",  "density",     "adj_collide",
                                           "adj_force",     "adj_mu",         "adj_wall",    "adj_sum"};
    return (c >= 0 && c < K_CLASSES) ? names[c] : "?";
}

// Event-bracketing hook: when non-null, every launch is wrapped in a pair of
// CUDA events on the launching stream.
struct LaunchHook {
    struct Rec {
        int cls;
        cudaEvent_t a, b;
    };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double ms[K_CLASSES] = {0};
    long long launches[K_CLASSES] = {0};
    cudaEvent_t cur_a = nullptr;

    cudaEvent_t get()
    {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    void fold()
    {
        for (auto &r : pending) {
            cudaEventSynchronize(r.b);
            float t = 0;
            cudaEventElapsedTime(&t, r.a, r.b);
            ms[r.cls] += t;
            launches[r.cls] += 1;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        pending.clear();
    }
    void reset()
    {
        fold();
        for (int c = 0; c < K_CLASSES; ++c) {
            ms[c] = 0;
            launches[c] = 0;
        }
    }
    ~LaunchHook()
    {
        for (auto &r : pending) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

inline void hook_begin(LaunchHook *h, int cls, cudaStream_t st)
{
    (void)cls;
    if (!h) return;
    h->cur_a = h->get();
    cudaEventRecord(h->cur_a, st);
}
inline void hook_end(LaunchHook *h, int cls, cudaStream_t st)
{
    if (!h) return;
    cudaEvent_t b = h->get();
    cudaEventRecord(b, st);
    h->pending.push_back({cls, h->cur_a, b});
    if (h->pending.size() > 4096) h->fold();
}

// Node pairs per z column of the density pass (an odd DZ adds a lone node);
// its block: DENSITY_BZ pairs along z x DENSITY_BY rows; the batched density
// pass: BATCH_DENSITY_BLOCK consecutive pairs of an x plane per block; the
// batched wall pass: BATCH_WALL_BLOCK columns per block.
__host__ __device__ inline int pairs_per_column(int dz) { return (dz + 1) / 2; }
constexpr int DENSITY_BZ = 32, DENSITY_BY = 4;
constexpr int BATCH_DENSITY_BLOCK = 128;
constexpr int BATCH_WALL_BLOCK = 128;

// Buffers of one box of a batch (the KParams of every box live in a device
// array next to these).
struct BatchBox {
    void *h;
    float *f0[2];
    float *rho[2];         // rho[0] is the density read at even steps
    long long item0;       // first collide work item of this box
    long long wblk0;       // first block of this box in the flattened wall-pass grid
    long long dblk0;       // first block of this box in the flattened density-pass grid
    int tiles_z, tiles_y;  // column tiles per x plane
};

// Initial droplet (SetFlowField, FluidCuda.cu:199-241).
struct DropletDev {
    double cx, cy, cz, radius, width, den_g, den_l;
    int ref_centre;
};

__host__ __device__ inline double droplet_density(const DropletDev &d, int i, int j, int k, int dx, int dy)
{
    double r;
    if (d.ref_centre) {
        // the reference's centre (DX/2, DY/2, Radius+2) with integer halves,
        // radius through single-precision sqrtf (FluidCuda.cu:215)
        const double ax = (double)i - dx / 2, ay = (double)j - dy / 2, az = (double)k - (d.radius + 2);
        r = (double)sqrtf((float)(ax * ax + ay * ay + az * az));
    } else {
        const double ax = i - d.cx, ay = j - d.cy, az = k - d.cz;
        r = sqrt(ax * ax + ay * ay + az * az);
    }
    return (d.den_l + d.den_g) / 2 - (d.den_l - d.den_g) / 2 * tanh((r - d.radius) * 2 / d.width);
}

}  // namespace cpmp
