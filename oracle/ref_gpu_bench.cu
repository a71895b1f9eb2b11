// ref_gpu_bench.cu -- times the reference's own CUDA step on this GPU.
//
// BASELINE MEASUREMENT ONLY (not part of the library).  oracle/build_ref.py
// writes into oracle/_ref/ (git-ignored) from the reference sources:
//   Common_gpu.h     reference Common.h with the grid constants DX, DY, DZ
//                    taken from the macros REF_DX, REF_DY, REF_DZ, so the grid
//                    stays a compile-time constant as in the reference;
//   ref_kernels.inc  reference FluidCuda.cu:115-116 and 188-463 verbatim.
// This file declares the reference's __constant__ parameters under their own
// names (FluidCuda.cu:67, the kernels read them by name), fills them, and
// runs the reference's step loop body (FluidCuda.cu:1277-1292): ChemBoundary
// on a (DX) x (DY) launch, ChemPotential, NonidealForce, GlobalCollide on
// 64-thread blocks (FluidCuda.cu:113), the host pointer swap, MacroCalculate
// and a device synchronize, in FP64 as the reference computes.  Compile-time
// switches as the reference's defaults (FluidCuda.cu:1-7): CONTACTANGLE,
// PTCALCFIVEPOINT, COMPLEXCHEMBOUNDARY.
//
// Usage: ref_gpu_bench STEPS WARMUP K A B T KA DEN_G DEN_L BASEPT RADIUS WIDTH TAU
// Prints one JSON line with the device time per step (CUDA events around the
// STEPS timed iterations) and the fluid mass before and after.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <utility>
#include <vector>

struct DVector {
    double x, y, z;
};

#include "Common_gpu.h"

// the reference indexes populations as f*DXYZ + I in int, and launches
// ChemBoundary with DY threads per block
static_assert((long long)DQ * DXYZ < 2147483647LL, "grid too large for the reference's int indexing");
static_assert(DY <= 1024, "ChemBoundary runs DY threads per block");

__constant__ double _K, _A, _B, _T, _Ka, _Kq, _DenG, _DenL, _Tau, _Ts[DQ], _ReTau, _NowStep, _DropStep, _DimA,
    _Gravity, _Radius, _Width, _BasePt, _BasePt2, _K1, _K2;

#define CONTACTANGLE
#define PTCALCFIVEPOINT
#define COMPLEXCHEMBOUNDARY
#include "ref_kernels.inc"

#define CKR(x)                                                                                   \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) {                                                                 \
            std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            return 1;                                                                            \
        }                                                                                        \
    } while (0)

static double mass_of(const std::vector<char> &type, const std::vector<double> &dens)
{
    double m = 0;
    for (size_t i = 0; i < dens.size(); ++i)
        if (type[i] == FLUID) m += dens[i];
    return m;
}

int main(int argc, char **argv)
{
    if (argc != 14) {
        std::fprintf(stderr, "usage: %s STEPS WARMUP K A B T KA DEN_G DEN_L BASEPT RADIUS WIDTH TAU\n", argv[0]);
        return 2;
    }
    const int steps = std::atoi(argv[1]), warmup = std::atoi(argv[2]);
    double v[11];
    for (int i = 0; i < 11; ++i) v[i] = std::atof(argv[3 + i]);
    const double K = v[0], A = v[1], B = v[2], T = v[3], Ka = v[4], dg = v[5], dl = v[6], bp = v[7], rad = v[8],
                 wid = v[9], tau = v[10];
    // MRT rates of Initialize (FluidCuda.cu:154-157)
    double ts[DQ];
    for (int q = 0; q < DQ; ++q) ts[q] = 1.0;
    ts[2] = ts[4] = ts[6] = ts[8] = 1.1;
    ts[9] = ts[11] = ts[13] = ts[14] = ts[15] = 1.0 / tau;
    const double zero = 0.0, retau = 1.0 / tau;
    CKR(cudaMemcpyToSymbol(_K, &K, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_A, &A, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_B, &B, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_T, &T, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_Ka, &Ka, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_DenG, &dg, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_DenL, &dl, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_BasePt, &bp, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_Radius, &rad, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_Width, &wid, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_Tau, &tau, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_ReTau, &retau, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_K1, &zero, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_K2, &zero, sizeof(double)));
    CKR(cudaMemcpyToSymbol(_Ts, ts, sizeof(ts)));

    const size_t n = (size_t)DXYZ;
    char *Type;
    double *Dens, *Pote, *Dist, *Temp, *Vx, *Vy, *Vz, *MVx, *MVy, *MVz, *Fx, *Fy, *Fz;
    CKR(cudaMalloc(&Type, n));
    double **fields[] = {&Dens, &Pote, &Vx, &Vy, &Vz, &MVx, &MVy, &MVz, &Fx, &Fy, &Fz};
    for (double **f : fields) {
        CKR(cudaMalloc(f, n * sizeof(double)));
        CKR(cudaMemset(*f, 0, n * sizeof(double)));
    }
    CKR(cudaMalloc(&Dist, DQ * n * sizeof(double)));
    CKR(cudaMalloc(&Temp, DQ * n * sizeof(double)));
    CKR(cudaMemset(Dist, 0, DQ * n * sizeof(double)));
    CKR(cudaMemset(Temp, 0, DQ * n * sizeof(double)));

    const dim3 DimBlock((unsigned)((n + 64 - 1) / 64)), DimThread(64);
    const dim3 Block(DX, 1, 1), Thread(DY, 1, 1);
    SetFlowField<<<DimBlock, DimThread>>>(Type, Dens, Pote, Dist, Temp);
    CKR(cudaGetLastError());
    CKR(cudaDeviceSynchronize());
    std::vector<char> htype(n);
    std::vector<double> hd(n);
    CKR(cudaMemcpy(htype.data(), Type, n, cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(hd.data(), Dens, n * sizeof(double), cudaMemcpyDeviceToHost));
    const double m0 = mass_of(htype, hd);

    auto step = [&]() -> cudaError_t {
        ChemBoundary<<<Block, Thread>>>(Type, Dens, Pote);
        ChemPotential<<<DimBlock, DimThread>>>(Type, Dens, Pote);
        NonidealForce<<<DimBlock, DimThread>>>(Type, Dens, Pote, Fx, Fy, Fz);
        GlobalCollide<<<DimBlock, DimThread>>>(Type, Dens, Pote, Dist, Temp, MVx, MVy, MVz, Vx, Vy, Vz, Fx, Fy, Fz);
        std::swap(Dist, Temp);
        MacroCalculate<<<DimBlock, DimThread>>>(Type, Dens, Dist, Vx, Vy, Vz);
        return cudaDeviceSynchronize();
    };
    for (int s = 0; s < warmup; ++s) CKR(step());
    cudaEvent_t e0, e1;
    CKR(cudaEventCreate(&e0));
    CKR(cudaEventCreate(&e1));
    CKR(cudaEventRecord(e0));
    for (int s = 0; s < steps; ++s) CKR(step());
    CKR(cudaEventRecord(e1));
    CKR(cudaEventSynchronize(e1));
    float ms = 0;
    CKR(cudaEventElapsedTime(&ms, e0, e1));
    CKR(cudaMemcpy(hd.data(), Dens, n * sizeof(double), cudaMemcpyDeviceToHost));
    const double m1 = mass_of(htype, hd);
    const double ms_step = ms / steps;
    std::printf("{\"grid\": [%d, %d, %d], \"steps\": %d, \"warmup\": %d, \"ms_per_step\": %.6f, \"mlups\": %.3f, "
                "\"mass_before\": %.12e, \"mass_after\": %.12e}\n",
                DX, DY, DZ, steps, warmup, ms_step, (double)n / (ms_step * 1e3), m0, m1);
    for (double **f : fields) cudaFree(*f);
    cudaFree(Dist);
    cudaFree(Temp);
    cudaFree(Type);
    return 0;
}
