// ref_shim.cpp -- runs the reference's own CUDA kernel bodies on the host.
//
// TEST INFRASTRUCTURE ONLY (the checker, and bench.py's reference arm).
//
// oracle/build_ref.py writes two files into oracle/_ref/ from the reference
// sources:
//   Common_rt.h      reference Common.h with the grid constants DX, DY, DZ,
//                    DXYZ, DXY turned into run-time ints (Common.h:25-34);
//   ref_kernels.inc  reference FluidCuda.cu:188-463 verbatim (Feq,
//                    SetFlowField, LocalCollideMrt, GlobalCollide,
//                    MacroCalculate, ChemBoundary, NonidealForce,
//                    ChemPotential).
// This file supplies what nvcc would: the CUDA qualifiers as no-ops, and
// blockIdx/threadIdx/blockDim as per-thread variables, then launches each
// kernel as a host loop (OpenMP over the 1-D grid) in the reference's step
// order (FluidCuda.cu:1279-1291).
//
// The reference's ChemBoundary reads neighbour columns that other threads of
// the same launch rewrite (FluidCuda.cu:389-400).  Run serially three times
// over all columns, the layered result is reached deterministically: the
// first sweep makes layer 2 final everywhere, the second makes layer 1 final,
// the third makes layer 0 final (each sweep rewrites the earlier layers with
// the same values).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>

#define __global__
#define __device__
#define __constant__
#define __inline__ inline

struct dim3 {
    unsigned x, y, z;
};
static thread_local dim3 blockIdx, threadIdx, blockDim;

struct DVector {
    double x, y, z;
};

#include "Common_rt.h"

// reference FluidCuda.cu:67
double _K, _A, _B, _T, _Ka, _Kq, _DenG, _DenL, _Tau, _Ts[DQ], _ReTau, _NowStep, _DropStep, _DimA,
    _Gravity, _Radius, _Width, _BasePt, _BasePt2, _K1, _K2;

#define CONTACTANGLE
namespace v5c {
#define PTCALCFIVEPOINT
#define COMPLEXCHEMBOUNDARY
#include "ref_kernels.inc"
#undef PTCALCFIVEPOINT
#undef COMPLEXCHEMBOUNDARY
}  // namespace v5c
namespace v5s {
#define PTCALCFIVEPOINT
#include "ref_kernels.inc"
#undef PTCALCFIVEPOINT
}  // namespace v5s
namespace v7c {
#define PTCALCSEVENPOINT 1
#define COMPLEXCHEMBOUNDARY
#include "ref_kernels.inc"
#undef PTCALCSEVENPOINT
#undef COMPLEXCHEMBOUNDARY
}  // namespace v7c

// The reference's host droplet-impact diagnostics (FluidCuda.cu:737-898)
// over the reference's globals of the same names (FluidCuda.cu:52-66); they
// append their sums to text files under data/ of the working directory.
#include <cstdio>
#include <fstream>
#include <iostream>
namespace rh {
using namespace std;
char *Type;
double *Dens, *MVx, *MVy, *MVz;
double DenG, DenL, BasePt, Radius, Diameter, Tau, DropVy, DimTime;
int NowStep;
#include "ref_impact.inc"
}  // namespace rh

namespace {

template <class F>
void launch_1d(F &&kernel)
{
    const long n = (long)DXYZ;
    const long blocks = (n + 63) / 64;
#pragma omp parallel for schedule(static)
    for (long b = 0; b < blocks; ++b) {
        blockDim.x = 64;
        blockIdx.x = (unsigned)b;
        for (unsigned t = 0; t < 64; ++t) {
            threadIdx.x = t;
            kernel();
        }
    }
}

template <class F>
void launch_columns_serial(F &&kernel)
{
    blockDim.x = (unsigned)DY;
    for (int i = 0; i < DX; ++i)
        for (int j = 0; j < DY; ++j) {
            blockIdx.x = (unsigned)i;
            threadIdx.x = (unsigned)j;
            kernel();
        }
}

}  // namespace

extern "C" {

void ref_set_grid(int dx, int dy, int dz)
{
    DX = dx;
    DY = dy;
    DZ = dz;
    DXY = dx * dy;
    DXYZ = dx * dy * dz;
}

void ref_set_params(double K, double A, double B, double T, double Ka, double K1, double K2,
                    double den_g, double den_l, double base_pt, double radius, double width,
                    const double *ts)
{
    _K = K; _A = A; _B = B; _T = T; _Ka = Ka; _K1 = K1; _K2 = K2;
    _DenG = den_g; _DenL = den_l; _BasePt = base_pt; _Radius = radius; _Width = width;
    for (int q = 0; q < DQ; ++q) _Ts[q] = ts[q];
}

// SetFlowField (reference FluidCuda.cu:199-241).
void ref_init(char *type, double *dens, double *pote, double *dist, double *temp)
{
    launch_1d([&] { v5c::SetFlowField(type, dens, pote, dist, temp); });
}

// variant: 0 = five-point Laplacian + complex wall (reference default),
//          1 = five-point + simple wall, 2 = seven-point + complex wall.
// `dist` holds the current populations on entry and on return.
int ref_step(int variant, int nsteps, char *type, double *dens, double *pote, double *dist,
             double *temp, double *vx, double *vy, double *vz, double *fx, double *fy, double *fz,
             double *mvx, double *mvy, double *mvz)
{
    if (variant < 0 || variant > 2) return -1;
    const size_t nq = (size_t)DQ * (size_t)DXYZ;
    for (int s = 0; s < nsteps; ++s) {
        if (variant == 0) {
            for (int r = 0; r < 3; ++r)
                launch_columns_serial([&] { v5c::ChemBoundary(type, dens, pote); });
            launch_1d([&] { v5c::ChemPotential(type, dens, pote); });
            launch_1d([&] { v5c::NonidealForce(type, dens, pote, fx, fy, fz); });
            launch_1d([&] {
                v5c::GlobalCollide(type, dens, pote, dist, temp, mvx, mvy, mvz, vx, vy, vz, fx, fy, fz);
            });
            std::memcpy(dist, temp, nq * sizeof(double));
            launch_1d([&] { v5c::MacroCalculate(type, dens, dist, vx, vy, vz); });
        } else if (variant == 1) {
            launch_columns_serial([&] { v5s::ChemBoundary(type, dens, pote); });
            launch_1d([&] { v5s::ChemPotential(type, dens, pote); });
            launch_1d([&] { v5s::NonidealForce(type, dens, pote, fx, fy, fz); });
            launch_1d([&] {
                v5s::GlobalCollide(type, dens, pote, dist, temp, mvx, mvy, mvz, vx, vy, vz, fx, fy, fz);
            });
            std::memcpy(dist, temp, nq * sizeof(double));
            launch_1d([&] { v5s::MacroCalculate(type, dens, dist, vx, vy, vz); });
        } else {
            for (int r = 0; r < 3; ++r)
                launch_columns_serial([&] { v7c::ChemBoundary(type, dens, pote); });
            launch_1d([&] { v7c::ChemPotential(type, dens, pote); });
            launch_1d([&] { v7c::NonidealForce(type, dens, pote, fx, fy, fz); });
            launch_1d([&] {
                v7c::GlobalCollide(type, dens, pote, dist, temp, mvx, mvy, mvz, vx, vy, vz, fx, fy, fz);
            });
            std::memcpy(dist, temp, nq * sizeof(double));
            launch_1d([&] { v7c::MacroCalculate(type, dens, dist, vx, vy, vz); });
        }
    }
    return 0;
}

// Runs ComputeEnergy and Computetangential_velocity once for step `nowstep`
// (1 writes the files' header lines first, as the reference does).
void ref_impact(char *type, double *dens, double *mvx, double *mvy, double *mvz, double den_g, double den_l,
                double base_pt, int nowstep)
{
    rh::Type = type;
    rh::Dens = dens;
    rh::MVx = mvx;
    rh::MVy = mvy;
    rh::MVz = mvz;
    rh::DenG = den_g;
    rh::DenL = den_l;
    rh::BasePt = base_pt;
    rh::NowStep = nowstep;
    rh::ComputeEnergy();
    rh::Computetangential_velocity();
}

}  // extern "C"
