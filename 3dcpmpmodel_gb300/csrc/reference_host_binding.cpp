// reference_host_binding.cpp -- the binding a maintainer of the reference
// would add to its main() step loop (FluidCuda.cu:1277-1292) to run the step
// through this library's C ABI instead of the reference's kernels.  The grid
// and step counts are the reference's compile-time constants, given here as
// macros (-DDX=.. -DDY=.. -DDZ=.. -DAllStep=.. -DShowStep=..).  Not part of
// libcpmp.so; the integration guide shows the same code.
#include <cstdio>
#include "cpmp.h"

int main() {
    cpmp_params p;
    cpmp_params_default(&p);                 // Initialize(): CP-PRW, Tau 0.8, Tr 0.7, K 0.2, Ka 0.001
    p.dx = DX; p.dy = DY; p.dz = DZ;         // Common.h:25-27, now run time
    p.cocurve_dir = "CoCurve";               // SetMultiphase reads CoCurve/CoCurve_<EOS>_2.txt
    p.scheme = CPMP_SCHEME_FUSED;            // or CPMP_SCHEME_PLAIN for the reference's kernel order
    p.storage = CPMP_STORE_F16;
    cpmp_handle *h;
    if (cpmp_create(&p, &h) != CPMP_OK) { fprintf(stderr, "%s\n", cpmp_last_error()); return 1; }

    cpmp_droplet d = {0, 0, 0, /*Radius*/ 60, /*Width*/ 10, /*ref_centre*/ 1};
    cpmp_init_droplet(h, &d);                // SetFlowField<<<>>> (FluidCuda.cu:1262)

    for (double BasePt = -0.08; BasePt <= -0.015; BasePt += 0.005) {   // FluidCuda.cu:1264
        cpmp_set_base_pt(h, BasePt);                                    // cudaMemcpyToSymbol(_BasePt)
        for (int s = 0; s < AllStep / ShowStep; ++s) {
            cpmp_step(h, ShowStep);          // ChemBoundary .. MacroCalculate, ShowStep times
            cpmp_diag g;
            if (cpmp_reduce(h, &g) == CPMP_ERR_NONFINITE) break;        // err_den (FluidCuda.cu:1642-1646)
            printf("%9lld %.12f %.6f %f %f %f %f %f\n", g.step, g.mass, g.max_speed,
                   g.ca_left, g.ca_right, g.ca_cap, g.x_left, g.x_right);   // ShowData columns
        }
    }
    cpmp_destroy(h);                          // CudaFree
}
