// tec_ref_driver.cpp -- writes Tecplot files through the reference's own
// writer (ordered_tec.cpp), the way SaveTask (FluidCuda.cu:901-927) and
// SaveAllByType (FluidCuda.cu:1032-1092) call it.
// TEST INFRASTRUCTURE ONLY: the byte-level pin of the library's writer.
#include "ordered_tec.h"

using namespace ORDERED_TEC;

extern "C" int ref_tec_savetask(const char *dir, const char *name, int LX, int LY, int LZ, short *mi, short *mj,
                                short *mk, double *dens)
{
    try {
        TEC_FILE tec_file(name, dir);
        tec_file.Title = "Model3D";
        tec_file.Variables.push_back("i");
        tec_file.Variables.push_back("j");
        tec_file.Variables.push_back("k");
        tec_file.Variables.push_back("Density");
        tec_file.Zones.push_back(TEC_ZONE(name));
        tec_file.Zones[0].Max[0] = LZ;
        tec_file.Zones[0].Max[1] = LY;
        tec_file.Zones[0].Max[2] = LX;
        tec_file.Zones[0].Data.push_back(TEC_DATA(mi));
        tec_file.Zones[0].Data.push_back(TEC_DATA(mj));
        tec_file.Zones[0].Data.push_back(TEC_DATA(mk));
        tec_file.Zones[0].Data.push_back(TEC_DATA(dens));
        tec_file.write_plt(false);
    } catch (...) {
        return 1;
    }
    return 0;
}

extern "C" int ref_tec_allbytype(const char *dir, const char *name, int DX, int DY, int DZ, double *ai, double *aj,
                                 double *ak, double *ux, double *uy, double *uz, double *den)
{
    try {
        TEC_FILE tec_file(name, dir);
        tec_file.Title = "Field_3D";
        const char *vars[7] = {"i", "j", "k", "Ux", "Uy", "Uz", "Density"};
        for (const char *v : vars) tec_file.Variables.push_back(v);
        tec_file.Zones.push_back(TEC_ZONE(name));
        tec_file.Zones[0].Max[0] = DX;
        tec_file.Zones[0].Max[1] = DY;
        tec_file.Zones[0].Max[2] = DZ;
        double *d[7] = {ai, aj, ak, ux, uy, uz, den};
        for (double *p : d) tec_file.Zones[0].Data.push_back(TEC_DATA(p));
        tec_file.write_plt(false);
    } catch (...) {
        return 1;
    }
    return 0;
}
