// tecplot.cpp -- Tecplot binary (#!TDV112) writer for ordered zones.
//
// The on-disk output format of the reference (ordered_tec.cpp:674-717 header,
// :990-1013 zone header, :1015-1147 zone data, used by SaveTask,
// FluidCuda.cu:901-927, and SaveAllByType, FluidCuda.cu:1032-1092).  The
// layout is the published Tecplot binary data format, version 112:
//
//   "#!TDV112", int32 1 (byte order), int32 file type, title, int32 nvar,
//   variable names; per zone: float32 299, name, int32 -1 (parent),
//   int32 strand, float64 solution time, int32 -1, int32 0 (ordered),
//   int32 0 (nodal), int32 0, int32 0, int32 I/J/K max, int32 0 (no aux);
//   float32 357 (end of header); per zone: float32 299, int32 format per
//   variable, int32 0, int32 0, int32 -1, float64 min/max per variable, then
//   each variable's values with I fastest.
// Strings are written as one int32 per character and a terminating 0.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cpmp.h"

namespace {

struct Out {
    FILE *f;
    bool ok = true;
    void i32(int v) { ok = ok && std::fwrite(&v, 4, 1, f) == 1; }
    void f32(float v) { ok = ok && std::fwrite(&v, 4, 1, f) == 1; }
    void f64(double v) { ok = ok && std::fwrite(&v, 8, 1, f) == 1; }
    void str(const char *s)
    {
        // characters are widened as the platform's char (the reference
        // widens a std::string character), then a terminating zero
        for (const char *c = s; *c; ++c) i32((int)*c);
        i32(0);
    }
    void raw(const void *p, size_t bytes) { ok = ok && std::fwrite(p, 1, bytes, f) == bytes; }
};

size_t type_size(int t)
{
    switch (t) {
    case CPMP_TEC_FLOAT: return 4;
    case CPMP_TEC_DOUBLE: return 8;
    case CPMP_TEC_INT32: return 4;
    case CPMP_TEC_INT16: return 2;
    case CPMP_TEC_BYTE: return 1;
    default: return 0;
    }
}

template <class T>
void minmax_of(const void *data, size_t n, double *mn, double *mx)
{
    const T *d = (const T *)data;
    T lo = d[0], hi = d[0];
    for (size_t i = 1; i < n; ++i) {
        if (d[i] < lo) lo = d[i];
        if (d[i] > hi) hi = d[i];
    }
    *mn = (double)lo;
    *mx = (double)hi;
}

void minmax(int t, const void *data, size_t n, double *mn, double *mx)
{
    switch (t) {
    case CPMP_TEC_FLOAT: minmax_of<float>(data, n, mn, mx); break;
    case CPMP_TEC_DOUBLE: minmax_of<double>(data, n, mn, mx); break;
    case CPMP_TEC_INT32: minmax_of<int>(data, n, mn, mx); break;
    case CPMP_TEC_INT16: minmax_of<short>(data, n, mn, mx); break;
    default: minmax_of<signed char>(data, n, mn, mx); break;
    }
}

}  // namespace

extern "C" void cpmp_internal_set_error(const char *msg);

extern "C" cpmp_status cpmp_tecplot_write(const char *path, const char *title, const char *zone_name, int nvar,
                                          const char *const *names, const int *types, const void *const *data,
                                          int imax, int jmax, int kmax)
{
    if (!path || !title || !zone_name || nvar < 1 || !names || !types || !data) {
        cpmp_internal_set_error("cpmp_tecplot_write: null argument or no variables");
        return CPMP_ERR_PARAM;
    }
    if (imax < 1 || jmax < 1 || kmax < 1) {
        cpmp_internal_set_error("cpmp_tecplot_write: I/J/K max must be positive");
        return CPMP_ERR_PARAM;
    }
    for (int v = 0; v < nvar; ++v)
        if (!type_size(types[v]) || !data[v] || !names[v]) {
            cpmp_internal_set_error("cpmp_tecplot_write: bad variable type or null data");
            return CPMP_ERR_PARAM;
        }
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        cpmp_internal_set_error((std::string("cpmp_tecplot_write: cannot open ") + path).c_str());
        return CPMP_ERR_PARAM;
    }
    Out o{f};
    const size_t npts = (size_t)imax * jmax * kmax;
    // header section
    o.raw("#!TDV112", 8);
    o.i32(1);
    o.i32(0);  // full data file
    o.str(title);
    o.i32(nvar);
    for (int v = 0; v < nvar; ++v) o.str(names[v]);
    o.f32(299.0f);
    o.str(zone_name);
    o.i32(-1);    // parent zone
    o.i32(-1);    // strand id
    o.f64(0.0);   // solution time
    o.i32(-1);    // unused
    o.i32(0);     // ordered zone
    o.i32(0);     // values at the nodes
    o.i32(0);     // no face neighbours supplied
    o.i32(0);     // no user face connections
    o.i32(imax);
    o.i32(jmax);
    o.i32(kmax);
    o.i32(0);     // no auxiliary data
    o.f32(357.0f);
    // data section
    o.f32(299.0f);
    for (int v = 0; v < nvar; ++v) o.i32(types[v]);
    o.i32(0);   // no passive variables
    o.i32(0);   // no variable sharing
    o.i32(-1);  // no connectivity sharing
    for (int v = 0; v < nvar; ++v) {
        double mn, mx;
        minmax(types[v], data[v], npts, &mn, &mx);
        o.f64(mn);
        o.f64(mx);
    }
    for (int v = 0; v < nvar; ++v) o.raw(data[v], npts * type_size(types[v]));
    const bool ok = o.ok && std::fclose(f) == 0;
    if (!ok) {
        cpmp_internal_set_error((std::string("cpmp_tecplot_write: write failed: ") + path).c_str());
        return CPMP_ERR_PARAM;
    }
    return CPMP_OK;
}

extern "C" cpmp_status cpmp_write_tecplot(cpmp_handle *h, const char *path, int layout, int decimate, int flags,
                                          double vel_scale)
{
    if (!h || !path) {
        cpmp_internal_set_error("cpmp_write_tecplot: null argument");
        return CPMP_ERR_PARAM;
    }
    double dg, dl, A, B, T, Rc;
    cpmp_status s = cpmp_get_eos(h, &dg, &dl, &A, &B, &T, &Rc);
    if (s != CPMP_OK) return s;
    // grid dimensions from the TYPE field size: read them from the handle
    int dims[3];
    if ((s = cpmp_get_dims(h, dims)) != CPMP_OK) return s;
    const int DX = dims[0], DY = dims[1], DZ = dims[2];
    const size_t N = (size_t)DX * DY * DZ;
    std::vector<double> rho(N);
    if ((s = cpmp_get_field(h, CPMP_FIELD_RHO, CPMP_F64, rho.data(), N * 8)) != CPMP_OK) return s;
    std::string base(path);
    std::string zone = base;
    const size_t slash = zone.find_last_of('/');
    if (slash != std::string::npos) zone = zone.substr(slash + 1);
    if (zone.size() > 4 && zone.compare(zone.size() - 4, 4, ".plt") == 0) zone = zone.substr(0, zone.size() - 4);
    if (layout == CPMP_TEC_SAVETASK) {
        // SaveTask: decimated density with i, j, k of the decimated grid
        const int DR = decimate > 0 ? decimate : 5;
        const int LX = DX / DR, LY = DY / DR, LZ = DZ / DR;
        const int lx = LX > 0 ? LX : 1, ly = LY > 0 ? LY : 1, lz = LZ > 0 ? LZ : 1;
        const size_t L = (size_t)lx * ly * lz;
        std::vector<short> vi(L), vj(L), vk(L);
        std::vector<double> d(L);
        for (int i = 0; i < lx; ++i)
            for (int j = 0; j < ly; ++j)
                for (int k = 0; k < lz; ++k) {
                    const size_t m = ((size_t)i * ly + j) * lz + k;
                    vi[m] = (short)i;
                    vj[m] = (short)j;
                    vk[m] = (short)k;
                    size_t src;
                    if (flags & CPMP_TEC_REFERENCE_STRIDE)
                        // the reference's CompressField strides the flat index
                        // (FluidCuda.cu:470), not each axis
                        src = ((size_t)i * DY * DZ + (size_t)j * DZ + k) * DR;
                    else
                        src = ((size_t)(i * DR) * DY + (size_t)j * DR) * DZ + (size_t)k * DR;
                    d[m] = src < N ? rho[src] : 0.0;
                }
        const char *names[4] = {"i", "j", "k", "Density"};
        const int types[4] = {CPMP_TEC_INT16, CPMP_TEC_INT16, CPMP_TEC_INT16, CPMP_TEC_DOUBLE};
        const void *data[4] = {vi.data(), vj.data(), vk.data(), d.data()};
        return cpmp_tecplot_write(path, "Model3D", zone.c_str(), 4, names, types, data, lz, ly, lx);
    }
    if (layout == CPMP_TEC_ALLBYTYPE) {
        // SaveAllByType: every node, x fastest, velocity * DimV where
        // rho >= midpoint
        std::vector<double> mv(3 * N);
        if ((s = cpmp_get_field(h, CPMP_FIELD_MV, CPMP_F64, mv.data(), 3 * N * 8)) != CPMP_OK) return s;
        std::vector<double> ai(N), aj(N), ak(N), ux(N), uy(N), uz(N), ad(N);
        const double mid = (dg + dl) / 2;
        for (int i = 0; i < DX; ++i)
            for (int j = 0; j < DY; ++j)
                for (int k = 0; k < DZ; ++k) {
                    const size_t p = ((size_t)i * DY + j) * DZ + k;
                    const size_t x = (size_t)i + (size_t)j * DX + (size_t)k * DY * DX;
                    ai[x] = i;
                    aj[x] = j;
                    ak[x] = k;
                    ad[x] = rho[p];
                    const bool liq = rho[p] >= mid;
                    ux[x] = liq ? mv[p] * vel_scale : -2;
                    uy[x] = liq ? mv[p + N] * vel_scale : -2;
                    uz[x] = liq ? mv[p + 2 * N] * vel_scale : -2;
                }
        const char *names[7] = {"i", "j", "k", "Ux", "Uy", "Uz", "Density"};
        const int types[7] = {CPMP_TEC_DOUBLE, CPMP_TEC_DOUBLE, CPMP_TEC_DOUBLE, CPMP_TEC_DOUBLE,
                              CPMP_TEC_DOUBLE, CPMP_TEC_DOUBLE, CPMP_TEC_DOUBLE};
        const void *data[7] = {ai.data(), aj.data(), ak.data(), ux.data(), uy.data(), uz.data(), ad.data()};
        return cpmp_tecplot_write(path, "Field_3D", zone.c_str(), 7, names, types, data, DX, DY, DZ);
    }
    cpmp_internal_set_error("cpmp_write_tecplot: unknown layout");
    return CPMP_ERR_PARAM;
}
