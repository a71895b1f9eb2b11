// eos.cpp -- equation-of-state constants, coexistence densities.
//
// eos_constants() is SetMultiphase's parameter table (FluidCuda.cu:1318-1344);
// read_cocurve() reads a CoCurve_<EOS>_2.txt table the way SetMultiphase does
// (FluidCuda.cu:1355-1384: first row whose T/Tc equals Tr within 1e-12,
// Common.h:157-160); maxwell() solves mu0(g) = mu0(l), p(g) = p(l) by Newton
// iteration from the spinodal bracket, which is what the tables tabulate.
#include "eos.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "cpmp.h"

namespace cpmp {

int eos_of_model(int model)
{
    switch (model) {
    case CPMP_MP_CPVDW: return EOS_VDW;
    case CPMP_MP_CPPRW:
    case CPMP_MP_CPPRM: return EOS_PR;
    case CPMP_MP_CPRKE:
    case CPMP_MP_CPRKS: return EOS_RK;
    case CPMP_MP_CPCSE: return EOS_CS;
    default: return -1;
    }
}

const char *table_tag(int model)
{
    switch (model) {
    case CPMP_MP_CPVDW: return "VDW";
    case CPMP_MP_CPPRW: return "PRW";
    case CPMP_MP_CPPRM: return "PRM";
    case CPMP_MP_CPRKE: return "RKE";
    case CPMP_MP_CPRKS: return "RKS";
    case CPMP_MP_CPCSE: return "CSE";
    default: return nullptr;
    }
}

bool eos_constants(int model, double tr, double a, double b, double omega, double *A, double *B,
                   double *Tc, double *Rc)
{
    switch (model) {
    case CPMP_MP_CPVDW:
        *A = 9.0 / 49; *B = 2.0 / 21; *Tc = 4.0 / 7; *Rc = 7.0 / 2;
        return true;
    case CPMP_MP_CPCSE: {
        // B is b/4; corresponding states: Tc = 0.0943287 a / B, rho_c = 0.13044388 / B
        const double aa = a > 0 ? a : 1.0, bb = b > 0 ? b : 4.0;
        *A = aa; *B = bb / 4;
        *Tc = 0.09432870 * aa / (bb / 4);
        *Rc = 0.13044388 / (bb / 4);
        return true;
    }
    case CPMP_MP_CPRKE:
        *Tc = 0.196133; *Rc = 2.729171; *B = 2.0 / 21;
        *A = 2.0 / 49 * (1.0 / std::sqrt(*Tc * tr));
        return true;
    case CPMP_MP_CPRKS: {
        const double w = omega > 0 ? omega : 0.344;
        const double s = 1.0 + (0.480 + 1.574 * w - 0.176 * w * w) * (1.0 - std::sqrt(tr));
        *A = 2.0 / 49 * s * s; *B = 2.0 / 21; *Tc = 0.086861; *Rc = 2.729171;
        return true;
    }
    case CPMP_MP_CPPRW:
    case CPMP_MP_CPPRM: {
        const double w = omega > 0 ? omega : (model == CPMP_MP_CPPRW ? 0.344 : 0.011);
        const double s = 1.0 + (0.37464 + 1.54226 * w - 0.26992 * w * w) * (1.0 - std::sqrt(tr));
        *A = 2.0 / 49 * s * s; *B = 2.0 / 21; *Tc = 0.072919; *Rc = 2.65730416;
        return true;
    }
    default: return false;
    }
}

double mu0_host(int eos, double A, double B, double T, double r)
{
    const double bd = B * r;
    switch (eos) {
    case EOS_VDW: return T * std::log(r / (1 - bd)) + T / (1 - bd) - 2 * A * r;
    case EOS_CS: {
        const double om = 1 - bd;
        return T * std::log(r) + T + T * (8 * bd - 9 * bd * bd + 3 * bd * bd * bd) / (om * om * om) - 2 * A * r;
    }
    case EOS_RK: return T * std::log(r / (1 - bd)) + T / (1 - bd) - A / B * std::log(1 + bd) - A * r / (1 + bd);
    default: {
        const double s2 = 1.4142135623730950488016887242097;
        return T * std::log(r / (1 - bd)) - A / (s2 * 2 * B) * std::log((s2 - 1 + bd) / (s2 + 1 - bd)) +
               T / (1 - bd) - A * r / (1 + bd * 2 - bd * bd);
    }
    }
}

double pressure_host(int eos, double A, double B, double T, double r)
{
    const double bd = B * r;
    switch (eos) {
    case EOS_VDW: return T * r / (1 - bd) - A * r * r;
    case EOS_CS: {
        const double om = 1 - bd;
        return r * T * (1 + bd + bd * bd - bd * bd * bd) / (om * om * om) - A * r * r;
    }
    case EOS_RK: return T * r / (1 - bd) - A * r * r / (1 + bd);
    default: return T * r / (1 - bd) - A * r * r / (1 + bd * 2 - bd * bd);
    }
}

int maxwell(int eos, double A, double B, double T, double *g_out, double *l_out)
{
    // spinodal bracket: the two zeros of dp/drho on (0, 1/B)
    const double rmax = 0.999 / B;
    const int ns = 400000;
    double sp1 = -1, sp2 = -1;
    double prev = pressure_host(eos, A, B, T, rmax * 1e-9);
    double prevd = 0;
    bool have_prevd = false;
    for (int s = 1; s <= ns; ++s) {
        const double r = rmax * s / ns;
        const double p = pressure_host(eos, A, B, T, r);
        const double d = p - prev;
        if (have_prevd) {
            if (prevd > 0 && d <= 0 && sp1 < 0) sp1 = r;
            else if (prevd <= 0 && d > 0 && sp1 > 0 && sp2 < 0) { sp2 = r; break; }
        }
        prevd = d;
        have_prevd = true;
        prev = p;
    }
    if (sp1 < 0 || sp2 < 0) return -1;  // supercritical
    double g = sp1 * 0.5, l = std::fmin(sp2 * 1.5, rmax * 0.99);
    for (int it = 0; it < 400; ++it) {
        const double mg = mu0_host(eos, A, B, T, g), ml = mu0_host(eos, A, B, T, l);
        const double pg = pressure_host(eos, A, B, T, g), pl = pressure_host(eos, A, B, T, l);
        const double F0 = mg - ml, F1 = pg - pl;
        if (std::fabs(F0) < 1e-16 && std::fabs(F1) < 1e-16) break;
        const double hh = 1e-7;
        const double dmg = (mu0_host(eos, A, B, T, g * (1 + hh)) - mu0_host(eos, A, B, T, g * (1 - hh))) / (2 * g * hh);
        const double dml = (mu0_host(eos, A, B, T, l * (1 + hh)) - mu0_host(eos, A, B, T, l * (1 - hh))) / (2 * l * hh);
        // J = [[dmg, -dml], [g dmg, -l dml]]  (dp/drho = rho dmu/drho)
        const double j00 = dmg, j01 = -dml, j10 = g * dmg, j11 = -l * dml;
        const double det = j00 * j11 - j01 * j10;
        if (det == 0) break;
        const double dx0 = (-F0 * j11 + F1 * j01) / det;
        const double dx1 = (-j00 * F1 + j10 * F0) / det;
        double step = 1.0, ng = g, nl = l;
        for (int k = 0; k < 60; ++k) {
            ng = g + step * dx0;
            nl = l + step * dx1;
            if (ng > 0 && ng < sp1 && nl > sp2 && nl < rmax) break;
            step *= 0.5;
        }
        const double dg = std::fabs(ng - g), dl = std::fabs(nl - l);
        g = ng;
        l = nl;
        if (dg <= 1e-16 * g && dl <= 1e-16 * l) break;
    }
    *g_out = g;
    *l_out = l;
    return 0;
}

int read_cocurve(const char *dir, int model, double tr, double *g, double *l)
{
    const char *tag = table_tag(model);
    if (!tag || !dir) return -1;
    std::string path = std::string(dir) + "/CoCurve_" + tag + "_2.txt";
    std::ifstream f(path.c_str());
    if (!f.is_open()) return -2;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        double t0, dg, dl;
        if (!(is >> t0 >> dg >> dl)) continue;
        if ((t0 > tr ? t0 - tr : tr - t0) < 1e-12) {
            *g = dg;
            *l = dl;
            return 0;
        }
    }
    return -3;
}

}  // namespace cpmp
