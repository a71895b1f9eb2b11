// eos.h -- host-side equation-of-state helpers (see eos.cpp).
#pragma once

namespace cpmp {

enum { EOS_PR = 0, EOS_VDW = 1, EOS_CS = 2, EOS_RK = 3 };

int eos_of_model(int model);
const char *table_tag(int model);
bool eos_constants(int model, double tr, double a, double b, double omega, double *A, double *B,
                   double *Tc, double *Rc);
double mu0_host(int eos, double A, double B, double T, double rho);
double pressure_host(int eos, double A, double B, double T, double rho);
// Coexistence densities in lattice units; returns 0 on success.
int maxwell(int eos, double A, double B, double T, double *g, double *l);
// Reduced (rho / rho_c) coexistence densities from CoCurve_<tag>_2.txt.
int read_cocurve(const char *dir, int model, double tr, double *g, double *l);

}  // namespace cpmp
