/*
 * cpmp_oracle.c -- FP64 CPU restatement of the reference time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library
 * (tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it);
 * nothing in the shipped library calls, links or loads it.
 *
 * Parity pin: compiled with -ffp-contract=off, every function below evaluates
 * the same floating-point expressions in the same order as the reference
 * kernels, so on PR-family EOS it is bit-identical to the reference kernels
 * compiled on the host (oracle/build_ref.py + oracle/ref_shim.cpp), and the
 * committed fixtures in tests/golden/ were produced by that reference build.
 *
 * Reference file:line citations are into zhou-yiling/3DCPMPmodel.
 *
 * Layout (reference Common.h:164, FluidCuda.cu:238): node index
 *   I = (i*DY + j)*DZ + k   (z fastest), populations SoA  f[q*N + I].
 *
 * Extensions beyond the reference (all default to the reference behaviour):
 *   - wall_mode 0: fully periodic box (the reference always has z walls);
 *   - wall_pot: per-column wall chemical potential instead of one BasePt;
 *   - eos: VdW / CS / RK mu0 (the reference evaluates the PR mu0 for every
 *     model id, FluidCuda.cu:453);
 *   - chem_boundary is evaluated layer by layer (deterministic); the
 *     reference kernel reads neighbour columns that other threads rewrite in
 *     the same launch (FluidCuda.cu:389-400).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define Q 19
#define FLUID 1
#define SOLID 2

/* D3Q19 lattice, reference Common.h:96-100 */
static const int EX[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int EY[Q] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int EZ[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int OPP[Q] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
static const double W[Q] = {1. / 3,  1. / 18, 1. / 18, 1. / 18, 1. / 18, 1. / 18, 1. / 18,
                            1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36,
                            1. / 36, 1. / 36, 1. / 36, 1. / 36, 1. / 36};

/* Moment matrix and its inverse (reference Common.h:104-146).  The entries are
 * the standard d'Humieres D3Q19 basis; the inverse is stored, not computed, so
 * the products round exactly as the reference's. */
static const double MM[Q][Q] = {
    {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
    {-30, -11, -11, -11, -11, -11, -11, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8},
    {12, -4, -4, -4, -4, -4, -4, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
    {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0},
    {0, -4, 4, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0},
    {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1},
    {0, 0, 0, -4, 4, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1},
    {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1},
    {0, 0, 0, 0, 0, -4, 4, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1},
    {0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
    {0, -4, -4, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2},
    {0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
    {0, 0, 0, -2, -2, 2, 2, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0, -1, -1, 1, 1, 0, 0, 0, 0, 1, -1, 1, -1},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, -1, -1, 1, 1}};

/* Inverse: row q = direction, column = moment.  Written as the reference's
 * rational literals (Common.h:126-146) so each entry rounds identically. */
static double MINV[Q][Q];
static int minv_ready = 0;
static void build_minv(void)
{
    /* M is orthogonal: M^-1 = M^T diag(1/|row|^2).  The reference literals are
     * exactly M[m][q] / norm[m] evaluated in double (e.g. 1./19, -5./399,
     * -11./2394, 4./1197, 1./252 ...), so computing the quotient of the two
     * integers reproduces each literal's correctly rounded double. */
    for (int m = 0; m < Q; ++m) {
        long n2 = 0;
        for (int q = 0; q < Q; ++q) n2 += (long)(MM[m][q] * MM[m][q]);
        for (int q = 0; q < Q; ++q) {
            long num = (long)MM[m][q];
            /* reduce num/n2 the way the literals are written: the double of an
             * exact rational is unique, so any exact evaluation agrees */
            MINV[q][m] = (double)num / (double)n2;
        }
    }
    minv_ready = 1;
}

typedef struct orc_params {
    int dx, dy, dz;
    double K, A, B, T, Ka, K1, K2;
    double ts[Q];
    int eos;        /* 0 PR (reference), 1 VdW, 2 CS, 3 RK */
    int lap_order;  /* 5: GradD5 (reference default), 7: GradD7 */
    int complex_bc; /* 1: layered wall extrapolation (reference default) */
    int wall_mode;  /* 0: periodic, 1: solid layers k<3 and k>DZ-4 */
    double base_pt; /* wall chemical potential when wall_pot is NULL */
    const double *wall_pot; /* optional [2][dx*dy]: bottom then top wall */
} orc_params;

typedef struct orc_droplet {
    double cx, cy, cz, radius, width, den_g, den_l;
    int ref_centre; /* 1: reference placement (DX/2, DY/2, R+2) with sqrtf */
} orc_droplet;

#define IDX(p, i, j, k) ((((long)(i)) * (p)->dy + (j)) * (long)(p)->dz + (k))

static inline int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

static inline int is_solid_layer(const orc_params *p, int k)
{
    return p->wall_mode == 1 && (k < 3 || k > p->dz - 4);
}

/* Equilibrium, reference FluidCuda.cu:189-193 */
static inline double feq(int q, double rho, double ux, double uy, double uz)
{
    double eu = ux * EX[q] + uy * EY[q] + uz * EZ[q];
    return rho * W[q] * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * (ux * ux + uy * uy + uz * uz));
}

/* ---------------------------------------------------------------- init --- */
/* SetFlowField, reference FluidCuda.cu:199-241 (CONTACTANGLE branch). */
void orc_init(const orc_params *p, const orc_droplet *d, uint8_t *type, double *dens,
              double *pote, double *dist, double *vx, double *vy, double *vz)
{
    const int DX = p->dx, DY = p->dy, DZ = p->dz;
    const long N = (long)DX * DY * DZ;
#pragma omp parallel for schedule(static)
    for (long I = 0; I < N; ++I) {
        int i = (int)(I / DY / DZ), j = (int)((I / DZ) % DY), k = (int)(I % DZ);
        if (is_solid_layer(p, k)) {
            type[I] = SOLID;
            double wp = p->wall_pot ? p->wall_pot[(k < 3 ? 0 : (long)DX * DY) + (long)i * DY + j]
                                    : p->base_pt;
            dens[I] = pote[I] = wp;
        } else {
            type[I] = FLUID;
            pote[I] = 0;
            double r;
            if (d->ref_centre) {
                /* the reference takes sqrtf of a double sum (FluidCuda.cu:215) */
                double s = (((double)i - DX / 2) * ((double)i - DX / 2)) +
                           (((double)j - DY / 2) * ((double)j - DY / 2)) +
                           (((double)k - (d->radius + 2)) * ((double)k - (d->radius + 2)));
                r = (double)sqrtf((float)s);
            } else {
                double ax = i - d->cx, ay = j - d->cy, az = k - d->cz;
                r = sqrt(ax * ax + ay * ay + az * az);
            }
            dens[I] = (d->den_l + d->den_g) / 2 -
                      (d->den_l - d->den_g) / 2 * tanh((r - d->radius) * 2 / d->width);
        }
        for (int q = 0; q < Q; ++q) dist[q * N + I] = feq(q, dens[I], 0, 0, 0);
        vx[I] = vy[I] = vz[I] = 0;
    }
}

/* ------------------------------------------------------- wall boundary --- */
/* Six-point extrapolation of one wall layer from the adjacent layer:
 * (2*centre + four xy-diagonal neighbours)/6, reference FluidCuda.cu:382. */
static inline double wall_avg(const orc_params *p, const double *dens, int i, int j, int k)
{
    const int DX = p->dx, DY = p->dy;
    int i1 = i > 0 ? i - 1 : DX - 1, i2 = i < DX - 1 ? i + 1 : 0;
    int j1 = j > 0 ? j - 1 : DY - 1, j2 = j < DY - 1 ? j + 1 : 0;
    return (dens[IDX(p, i, j, k)] * 2 + dens[IDX(p, i1, j1, k)] + dens[IDX(p, i1, j2, k)] +
            dens[IDX(p, i2, j1, k)] + dens[IDX(p, i2, j2, k)]) / 6;
}

/* ChemBoundary, reference FluidCuda.cu:376-401, evaluated layer by layer:
 * pass 1 sets all three solid layers from the first fluid layer; the complex
 * pass then recomputes layer 1 (resp. DZ-2) from layer 2 (DZ-3) over the whole
 * plane, then layer 0 (DZ-1) from layer 1 (DZ-2). */
void orc_chem_boundary(const orc_params *p, double *dens, double *pote)
{
    if (p->wall_mode != 1) return;
    const int DX = p->dx, DY = p->dy, DZ = p->dz;
    const long NP = (long)DX * DY;
    double *tmp = (double *)malloc(sizeof(double) * NP * 2);
    /* pass 1 */
    for (long c = 0; c < NP; ++c) {
        int i = (int)(c / DY), j = (int)(c % DY);
        tmp[c] = wall_avg(p, dens, i, j, 3);
        tmp[NP + c] = wall_avg(p, dens, i, j, DZ - 4);
    }
    for (long c = 0; c < NP; ++c) {
        int i = (int)(c / DY), j = (int)(c % DY);
        dens[IDX(p, i, j, 0)] = dens[IDX(p, i, j, 1)] = dens[IDX(p, i, j, 2)] = tmp[c];
        dens[IDX(p, i, j, DZ - 3)] = dens[IDX(p, i, j, DZ - 1)] = dens[IDX(p, i, j, DZ - 2)] =
            tmp[NP + c];
        double wb = p->wall_pot ? p->wall_pot[c] : p->base_pt;
        double wt = p->wall_pot ? p->wall_pot[NP + c] : p->base_pt;
        pote[IDX(p, i, j, 0)] = pote[IDX(p, i, j, 1)] = pote[IDX(p, i, j, 2)] = wb;
        pote[IDX(p, i, j, DZ - 3)] = pote[IDX(p, i, j, DZ - 2)] = pote[IDX(p, i, j, DZ - 1)] = wt;
    }
    if (p->complex_bc) {
        /* layer 1 from layer 2, layer DZ-2 from layer DZ-3 */
        for (long c = 0; c < NP; ++c) {
            int i = (int)(c / DY), j = (int)(c % DY);
            tmp[c] = wall_avg(p, dens, i, j, 2);
            tmp[NP + c] = wall_avg(p, dens, i, j, DZ - 3);
        }
        for (long c = 0; c < NP; ++c) {
            int i = (int)(c / DY), j = (int)(c % DY);
            dens[IDX(p, i, j, 1)] = tmp[c];
            dens[IDX(p, i, j, DZ - 2)] = tmp[NP + c];
        }
        /* layer 0 from layer 1, layer DZ-1 from layer DZ-2 */
        for (long c = 0; c < NP; ++c) {
            int i = (int)(c / DY), j = (int)(c % DY);
            tmp[c] = wall_avg(p, dens, i, j, 1);
            tmp[NP + c] = wall_avg(p, dens, i, j, DZ - 2);
        }
        for (long c = 0; c < NP; ++c) {
            int i = (int)(c / DY), j = (int)(c % DY);
            dens[IDX(p, i, j, 0)] = tmp[c];
            dens[IDX(p, i, j, DZ - 1)] = tmp[NP + c];
        }
    }
    free(tmp);
}

/* ------------------------------------------------------------- stencils --- */
/* Neighbour offsets along one axis with periodic wrap, radius r. */
typedef struct { int m[4], pl[4]; } nb_t; /* m[d] = index - d, pl[d] = index + d, d=1..3 */
static inline nb_t nbs(int a, int n)
{
    nb_t o;
    for (int d = 1; d <= 3; ++d) {
        int lo = a, hi = a;
        for (int s = 0; s < d; ++s) { lo = lo > 0 ? lo - 1 : n - 1; hi = hi < n - 1 ? hi + 1 : 0; }
        o.m[d] = lo; o.pl[d] = hi;
    }
    o.m[0] = o.pl[0] = a;
    return o;
}

/* 4th-order 13-point Laplacian, reference Common.h:189-192 (GradD5). */
static inline double lap5(const orc_params *p, const double *x, int i, int j, int k)
{
    nb_t a = nbs(i, p->dx), b = nbs(j, p->dy), c = nbs(k, p->dz);
#define X(ii, jj, kk) x[IDX(p, ii, jj, kk)]
    return (-X(i, j, k) * 90 +
            (-X(a.m[2], j, k) + X(a.m[1], j, k) * 16 + X(a.pl[1], j, k) * 16 - X(a.pl[2], j, k)) +
            (-X(i, b.m[2], k) + X(i, b.m[1], k) * 16 + X(i, b.pl[1], k) * 16 - X(i, b.pl[2], k)) +
            (-X(i, j, c.m[2]) + X(i, j, c.m[1]) * 16 + X(i, j, c.pl[1]) * 16 - X(i, j, c.pl[2]))) /
           12;
}

/* 6th-order 19-point Laplacian, reference Common.h:243-246 (GradD7), returned
 * WITHOUT its final /180: the reference macro has no outer parentheses, so at
 * its use site (FluidCuda.cu:460) it evaluates (Ka * sum) / 180. */
static inline double lap7_sum(const orc_params *p, const double *x, int i, int j, int k)
{
    nb_t a = nbs(i, p->dx), b = nbs(j, p->dy), c = nbs(k, p->dz);
    return (-X(i, j, k) * 490 * 3 +
            (2 * X(a.m[3], j, k) - 27 * X(a.m[2], j, k) + 270 * X(a.m[1], j, k) +
             270 * X(a.pl[1], j, k) - 27 * X(a.pl[2], j, k) + 2 * X(a.pl[3], j, k)) +
            (2 * X(i, b.m[3], k) - 27 * X(i, b.m[2], k) + 270 * X(i, b.m[1], k) +
             270 * X(i, b.pl[1], k) - 27 * X(i, b.pl[2], k) + 2 * X(i, b.pl[3], k)) +
            (2 * X(i, j, c.m[3]) - 27 * X(i, j, c.m[2]) + 270 * X(i, j, c.m[1]) +
             270 * X(i, j, c.pl[1]) - 27 * X(i, j, c.pl[2]) + 2 * X(i, j, c.pl[3])));
}

/* One 6th-order first-difference along a lattice line through (i,j,k):
 * sum_d c_d (x(+d) - x(-d)) with c = (45, -9, 1), written in the reference's
 * term order  -x(-3) + 9x(-2) - 45x(-1) + 45x(+1) - 9x(+2) + x(+3). */
#define LINE(A1, B1, C1, A2, B2, C2, A3, B3, C3, A5, B5, C5, A6, B6, C6, A7, B7, C7) \
    (-X(A1, B1, C1) + X(A2, B2, C2) * 9 - X(A3, B3, C3) * 45 + X(A5, B5, C5) * 45 -   \
     X(A6, B6, C6) * 9 + X(A7, B7, C7))

/* D3Q19-weighted gradient, reference Common.h:222-241 (Gradx7/y7/z7).
 * Index convention of the reference: 1,2,3 = -3,-2,-1 and 5,6,7 = +1,+2,+3. */
static inline void grad7(const orc_params *p, const double *x, int i, int j, int k, double g[3])
{
    nb_t a = nbs(i, p->dx), b = nbs(j, p->dy), c = nbs(k, p->dz);
    int i1 = a.m[3], i2 = a.m[2], i3 = a.m[1], i5 = a.pl[1], i6 = a.pl[2], i7 = a.pl[3];
    int j1 = b.m[3], j2 = b.m[2], j3 = b.m[1], j5 = b.pl[1], j6 = b.pl[2], j7 = b.pl[3];
    int k1 = c.m[3], k2 = c.m[2], k3 = c.m[1], k5 = c.pl[1], k6 = c.pl[2], k7 = c.pl[3];
    g[0] = (LINE(i1, j, k, i2, j, k, i3, j, k, i5, j, k, i6, j, k, i7, j, k) * 2 +
            LINE(i1, j, k1, i2, j, k2, i3, j, k3, i5, j, k5, i6, j, k6, i7, j, k7) +
            LINE(i1, j, k7, i2, j, k6, i3, j, k5, i5, j, k3, i6, j, k2, i7, j, k1) +
            LINE(i1, j1, k, i2, j2, k, i3, j3, k, i5, j5, k, i6, j6, k, i7, j7, k) +
            LINE(i1, j7, k, i2, j6, k, i3, j5, k, i5, j3, k, i6, j2, k, i7, j1, k)) /
           360;
    g[1] = (LINE(i, j1, k, i, j2, k, i, j3, k, i, j5, k, i, j6, k, i, j7, k) * 2 +
            LINE(i, j1, k1, i, j2, k2, i, j3, k3, i, j5, k5, i, j6, k6, i, j7, k7) +
            LINE(i, j1, k7, i, j2, k6, i, j3, k5, i, j5, k3, i, j6, k2, i, j7, k1) +
            LINE(i1, j1, k, i2, j2, k, i3, j3, k, i5, j5, k, i6, j6, k, i7, j7, k) +
            LINE(i7, j1, k, i6, j2, k, i5, j3, k, i3, j5, k, i2, j6, k, i1, j7, k)) /
           360;
    g[2] = (LINE(i, j, k1, i, j, k2, i, j, k3, i, j, k5, i, j, k6, i, j, k7) * 2 +
            LINE(i1, j, k1, i2, j, k2, i3, j, k3, i5, j, k5, i6, j, k6, i7, j, k7) +
            LINE(i7, j, k1, i6, j, k2, i5, j, k3, i3, j, k5, i2, j, k6, i1, j, k7) +
            LINE(i, j1, k1, i, j2, k2, i, j3, k3, i, j5, k5, i, j6, k6, i, j7, k7) +
            LINE(i, j7, k1, i, j6, k2, i, j5, k3, i, j3, k5, i, j2, k6, i, j1, k7)) /
           360;
}
#undef X

/* ------------------------------------------------------------------ EOS --- */
#define SQRT2 1.4142135623730950488016887242097

/* Bulk chemical potential mu0(rho).  PR is the reference's expression
 * (FluidCuda.cu:453) including its density soft cap (FluidCuda.cu:450-451);
 * the other forms are d(psi)/d(rho) of the same free-energy convention
 * psi = rho*T*ln(rho/(1-B rho)) + attraction (so every form tends to
 * T ln(rho) + T at low density, like the reference's PR form). */
double orc_mu0(int eos, double A, double B, double T, double rho)
{
    double Den = rho, R0 = 9.7, W0 = 1.5;
    if (Den > R0) { Den = R0 + (Den - R0) / (1.0 + (Den - R0) * W0); }
    switch (eos) {
    case 1: /* van der Waals */
        return T * log(Den / (1.0 - B * Den)) + T / (1.0 - B * Den) - 2 * A * Den;
    case 2: { /* Carnahan-Starling, eta = B rho (B = b/4) */
        double e = B * Den, om = 1.0 - e;
        return T * log(Den) + T + T * (8 * e - 9 * e * e + 3 * e * e * e) / (om * om * om) -
               2 * A * Den;
    }
    case 3: /* Redlich-Kwong (RKS / RKE: alpha folded into A) */
        return T * log(Den / (1.0 - B * Den)) + T / (1.0 - B * Den) - A / B * log(1.0 + B * Den) -
               A * Den / (1.0 + B * Den);
    default: /* Peng-Robinson, reference expression */
        return T * log(Den / (1.0 - B * Den)) -
               A / (SQRT2 * 2 * B) * log((SQRT2 - 1 + B * Den) / (SQRT2 + 1 - B * Den)) +
               T / (1.0 - B * Den) - A * Den / (1.0 + B * Den * 2 - (B * Den) * (B * Den));
    }
}

/* Equation-of-state pressure (no cap); PR and VdW follow FluidCuda.cu:1567-1569. */
double orc_pressure(int eos, double A, double B, double T, double rho)
{
    switch (eos) {
    case 1: return T * rho / (1.0 - B * rho) - A * rho * rho;
    case 2: {
        double e = B * rho, om = 1.0 - e;
        return rho * T * (1 + e + e * e - e * e * e) / (om * om * om) - A * rho * rho;
    }
    case 3: return T * rho / (1.0 - B * rho) - A * rho * rho / (1.0 + B * rho);
    default: return T * rho / (1.0 - B * rho) - A * rho * rho / (1.0 + B * rho * 2 - (B * rho) * (B * rho));
    }
}

/* ChemPotential, reference FluidCuda.cu:444-463. */
void orc_chem_potential(const orc_params *p, const uint8_t *type, const double *dens, double *pote)
{
    const int DY = p->dy, DZ = p->dz;
    const long N = (long)p->dx * DY * DZ;
#pragma omp parallel for schedule(static)
    for (long I = 0; I < N; ++I) {
        if (type[I] != FLUID) continue;
        int i = (int)(I / DY / DZ), j = (int)((I / DZ) % DY), k = (int)(I % DZ);
        double mu = orc_mu0(p->eos, p->A, p->B, p->T, dens[I]);
        if (p->lap_order == 7)
            pote[I] = (p->K * p->K) * mu - p->Ka * lap7_sum(p, dens, i, j, k) / 180;
        else
            pote[I] = (p->K * p->K) * mu - p->Ka * lap5(p, dens, i, j, k);
    }
}

/* NonidealForce, reference FluidCuda.cu:431-441. */
void orc_force(const orc_params *p, const uint8_t *type, const double *dens, const double *pote,
               double *fx, double *fy, double *fz)
{
    const int DY = p->dy, DZ = p->dz;
    const long N = (long)p->dx * DY * DZ;
#pragma omp parallel for schedule(static)
    for (long I = 0; I < N; ++I) {
        if (type[I] != FLUID) continue;
        int i = (int)(I / DY / DZ), j = (int)((I / DZ) % DY), k = (int)(I % DZ);
        double gm[3], gr[3];
        grad7(p, pote, i, j, k, gm);
        grad7(p, dens, i, j, k, gr);
        fx[I] = -gm[0] * dens[I] + gr[0] / 3;
        fy[I] = -gm[1] * dens[I] + gr[1] / 3;
        fz[I] = -gm[2] * dens[I] + gr[2] / 3;
    }
}

/* --------------------------------------------------------- collide/stream --- */
/* GlobalCollide + LocalCollideMrt, reference FluidCuda.cu:245-347.
 * Collision in moment space with the bare velocity, exact-difference forcing
 * with the shifted velocity u + F/rho, push streaming into `tmp` with periodic
 * wrap and half-way bounce-back onto the source node when the destination is
 * solid.  Writes the physical velocity u + F/(2 rho). */
void orc_collide(const orc_params *p, const uint8_t *type, const double *dens, double *dist,
                 double *tmp, const double *vx, const double *vy, const double *vz,
                 const double *fx, const double *fy, const double *fz, double *mvx, double *mvy,
                 double *mvz)
{
    if (!minv_ready) build_minv();
    const int DX = p->dx, DY = p->dy, DZ = p->dz;
    const long N = (long)DX * DY * DZ;
    const int with_qp = (p->K1 != 0 || p->K2 != 0);
#pragma omp parallel for schedule(static)
    for (long I = 0; I < N; ++I) {
        if (type[I] != FLUID) continue;
        int i = (int)(I / DY / DZ), j = (int)((I / DZ) % DY), k = (int)(I % DZ);
        double rho = dens[I];
        double Vx = vx[I], Vy = vy[I], Vz = vz[I];
        mvx[I] = Vx + fx[I] / rho * 0.5;
        mvy[I] = Vy + fy[I] / rho * 0.5;
        mvz[I] = Vz + fz[I] / rho * 0.5;
        double EVx = Vx + fx[I] / rho, EVy = Vy + fy[I] / rho, EVz = Vz + fz[I] / rho;

        double qp[Q] = {0};
        if (with_qp) { /* K1/K2 pressure-tensor term, FluidCuda.cu:260-266 */
            double g[3];
            grad7(p, dens, i, j, k, g);
            qp[1] = -19 * (p->K1 + 3 * p->K2) * (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            qp[9] = -p->K1 * (2 * g[0] * g[0] - g[1] * g[1] - g[2] * g[2]);
            qp[11] = -p->K1 * (g[1] * g[1] - g[2] * g[2]);
            qp[13] = -p->K1 * g[0] * g[1];
            qp[14] = -p->K1 * g[2] * g[1];
            qp[15] = -p->K1 * g[0] * g[2];
        }
        double u2 = Vx * Vx + Vy * Vy + Vz * Vz;
        double meq[Q];
        meq[0] = rho;
        meq[1] = rho * (-11.0 + 19.0 * u2);
        meq[2] = rho * (3.0 - 11.0 / 2 * u2);
        meq[3] = rho * Vx;
        meq[4] = rho * Vx * -2 / 3;
        meq[5] = rho * Vy;
        meq[6] = rho * Vy * -2 / 3;
        meq[7] = rho * Vz;
        meq[8] = rho * Vz * -2 / 3;
        meq[9] = rho * (Vx * Vx * 2 - Vy * Vy - Vz * Vz);
        meq[10] = rho * (Vx * Vx * 2 - Vy * Vy - Vz * Vz) / -2;
        meq[11] = rho * (Vy * Vy - Vz * Vz);
        meq[12] = rho * (Vy * Vy - Vz * Vz) / -2;
        meq[13] = rho * Vx * Vy;
        meq[14] = rho * Vy * Vz;
        meq[15] = rho * Vx * Vz;
        meq[16] = meq[17] = meq[18] = 0;

        double f[Q], m[Q];
        for (int q = 0; q < Q; ++q) f[q] = dist[q * N + I];
        for (int a = 0; a < Q; ++a) {
            double s = 0;
            for (int q = 0; q < Q; ++q) s += MM[a][q] * f[q];
            m[a] = s;
        }
        for (int a = 0; a < Q; ++a) m[a] = m[a] - p->ts[a] * (m[a] - meq[a]) + qp[a] * p->ts[a];
        for (int q = 0; q < Q; ++q) {
            double s = 0;
            for (int a = 0; a < Q; ++a) s += MINV[q][a] * m[a];
            f[q] = s;
            dist[q * N + I] = s; /* the reference writes the post-collision value in place */
        }
        for (int q = 0; q < Q; ++q) {
            int ii = wrap(i + EX[q], DX), jj = wrap(j + EY[q], DY), kk = wrap(k + EZ[q], DZ);
            double df = f[q] + feq(q, rho, EVx, EVy, EVz) - feq(q, rho, Vx, Vy, Vz);
            long D = IDX(p, ii, jj, kk);
            if (type[D] == FLUID) tmp[q * N + D] = df;
            else tmp[OPP[q] * N + I] = df;
        }
    }
}

/* MacroCalculate, reference FluidCuda.cu:351-372. */
void orc_macro(const orc_params *p, const uint8_t *type, double *dens, const double *dist,
               double *vx, double *vy, double *vz)
{
    const long N = (long)p->dx * p->dy * p->dz;
#pragma omp parallel for schedule(static)
    for (long I = 0; I < N; ++I) {
        if (type[I] != FLUID) continue;
        double r = 0;
        for (int q = 0; q < Q; ++q) r += dist[q * N + I];
        dens[I] = r;
#define DF(q) dist[(long)(q) * N + I]
        vx[I] = (DF(1) + DF(7) + DF(9) + DF(11) + DF(13) - DF(2) - DF(8) - DF(10) - DF(12) - DF(14)) / r;
        vy[I] = (DF(3) + DF(7) + DF(8) + DF(15) + DF(17) - DF(4) - DF(9) - DF(10) - DF(16) - DF(18)) / r;
        vz[I] = (DF(5) + DF(11) + DF(12) + DF(15) + DF(16) - DF(6) - DF(13) - DF(14) - DF(17) - DF(18)) / r;
#undef DF
    }
}

/* One full time step in the reference's launch order (FluidCuda.cu:1279-1291).
 * `dist` holds the current populations on entry and on return (the
 * reference's pointer swap is undone by copying). */
void orc_step(const orc_params *p, int nsteps, const uint8_t *type, double *dens, double *pote,
              double *dist, double *tmp, double *vx, double *vy, double *vz, double *fx, double *fy,
              double *fz, double *mvx, double *mvy, double *mvz)
{
    const long N = (long)p->dx * p->dy * p->dz;
    for (int s = 0; s < nsteps; ++s) {
        orc_chem_boundary(p, dens, pote);
        orc_chem_potential(p, type, dens, pote);
        orc_force(p, type, dens, pote, fx, fy, fz);
        orc_collide(p, type, dens, dist, tmp, vx, vy, vz, fx, fy, fz, mvx, mvy, mvz);
        memcpy(dist, tmp, sizeof(double) * (size_t)Q * N);
        orc_macro(p, type, dens, dist, vx, vy, vz);
    }
}

/* --------------------------------------------------------- diagnostics --- */
/* CalcMacroCPU, reference FluidCuda.cu:1626-1657: FP64 mass over fluid nodes,
 * non-finite / negative flag, max |MV|.  Sequential sum in index order. */
void orc_mass(const orc_params *p, const uint8_t *type, const double *dens, const double *mvx,
              const double *mvy, const double *mvz, double out[3])
{
    const long N = (long)p->dx * p->dy * p->dz;
    double mass = 0, mx = 0;
    int bad = 0;
    for (long I = 0; I < N; ++I) {
        if (type[I] != FLUID) continue;
        double d = dens[I];
        if (d != d || d < 0) bad = 1;
        mass += d;
        double m = mvx[I] * mvx[I] + mvy[I] * mvy[I] + mvz[I] * mvz[I];
        if (m > mx) mx = m;
    }
    out[0] = mass;
    out[1] = sqrt(mx);
    out[2] = bad;
}

/* ContactAngle(side = 0, tier), reference FluidCuda.cu:557-734, on the x-z
 * slice j = tier.  out = {CaLeft, CaRight, CaCap, XLeft, XRight, H, L}. */
void orc_contact_angle(const orc_params *p, const double *dens, int tier, double den_g,
                       double den_l, double out[7])
{
    const int DX = p->dx, DY = p->dy, DZ = p->dz;
    const double PI2 = 3.14159265358979323846264338327950288;
    double mid = (den_g + den_l) / 2;
    double px[8] = {0};
#define T(ii, kk) dens[IDX(p, ii, tier, kk)]
    for (int kk = 2; kk <= 5; ++kk) {
        int n = (kk - 2) * 2;
        for (int i = 0; i < DX / 2 + 2; ++i) {
            double t1 = T(i + 1, kk), t2 = T(i + 2, kk);
            if (t1 < mid && t2 >= mid) { px[n] = (double)(i + 1) + (t1 - mid) / (t1 - t2); break; }
        }
        for (int i = DX - 2; i > DX / 2 - 2; --i) {
            double t1 = T(i - 1, kk), t2 = T(i - 2, kk);
            if (t1 < mid && t2 >= mid) { px[n + 1] = (double)(i - 1) - (t1 - mid) / (t1 - t2); break; }
        }
    }
    double y0 = 2, y1 = 3, y2 = 4;
    double xl, xr, cl, cr, cap = 0, H = 0, L = 0;
    if (px[0] != 0.0 && px[1] != 0.0) {
        xl = px[2] * ((y0 - y2) / (y1 - y2)) + px[4] * ((y0 - y1) / (y2 - y1));
        xr = px[3] * ((y0 - y2) / (y1 - y2)) + px[5] * ((y0 - y1) / (y2 - y1));
        double ca = atan((y1 - y0) / (px[2] - xl));
        if (ca < 0) ca += PI2;
        cl = ca / PI2 * 180;
        ca = atan(-(y1 - y0) / (px[3] - xr));
        if (ca < 0) ca += PI2;
        cr = ca / PI2 * 180;
        L = xr - xl;
        int ic = (int)((px[4] + px[5]) / 2 + 0.5);
        for (int kk = 2; kk < DZ - 2; ++kk) {
            double t = T(ic, kk), t1 = T(ic, kk + 1);
            if (t >= mid && t1 < mid) H = (double)kk + (t - mid) / (t - t1) - y0;
        }
        if (L <= 0) { L = px[3] - px[2]; H = H - 0.5; }
        if (xl > DY / 2 && xr < DY / 2) { xl = DY / 2; xr = DY / 2; }
        double R = (H * H * 4 + L * L) / H / 8;
        cap = atan(L / (R - H) / 2);
        if (cap < 0) cap += PI2;
        cap = cap / PI2 * 180;
    } else {
        xl = xr = DY / 2;
        cl = cr = 0;
    }
#undef T
    out[0] = cl; out[1] = cr; out[2] = cap; out[3] = xl; out[4] = xr; out[5] = H; out[6] = L;
}

/* Droplet-impact sums, FP64, sequential in the reference's loop order.
 * ComputeEnergy (FluidCuda.cu:737-787) and Computetangential_velocity
 * (:790-898): fluid nodes with rho > mid, 2 <= i < DX-2, 2 <= j < DY-2,
 * 2 <= k < DZ-2, loops i, j, k.  SaveSpreadtime (:1128-1150): every node with
 * rho > mid and 2 <= k < DZ-2, loops i, j, k.
 * out = {V, VXY, VZ, MV, MVXY, MVZ, energy, energyXY, energyZ,
 *        tangential_vel, Mtangential_vel, mvel, dropmass} */
void orc_impact(const orc_params *p, const uint8_t *type, const double *dens, const double *mvx,
                const double *mvy, const double *mvz, double den_g, double den_l, double out[13])
{
    const int DX = p->dx, DY = p->dy, DZ = p->dz;
    const double PI2 = 3.14159265358979323846264338327950288;
    const double mid = (den_g + den_l) / 2;
    double s[11] = {0};
    for (int i = 2; i < DX - 2; i++)
        for (int j = 2; j < DY - 2; j++)
            for (int k = 2; k < DZ - 2; k++) {
                const long I = IDX(p, i, j, k);
                if (type[I] == FLUID && dens[I] > mid) {
                    const double a = mvx[I], b = mvy[I], c = mvz[I], d = dens[I];
                    s[0] += sqrt(a * a + b * b + c * c);
                    s[1] += sqrt(a * a + b * b);
                    s[2] += c;
                    s[3] += d * sqrt(a * a + b * b + c * c);
                    s[4] += d * sqrt(a * a + b * b);
                    s[5] += d * c;
                    s[6] += d * (a * a + b * b + c * c) / 2;
                    s[7] += d * (a * a + b * b) / 2;
                    s[8] += d * (c * c) / 2;
                }
            }
    for (int i = 2; i < DX - 2; i++)
        for (int j = 2; j < DY - 2; j++)
            for (int k = 2; k < DZ - 2; k++) {
                const long I = IDX(p, i, j, k);
                if (type[I] == FLUID && dens[I] > mid) {
                    double alpha = atan2((double)(j - DY / 2), (double)(i - DX / 2)) / PI2 * 180;
                    if (alpha < 0) alpha = alpha + 360;
                    alpha = alpha / 180 * PI2;
                    const double t = mvx[I] * sin(alpha) + mvy[I] * cos(alpha);
                    s[9] += t;
                    s[10] += t * dens[I];
                }
            }
    double mvel = 0, mass = 0;
    for (int i = 0; i < DX; i++)
        for (int j = 0; j < DY; j++)
            for (int k = 2; k < DZ - 2; k++) {
                const long I = IDX(p, i, j, k);
                if (dens[I] > mid) {
                    mvel += dens[I] * sqrt(mvx[I] * mvx[I] + mvy[I] * mvy[I] + mvz[I] * mvz[I]);
                    mass += dens[I];
                }
            }
    for (int q = 0; q < 11; ++q) out[q] = s[q];
    out[11] = mvel;
    out[12] = mass;
}
