/*
 * cpmp.h -- C ABI of the GB300 chemical-potential multiphase D3Q19 MRT
 * lattice-Boltzmann step.
 *
 * The reference (zhou-yiling/3DCPMPmodel) has no library interface: its step
 * contract is a set of global device fields, __constant__ parameters, a
 * compile-time grid and a per-step launch sequence inside main().  Each entry
 * point below replaces one piece of that contract; the comment on each names
 * the reference code it stands in for (file:line in the reference tree).
 *
 * Conventions
 *   - The handle owns all device memory; host buffers are caller-owned.
 *   - Every call returns a cpmp_status and never aborts or traps;
 *     cpmp_last_error() gives a one-line message for the calling thread.
 *   - One handle is used from one host thread at a time.
 *   - Field layout is the reference's: node index I = (i*DY + j)*DZ + k
 *     (z fastest, Common.h:164); vector fields are three consecutive blocks
 *     of N values (x, y, z); populations are 19 consecutive blocks of N.
 */
#ifndef CPMP_H
#define CPMP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPMP_Q 19
#define CPMP_ABI_VERSION 1

typedef enum cpmp_status {
    CPMP_OK = 0,
    CPMP_ERR_PARAM = 1,       /* invalid argument or parameter set */
    CPMP_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    CPMP_ERR_NOMEM = 3,       /* device or host allocation failed */
    CPMP_ERR_COCURVE = 4,     /* coexistence table missing or T/Tc row absent */
    CPMP_ERR_NONFINITE = 5,   /* NaN or negative density seen by cpmp_reduce */
    CPMP_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
    CPMP_ERR_UNSUPPORTED = 7, /* option combination not provided */
    CPMP_ERR_SIZE = 8         /* buffer size does not match the field */
} cpmp_status;

/* Model ids of the chemical-potential family, reference Common.h:54-59. */
enum {
    CPMP_MP_CPVDW = 201,
    CPMP_MP_CPPRW = 202,
    CPMP_MP_CPPRM = 203,
    CPMP_MP_CPRKE = 204,
    CPMP_MP_CPRKS = 205,
    CPMP_MP_CPCSE = 206
};

enum { CPMP_WALL_NONE = 0, CPMP_WALL_Z = 1 };
enum { CPMP_STORE_F64 = 0, CPMP_STORE_F32 = 1, CPMP_STORE_F16 = 2, CPMP_STORE_BF16 = 3 };
/* PLAIN: one kernel per reference kernel, two population lattices, reference
 *        launch order (FluidCuda.cu:1279-1291); storage F64 or F32.
 * FUSED: wall + fused mu/force/MRT/forcing/stream kernel + density kernel,
 *        one in-place A-A population lattice; storage F32, F16 or BF16. */
enum { CPMP_SCHEME_PLAIN = 0, CPMP_SCHEME_FUSED = 1 };
enum { CPMP_F64 = 0, CPMP_F32 = 1 }; /* host dtype of cpmp_get_field/cpmp_set_field */

typedef enum cpmp_field {
    CPMP_FIELD_RHO = 0,   /* density, N            (reference Dens) */
    CPMP_FIELD_U = 1,     /* bare velocity, 3N     (reference Vx,Vy,Vz) */
    CPMP_FIELD_MV = 2,    /* physical velocity u+F/(2 rho), 3N (MVx,MVy,MVz) */
    CPMP_FIELD_MU = 3,    /* chemical potential, N (reference Pote) */
    CPMP_FIELD_FORCE = 4, /* non-ideal force, 3N   (reference Fx,Fy,Fz) */
    CPMP_FIELD_DIST = 5,  /* post-stream populations, 19N (reference Dist) */
    CPMP_FIELD_TYPE = 6   /* node tags FLUID=1 / SOLID=2, N bytes (Type) */
} cpmp_field;

/* Every knob of the reference's Initialize() (FluidCuda.cu:119-163),
 * SetMultiphase() (FluidCuda.cu:1314-1394), the compile-time grid
 * (Common.h:25-27) and the compile-time switches (FluidCuda.cu:1-7). */
typedef struct cpmp_params {
    int dx, dy, dz;       /* grid (Common.h:25-27) */
    int model;            /* CPMP_MP_* (Initialize: MModel) */
    double tr;            /* T/Tc (Tr) */
    double k;             /* EOS scale: mu = K^2 mu0 - ka lap(rho) (K) */
    double ka;            /* kappa (Ka) */
    double k1, k2;        /* pressure-tensor correction (K1, K2) */
    double tau;           /* shear relaxation time (Tau) */
    double ts[CPMP_Q];    /* MRT rates (Ts[]); used when ts_from_tau == 0 */
    int ts_from_tau;      /* 1: the reference's rates built from tau (FluidCuda.cu:154-157) */
    double base_pt;       /* wall chemical potential (BasePt) */
    double eos_a, eos_b;  /* CS constants a, b (0: the reference's a=1, b=4) */
    double eos_omega;     /* PR/RKS acentric factor (0: the model's own) */
    double den_g, den_l;  /* > 0: coexistence densities given directly */
    const char *cocurve_dir; /* directory of CoCurve_<EOS>_2.txt; NULL: built-in
                                Maxwell construction */
    int wall_mode;        /* CPMP_WALL_Z: three solid layers at each z end
                             (CONTACTANGLE); CPMP_WALL_NONE: periodic box */
    int lap_order;        /* 5: GradD5 (PTCALCFIVEPOINT), 7: GradD7 (PTCALCSEVENPOINT) */
    int complex_bc;       /* 1: layered wall extrapolation (COMPLEXCHEMBOUNDARY),
                             0: SIMPLECHEMBOUNDARY */
    int storage;          /* CPMP_STORE_* */
    int scheme;           /* CPMP_SCHEME_* */
    int device;           /* CUDA device ordinal */
} cpmp_params;

/* Initial droplet, SetFlowField (FluidCuda.cu:199-241). */
typedef struct cpmp_droplet {
    double cx, cy, cz;    /* centre (ignored when ref_centre = 1) */
    double radius;        /* Radius */
    double width;         /* tanh width parameter (Width) */
    int ref_centre;       /* 1: the reference's placement (DX/2, DY/2, R+2) and
                             its single-precision radius (FluidCuda.cu:215) */
} cpmp_droplet;

/* Diagnostics of CalcMacroCPU (FluidCuda.cu:1626-1657), ContactAngle
 * (FluidCuda.cu:557-734) and the Laplace-law probe of SaveDataOriDen
 * (FluidCuda.cu:1159-1199). */
typedef struct cpmp_diag {
    double mass;          /* FP64 sum of rho over fluid nodes */
    double max_speed;     /* max |MV| over fluid nodes, MV = u + F / (2 rho) of the
                             state the last step collided (the reference's MV array,
                             written by its collide kernel; 0 before the first step) */
    int nonfinite;        /* 1 if any fluid density is NaN or negative */
    double ca_left, ca_right, ca_cap; /* contact angles (degrees), slice j = DY/2 */
    double x_left, x_right;           /* contact-line positions */
    double cap_h, cap_l;              /* spherical-cap height and base */
    double lap_r;         /* droplet radius from the mid-density crossing along y */
    double lap_dp;        /* EOS pressure jump p(inside) - p(outside) */
    double lap_sigma;     /* K^2 * dp * R / 2 */
    long long step;       /* steps taken since cpmp_init_droplet */
} cpmp_diag;

typedef struct cpmp_handle cpmp_handle;

/* Fills the reference's defaults: Initialize() + CONTACTANGLE, five-point
 * Laplacian, complex wall (FluidCuda.cu:1-7, 119-163); grid 64^3, FP32
 * storage, PLAIN scheme, device 0. */
void cpmp_params_default(cpmp_params *p);

/* Replaces SetMultiphase + CudaInitialize (FluidCuda.cu:1314-1437): derives
 * A, B, Tc, Rc and T, resolves the coexistence densities, allocates every
 * field on the device and uploads the parameters. */
cpmp_status cpmp_create(const cpmp_params *p, cpmp_handle **out);

/* Replaces CudaFree (FluidCuda.cu:1463-1485). */
void cpmp_destroy(cpmp_handle *h);

/* Replaces the SetFlowField launch (FluidCuda.cu:1262). */
cpmp_status cpmp_init_droplet(cpmp_handle *h, const cpmp_droplet *d);

/* Replaces cudaMemcpyToSymbol(_BasePt) in the BasePt sweep
 * (FluidCuda.cu:1264-1268); resets every wall column to this value. */
cpmp_status cpmp_set_base_pt(cpmp_handle *h, double base_pt);

/* Spatially varying wall chemical potential: 2*DX*DY values, bottom wall
 * (k < 3) then top wall (k > DZ-4), column index i*DY + j.  Generalises the
 * scalar _BasePt of ChemBoundary (FluidCuda.cu:387). */
cpmp_status cpmp_set_wall_field(cpmp_handle *h, const double *host, size_t count);

/* Replaces nsteps iterations of the step loop body (FluidCuda.cu:1277-1292):
 * ChemBoundary, ChemPotential, NonidealForce, GlobalCollide, swap,
 * MacroCalculate.  Asynchronous on the handle's stream (launch errors are
 * reported here, execution errors by the next synchronising call). */
cpmp_status cpmp_step(cpmp_handle *h, int nsteps);

/* Waits for the handle's stream. */
cpmp_status cpmp_sync(cpmp_handle *h);

/* Device-to-host copy of one field (replaces the host reads of unified
 * memory, e.g. FluidCuda.cu:563, 1626-1657).  dtype CPMP_F64 or CPMP_F32
 * (TYPE is always bytes); bytes must equal the field size exactly. */
cpmp_status cpmp_get_field(cpmp_handle *h, cpmp_field f, int dtype, void *host_dst, size_t bytes);

/* Host-to-device copy of RHO, U or DIST (seeded states for parity runs).
 * Setting DIST also recomputes RHO and U from it on fluid nodes; on the
 * FUSED scheme a page-locked host_src is read by the encode kernels in place
 * (no device staging copy). */
cpmp_status cpmp_set_field(cpmp_handle *h, cpmp_field f, int dtype, const void *host_src,
                           size_t bytes);

/* Device reductions: CalcMacroCPU (mass, max|MV|, non-finite flag),
 * ContactAngle(0, DY/2) and the Laplace probe.  Returns CPMP_ERR_NONFINITE
 * (with *out filled) when a fluid density is NaN or negative, the condition
 * on which the reference stops (FluidCuda.cu:1632-1646). */
cpmp_status cpmp_reduce(cpmp_handle *h, cpmp_diag *out);

/* Droplet-impact diagnostics (FP64 device sums, deterministic order).
 * "Liquid" means rho > (rho_g + rho_l)/2; MV is the physical velocity. */
typedef struct cpmp_impact {
    /* ComputeEnergy (FluidCuda.cu:737-787): fluid liquid nodes with
     * 2 <= i < DX-2, 2 <= j < DY-2, 2 <= k < DZ-2 */
    double v, v_xy, v_z;            /* sum |MV|, |MV_xy|, MV_z */
    double mv, mv_xy, mv_z;         /* the same weighted by rho */
    double energy, energy_xy, energy_z; /* sum rho |MV|^2 / 2, xy part, z part */
    /* Computetangential_velocity (FluidCuda.cu:790-898): same nodes; the
     * velocity along the azimuth about (DX/2, DY/2), and weighted by rho */
    double tangential, m_tangential;
    /* SaveSpreadtime (FluidCuda.cu:1128-1150): every liquid node with
     * 2 <= k < DZ-2; drop_velocity = drop_momentum / drop_mass */
    double drop_momentum, drop_mass, drop_velocity;
} cpmp_impact;
cpmp_status cpmp_impact_diag(cpmp_handle *h, cpmp_impact *out);

/* Coexistence densities (lattice units) the handle resolved, and the EOS
 * constants it derived (SetMultiphase, FluidCuda.cu:1318-1384). */
cpmp_status cpmp_get_eos(cpmp_handle *h, double *den_g, double *den_l, double *A, double *B,
                         double *T, double *Rc);

/* Stand-alone SetMultiphase: EOS constants and coexistence densities for a
 * model and T/Tc (cocurve_dir NULL: built-in Maxwell construction). */
cpmp_status cpmp_coexistence(int model, double tr, double eos_a, double eos_b, double eos_omega,
                             const char *cocurve_dir, double *den_g, double *den_l, double *A,
                             double *B, double *Tc, double *Rc);

/* Tile autotuner for the FUSED scheme (no reference counterpart: the
 * reference's launch shape is fixed at 64-thread 1-D blocks, FluidCuda.cu:113).
 * Times every instantiated (TY, TZ) column tile and x-march length on a scratch
 * copy of the current state (the state itself is not advanced) and keeps the
 * fastest for subsequent steps.  Outputs may be NULL.  PLAIN handles return
 * CPMP_OK without change. */
cpmp_status cpmp_autotune(cpmp_handle *h, int *tile_y, int *tile_z, int *march_x, double *ms_per_step);

/* Sets the FUSED kernel's column tile (tile_y x tile_z nodes) and x-march
 * length explicitly (no reference counterpart).  CPMP_ERR_UNSUPPORTED when the
 * tile is not instantiated or does not fit the device's shared memory. */
cpmp_status cpmp_set_tile(cpmp_handle *h, int tile_y, int tile_z, int march_x);
/* As cpmp_set_tile with the nodes each thread owns: 1, or 2 for the paired
 * kernel (two z-adjacent nodes per thread, paired FP32 instructions; same
 * results bit for bit).  cpmp_set_tile is nodes_per_thread = 1. */
cpmp_status cpmp_set_tile_ex(cpmp_handle *h, int tile_y, int tile_z, int march_x, int nodes_per_thread);
/* The tile in use (after cpmp_autotune: the one it kept).  Outputs may be NULL. */
cpmp_status cpmp_get_tile(cpmp_handle *h, int *tile_y, int *tile_z, int *march_x, int *nodes_per_thread);

/* Step forms of the FUSED scheme (no reference counterpart: the reference
 * always runs ChemPotential, NonidealForce and GlobalCollide as separate
 * kernels, FluidCuda.cu:1277-1292).  Both forms give the same results bit for
 * bit.
 *   CPMP_FORM_ONE_PASS  mu, the force, the collision and the A-A streaming of
 *                       a node in one kernel (the column tile is that kernel's);
 *   CPMP_FORM_TWO_PASS  a force pass (mu and F on a shared-memory column tile,
 *                       written to an FP32 field of 12 bytes per node, 24 with
 *                       the K1/K2 term) and a collide-stream pass without
 *                       shared memory; node pairs (nodes_per_thread 2), DZ a
 *                       multiple of 4, the column tile is the force pass's.
 * cpmp_autotune times the one-pass tiles only (the two-pass form is slower in
 * steady state on every workload measured); cpmp_set_tile_ex selects the
 * one-pass form. */
enum { CPMP_FORM_ONE_PASS = 0, CPMP_FORM_TWO_PASS = 1 };
cpmp_status cpmp_set_tile_form(cpmp_handle *h, int tile_y, int tile_z, int march_x, int nodes_per_thread,
                               int form);
cpmp_status cpmp_get_form(cpmp_handle *h, int *form);

/* The CUDA stream the handle launches on (cudaStream_t). */
void *cpmp_stream(cpmp_handle *h);

/* Per-kernel timing for roofline reporting: while enabled, every kernel
 * launch of cpmp_step is bracketed by CUDA events on the handle's stream and
 * its duration accumulated by kernel class.  cpmp_kernel_times returns, for
 * up to `cap` classes, the class name, launch count and total milliseconds;
 * the return value is the number of classes. */
cpmp_status cpmp_set_kernel_timing(cpmp_handle *h, int on);
int cpmp_kernel_times(cpmp_handle *h, const char **names, long long *launches, double *ms, int cap);

/* Number of the library's own kernel launches issued so far by this handle. */
long long cpmp_launch_count(cpmp_handle *h);

/* ---- Tecplot output --------------------------------------------------------
 * The reference's on-disk output format: Tecplot binary "#!TDV112", one
 * ordered zone (ordered_tec.cpp:674-717, 990-1147). */
enum { CPMP_TEC_FLOAT = 1, CPMP_TEC_DOUBLE = 2, CPMP_TEC_INT32 = 3, CPMP_TEC_INT16 = 4, CPMP_TEC_BYTE = 5 };
/* Layouts of cpmp_write_tecplot: SaveTask (FluidCuda.cu:901-927): variables
 * i, j, k (int16) and Density (double) on the grid decimated by `decimate`,
 * I = z fastest; SaveAllByType (FluidCuda.cu:1032-1092): i, j, k, Ux, Uy, Uz
 * (physical velocity where rho >= (rho_g + rho_l)/2, else -2) and Density,
 * all double, x fastest. */
enum { CPMP_TEC_SAVETASK = 0, CPMP_TEC_ALLBYTYPE = 1 };
/* flags: sample the density like the reference's CompressField, which
 * strides the flat node index instead of each axis (FluidCuda.cu:470). */
enum { CPMP_TEC_REFERENCE_STRIDE = 1 };

/* Writes one ordered zone of nvar variables (types CPMP_TEC_*, each
 * imax*jmax*kmax values, I fastest) to `path`.  Host only; needs no GPU. */
cpmp_status cpmp_tecplot_write(const char *path, const char *title, const char *zone_name, int nvar,
                               const char *const *names, const int *types, const void *const *data,
                               int imax, int jmax, int kmax);
/* Writes the handle's current fields in one of the reference's layouts; the
 * zone is named after the file (path without directory and ".plt").  A
 * decimated extent of 0 (DY < decimate) is written as 1, where the reference
 * writer throws.  vel_scale multiplies the ALLBYTYPE velocities: the
 * reference's DimV = DimLen / DimTime from DimConversion (FluidCuda.cu:474-486;
 * 1 keeps lattice units, and the reference's default Diameter = 0 makes it
 * NaN). */
cpmp_status cpmp_write_tecplot(cpmp_handle *h, const char *path, int layout, int decimate, int flags,
                               double vel_scale);
/* Grid dimensions of a handle: dims[3] = DX, DY, DZ. */
cpmp_status cpmp_get_dims(cpmp_handle *h, int *dims);

/* ---- Adjoint ---------------------------------------------------------------
 * No reference counterpart.  Sets kappa (Ka) of a handle (e.g. between
 * gradient evaluations); the next step uses it. */
cpmp_status cpmp_set_kappa(cpmp_handle *h, double ka);

/* Gradient of J = sum over fluid nodes of (rho^T - target)^2, rho^T the
 * density after `steps` steps from the handle's current state, with respect
 * to the wall chemical potential (2*DX*DY values, layout of
 * cpmp_set_wall_field) and kappa.  PLAIN scheme (FP32 or FP64), K1 = K2 = 0.
 * Runs the forward with a checkpoint of (f, rho, u) every checkpoint_every
 * steps (<= 0: ceil(sqrt(steps))), then the reverse sweep segment by segment,
 * replaying each segment's forward from its checkpoint.  The handle's state
 * is left at step `steps`.  target_rho: N host doubles; grad_wall: 2*DX*DY
 * host doubles (may be NULL); loss, grad_kappa: host scalars (may be NULL). */
cpmp_status cpmp_adjoint(cpmp_handle *h, int steps, int checkpoint_every, const double *target_rho,
                         double *loss, double *grad_wall, double *grad_kappa);

/* ---- Batches: many independent boxes stepped by one persistent launch ----
 * No reference counterpart (the reference runs one box per process).  All
 * boxes use the FUSED scheme and share storage, lap_order, wall_mode,
 * complex_bc and device; grid, EOS model, T/Tc, K, kappa, rates and wall
 * potential may differ per box.  Each time step is one batched wall pass
 * (the three wall layers of every box), ONE persistent fused-collide launch
 * whose CTAs take (box, tile, x-chunk) work items from a device counter until
 * none are left, and one batched density pass; cpmp_batch_step replays two
 * steps as a CUDA graph. */
typedef struct cpmp_batch cpmp_batch;

/* Creates count boxes from params[count] (every box an ordinary handle that
 * shares the batch's stream). */
cpmp_status cpmp_batch_create(const cpmp_params *params, int count, cpmp_batch **out);
/* Box `index` as a handle for cpmp_init_droplet, cpmp_set_base_pt,
 * cpmp_set_wall_field, cpmp_get_field, cpmp_set_field, cpmp_reduce.  The batch
 * owns it: do not cpmp_destroy or cpmp_step it (cpmp_step returns
 * CPMP_ERR_PARAM for batch boxes). */
cpmp_status cpmp_batch_handle(cpmp_batch *b, int index, cpmp_handle **h);
int cpmp_batch_count(cpmp_batch *b);
long long cpmp_batch_nodes(cpmp_batch *b);   /* total lattice nodes of all boxes */
/* nsteps time steps of every box (asynchronous on the batch stream). */
cpmp_status cpmp_batch_step(cpmp_batch *b, int nsteps);
cpmp_status cpmp_batch_sync(cpmp_batch *b);
/* cpmp_reduce of every box (out[count], count = the number of boxes), in
 * four launches for the whole batch and one wait: each out[i] equals what
 * cpmp_reduce on box i returns, bit for bit.  Returns CPMP_ERR_NONFINITE (with
 * every out[i] filled) when any box has a NaN or negative fluid density; the
 * error message names the first such box. */
cpmp_status cpmp_batch_reduce(cpmp_batch *b, cpmp_diag *out, int count);
/* Tile shape / x-march shared by all boxes; the autotuner times the
 * candidates on scratch copies of every box (the state is not advanced). */
cpmp_status cpmp_batch_set_tile(cpmp_batch *b, int tile_y, int tile_z, int march_x);
cpmp_status cpmp_batch_set_tile_ex(cpmp_batch *b, int tile_y, int tile_z, int march_x, int nodes_per_thread);
cpmp_status cpmp_batch_get_tile(cpmp_batch *b, int *tile_y, int *tile_z, int *march_x, int *nodes_per_thread);
cpmp_status cpmp_batch_autotune(cpmp_batch *b, int *tile_y, int *tile_z, int *march_x, double *ms_per_step);
cpmp_status cpmp_batch_set_kernel_timing(cpmp_batch *b, int on);
int cpmp_batch_kernel_times(cpmp_batch *b, const char **names, long long *launches, double *ms, int cap);
long long cpmp_batch_launch_count(cpmp_batch *b);
void *cpmp_batch_stream(cpmp_batch *b);
void cpmp_batch_destroy(cpmp_batch *b);

/* Largest node count cpmp_mass_noalloc accepts (the library's grid limit). */
#define CPMP_NOALLOC_MAX_NODES (1LL << 34)

/* Mass / max-speed / non-finite reduction that allocates nothing.  No
 * counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc -- code running inside a host or framework that owns device
 * memory, or stream-ordered pipelines where an allocation would synchronise
 * the device -- and that hold the fields themselves: type (N bytes, FLUID =
 * 1), rho (N floats) and, optionally, mv (3N floats, x then y then z blocks),
 * all device pointers in the reference's node layout.  It launches on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) and writes three
 * doubles to the device pointer `out`: the FP64 sum of rho over fluid nodes,
 * max |mv| over fluid nodes (0 when mv is NULL) and 1.0 if a fluid density is
 * NaN or negative (else 0.0).  Mass and the non-finite flag are the same
 * deterministic reduction, in the same order, as cpmp_reduce; so is max |mv|
 * given the PLAIN scheme's MV field (the FUSED scheme's cpmp_reduce takes max
 * |MV| from its collide kernel instead of from a field).  Its block partials
 * live in a fixed 24 KB device array inside the library (1024 partial
 * triples; every GPU that loads the library holds it until the process
 * exits), so every n from 1 to CPMP_NOALLOC_MAX_NODES fits and larger n is
 * rejected with CPMP_ERR_SIZE.  The first call on a device looks up that
 * array's device address there (cudaGetSymbolAddress, no allocation), with
 * that device current; make that first call before any stream capture.  Later
 * calls look the address up again, so a device reset between calls is
 * harmless.  All calls share the array: calls that overlap on the GPU (e.g. on two
 * streams at once) race and give wrong results; each call writes every
 * partial it reads, so nothing carries over between calls that follow one
 * another. */
cpmp_status cpmp_mass_noalloc(const uint8_t *type, const float *rho, const float *mv, long long n,
                              void *stream, double *out);

/* Message of the last failed call on this thread ("" if none). */
const char *cpmp_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* CPMP_H */
