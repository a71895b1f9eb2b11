// api.cpp -- the C ABI (include/cpmp.h): handle life cycle, parameter
// derivation, device memory, step dispatch (with CUDA-graph replay), field
// transfer and reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cpmp.h"
#include "eos.h"
#include "kernels.h"

using namespace cpmp;

namespace {

thread_local std::string g_err;

cpmp_status fail(cpmp_status s, const std::string &msg)
{
    g_err = msg;
    return s;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(CPMP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
    } while (0)

}  // namespace

struct cpmp_handle {
    cpmp_params p{};
    std::string cocurve;
    int eos = 0;
    double A = 0, B = 0, Tc = 0, Rc = 0, T = 0, den_g = 0, den_l = 0;
    double ts[CPMP_Q] = {0};
    long long n = 0;
    cudaStream_t st = nullptr;
    bool plain = true;
    bool f64 = false;  // PLAIN with FP64 storage/arithmetic
    uint8_t *type = nullptr;
    void *rho = nullptr, *mu = nullptr, *u = nullptr, *mv = nullptr, *F = nullptr;
    void *rho2 = nullptr;  // FUSED: next step's density (swapped with rho every step)
    void *fb[2] = {nullptr, nullptr};
    int cur = 0;
    void *h = nullptr;
    float *f0[2] = {nullptr, nullptr};
    void *wall = nullptr;
    double *partials = nullptr, *dout = nullptr;
    double *impact_partials = nullptr;  // allocated by the first cpmp_impact_diag
    // FUSED: max |MV|^2 of the last collision at each parity (float bits),
    // sdiag[P * sdiag_stride]; a batch box points into its batch's array
    unsigned *sdiag = nullptr;
    int sdiag_stride = 1;
    bool sdiag_owned = true;
    // FUSED: error word of the collide's bounded waits (non-zero: gave up)
    unsigned *kerr = nullptr;
    long long step = 0;
    bool initialised = false;
    std::unique_ptr<LaunchHook> hook;
    bool timing = false;
    long long launches = 0;
    FusedTile tile{8, 32, 16};
    cudaGraphExec_t gexec = nullptr;
    int gsteps = 0;
    int launches_per_step = 0;
    bool in_batch = false;       // stepped by its cpmp_batch, on the batch's stream
};

struct cpmp_batch {
    std::vector<cpmp_handle *> boxes;
    cudaStream_t st = nullptr;
    int device = 0, storage = 0, lap_order = 5, wall_mode = 1, complex_bc = 1;
    FusedTile tile{8, 32, 16};
    KParams<float> *d_params = nullptr;
    BatchBox *d_boxes = nullptr;
    unsigned *d_counter = nullptr;
    unsigned *d_mvmax = nullptr;  // [2][boxes]: each box's max |MV|^2 of its last collision, per parity
    DiagBox *d_diag = nullptr;    // [boxes]: the batched diagnostics' box table
    double *d_dout = nullptr;     // [boxes][kDiagStride]: their results
    long long total_items = 0, nodes = 0, wall_blocks = 0, density_blocks = 0, mass_blocks = 0, launches = 0;
    bool ref_rates = false;       // every box's rates follow the reference's pattern
    cudaGraphExec_t gexec = nullptr;
    std::unique_ptr<LaunchHook> hook;
    bool timing = false;
};

namespace {

size_t real_size(const cpmp_handle *h) { return h->f64 ? sizeof(double) : sizeof(float); }

template <class R>
KParams<R> make_kparams(const cpmp_handle *h)
{
    KParams<R> k{};
    k.dx = h->p.dx;
    k.dy = h->p.dy;
    k.dz = h->p.dz;
    k.n = h->n;
    k.wall_mode = h->p.wall_mode;
    k.eos = h->eos;
    k.lap_order = h->p.lap_order;
    k.complex_bc = h->p.complex_bc;
    k.qp = (h->p.k1 != 0.0 || h->p.k2 != 0.0) ? 1 : 0;
    k.kk = (R)(h->p.k * h->p.k);
    k.A = (R)h->A;
    k.B = (R)h->B;
    k.T = (R)h->T;
    k.ka = (R)h->p.ka;
    k.k1 = (R)h->p.k1;
    k.k2 = (R)h->p.k2;
    for (int q = 0; q < CPMP_Q; ++q) {
        k.ts[q] = (R)h->ts[q];
        k.omts[q] = (R)(1.0 - h->ts[q]);
    }
    k.wall = (const R *)h->wall;
    k.mvmax = h->sdiag;
    k.mvmax_stride = h->sdiag_stride;
    k.err = h->kerr;
    return k;
}

void free_all(cpmp_handle *h)
{
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    void *ptrs[] = {h->type, h->rho, h->rho2, h->mu, h->u, h->mv, h->F, h->fb[0], h->fb[1], h->h, h->f0[0], h->f0[1],
                    h->wall, h->partials, h->dout, h->impact_partials};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (h->sdiag && h->sdiag_owned) cudaFree(h->sdiag);
    h->sdiag = nullptr;
    if (h->kerr) cudaFree(h->kerr);
    h->kerr = nullptr;
    h->type = nullptr;
    h->rho = h->rho2 = h->mu = h->u = h->mv = h->F = h->fb[0] = h->fb[1] = h->h = h->wall = nullptr;
    h->f0[0] = h->f0[1] = nullptr;
    h->partials = h->dout = h->impact_partials = nullptr;
    if (h->st) cudaStreamDestroy(h->st);
    h->st = nullptr;
}

cpmp_status dalloc(void **ptr, size_t bytes, const char *what)
{
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(CPMP_ERR_NOMEM, std::string("cudaMalloc(") + what + ", " + std::to_string(bytes) +
                                        " bytes): " + cudaGetErrorString(e));
    }
    return CPMP_OK;
}

// The two-pass form's force field (FUSED scheme; the PLAIN scheme's F is its
// own field), allocated when that form is first selected: 3 floats per node,
// 6 with the K1/K2 term (grad rho).
size_t force_field_bytes(const cpmp_handle *h)
{
    return ((h->p.k1 != 0.0 || h->p.k2 != 0.0) ? 6 : 3) * (size_t)h->n * sizeof(float);
}
cpmp_status ensure_force_field(cpmp_handle *h)
{
    if (h->plain || h->F) return CPMP_OK;
    return dalloc(&h->F, force_field_bytes(h), "F");
}

// Heuristic default tile for the fused kernel (the autotuner refines it):
// the paired kernel where the grid allows it.
FusedTile default_tile(const cpmp_params &p)
{
    int ty = 8, tz = 32, np = 1;
    if (p.dy < 8) { ty = 4; tz = 32; }
    if (p.dz <= 16) { ty = p.dy < 16 ? 8 : 16; tz = 16; }
    if (pair_grid_ok(p.dz)) {
        np = 2;
        ty = 8;
        tz = p.dz > 32 ? 64 : 32;
    }
    const long long tiles = (long long)((p.dz + tz - 1) / tz) * ((p.dy + ty - 1) / ty);
    // aim for >= 4 CTAs per SM on a 152-SM part, but march at least 8 planes
    long long xl = (long long)p.dx * tiles / (4 * 152);
    xl = std::max<long long>(8, std::min<long long>(64, xl));
    xl = std::min<long long>(xl, p.dx);
    return FusedTile{ty, tz, (int)xl, np};
}

cpmp_status upload_wall(cpmp_handle *h, const std::vector<double> &w)
{
    const size_t cnt = w.size();
    if (h->f64) {
        CK(cudaMemcpyAsync(h->wall, w.data(), cnt * sizeof(double), cudaMemcpyHostToDevice, h->st));
    } else {
        std::vector<float> tmp(cnt);
        for (size_t i = 0; i < cnt; ++i) tmp[i] = (float)w[i];
        CK(cudaMemcpyAsync(h->wall, tmp.data(), cnt * sizeof(float), cudaMemcpyHostToDevice, h->st));
        CK(cudaStreamSynchronize(h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    return CPMP_OK;
}

// kernel launches of one time step (the two-pass form adds its force pass)
long long step_launches(const cpmp_handle *h)
{
    return h->launches_per_step + ((!h->plain && h->tile.form == 1) ? 1 : 0);
}

// one time step, launched directly (no graph)
void launch_one_step(cpmp_handle *h, LaunchHook *hook)
{
    if (h->plain) {
        if (h->f64) {
            auto k = make_kparams<double>(h);
            plain_launch_step<double, double>(k, h->type, (double *)h->rho, (double *)h->mu, (double *)h->u,
                                              (double *)h->F, (double *)h->mv, (const double *)h->fb[h->cur],
                                              (double *)h->fb[1 - h->cur], h->st, hook);
        } else {
            auto k = make_kparams<float>(h);
            plain_launch_step<float, float>(k, h->type, (float *)h->rho, (float *)h->mu, (float *)h->u,
                                            (float *)h->F, (float *)h->mv, (const float *)h->fb[h->cur],
                                            (float *)h->fb[1 - h->cur], h->st, hook);
        }
        h->cur ^= 1;
    } else {
        auto k = make_kparams<float>(h);
        const int P = (int)(h->step & 1);
        if (h->sdiag) cudaMemsetAsync(h->sdiag + P * h->sdiag_stride, 0, sizeof(unsigned), h->st);
        fused_launch_wall(k, (float *)h->rho, (float *)h->rho2, h->st, hook);
        fused_launch_collide(h->p.storage, k, P, h->tile, h->h, h->f0[P], h->f0[1 - P], (const float *)h->rho,
                             (float *)h->F,
                             h->st, hook);
        fused_launch_density(h->p.storage, k, 1 - P, h->h, h->f0[1 - P], (float *)h->rho2, h->st, hook);
        std::swap(h->rho, h->rho2);
    }
    h->step += 1;
    h->launches += step_launches(h);
}

bool step_parity_even(const cpmp_handle *h) { return h->plain ? h->cur == 0 : (h->step & 1) == 0; }

cpmp_status ensure_graph(cpmp_handle *h)
{
    if (h->gexec) return CPMP_OK;
    // a two-step graph starting at even parity
    cudaGraph_t g = nullptr;
    const long long save_step = h->step, save_launch = h->launches;
    const int save_cur = h->cur;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    launch_one_step(h, nullptr);
    launch_one_step(h, nullptr);
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    h->step = save_step;
    h->launches = save_launch;
    h->cur = save_cur;
    if (e != cudaSuccess) return fail(CPMP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        h->gexec = nullptr;
        return fail(CPMP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    return CPMP_OK;
}

template <class T>
void convert_copy(const T *src, void *dst, int dtype, size_t cnt)
{
    if (dtype == CPMP_F64) {
        double *d = (double *)dst;
        for (size_t i = 0; i < cnt; ++i) d[i] = (double)src[i];
    } else {
        float *d = (float *)dst;
        for (size_t i = 0; i < cnt; ++i) d[i] = (float)src[i];
    }
}

// Device buffer of `cnt` reals (the handle's real type) to host, converting.
cpmp_status d2h_real(cpmp_handle *h, const void *dsrc, size_t cnt, int dtype, void *hdst)
{
    const bool native = (h->f64 && dtype == CPMP_F64) || (!h->f64 && dtype == CPMP_F32);
    if (native) {
        CK(cudaMemcpyAsync(hdst, dsrc, cnt * real_size(h), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        return CPMP_OK;
    }
    std::vector<unsigned char> tmp(cnt * real_size(h));
    CK(cudaMemcpyAsync(tmp.data(), dsrc, tmp.size(), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (h->f64)
        convert_copy((const double *)tmp.data(), hdst, dtype, cnt);
    else
        convert_copy((const float *)tmp.data(), hdst, dtype, cnt);
    return CPMP_OK;
}

cpmp_status h2d_real(cpmp_handle *h, void *ddst, size_t cnt, int dtype, const void *hsrc)
{
    const bool native = (h->f64 && dtype == CPMP_F64) || (!h->f64 && dtype == CPMP_F32);
    if (native) {
        CK(cudaMemcpyAsync(ddst, hsrc, cnt * real_size(h), cudaMemcpyHostToDevice, h->st));
        CK(cudaStreamSynchronize(h->st));
        return CPMP_OK;
    }
    std::vector<unsigned char> tmp(cnt * real_size(h));
    if (h->f64) {
        double *d = (double *)tmp.data();
        for (size_t i = 0; i < cnt; ++i) d[i] = ((const float *)hsrc)[i];
    } else {
        float *d = (float *)tmp.data();
        for (size_t i = 0; i < cnt; ++i) d[i] = (float)((const double *)hsrc)[i];
    }
    CK(cudaMemcpyAsync(ddst, tmp.data(), tmp.size(), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return CPMP_OK;
}

// FUSED scheme: evaluate mu, F, u and mv of the current state into the
// (lazily allocated) diagnostic buffers.
cpmp_status fused_diag_fields(cpmp_handle *h)
{
    const size_t n = (size_t)h->n;
    cpmp_status s;
    if (!h->mu && (s = dalloc(&h->mu, n * sizeof(float), "mu")) != CPMP_OK) return s;
    if (!h->F && (s = dalloc(&h->F, 3 * n * sizeof(float), "F")) != CPMP_OK) return s;
    if (!h->u && (s = dalloc(&h->u, 3 * n * sizeof(float), "u")) != CPMP_OK) return s;
    if (!h->mv && (s = dalloc(&h->mv, 3 * n * sizeof(float), "mv")) != CPMP_OK) return s;
    CK(cudaMemsetAsync(h->mu, 0, n * sizeof(float), h->st));
    CK(cudaMemsetAsync(h->F, 0, 3 * n * sizeof(float), h->st));
    CK(cudaMemsetAsync(h->u, 0, 3 * n * sizeof(float), h->st));
    CK(cudaMemsetAsync(h->mv, 0, 3 * n * sizeof(float), h->st));
    auto k = make_kparams<float>(h);
    const int P = (int)(h->step & 1);
    plain_launch_mu_force<float>(k, h->type, (float *)h->rho, (float *)h->mu, (float *)h->F, h->st, nullptr);
    fused_launch_velocity(h->p.storage, k, P, h->h, h->f0[P], (const float *)h->rho, (float *)h->u, h->st);
    diag_launch_mv(h->type, (const float *)h->rho, (const float *)h->u, (const float *)h->F, (float *)h->mv,
                   h->n, h->st);
    h->launches += (h->p.wall_mode == 1 ? (h->p.complex_bc ? 3 : 1) : 0) + 4;
    CK(cudaGetLastError());
    return CPMP_OK;
}

}  // namespace

extern "C" {

const char *cpmp_last_error(void) { return g_err.c_str(); }

void cpmp_internal_set_error(const char *msg) { g_err = msg ? msg : ""; }

void cpmp_params_default(cpmp_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->dx = p->dy = p->dz = 64;
    p->model = CPMP_MP_CPPRW;
    p->tr = 0.7;
    p->k = 0.2;
    p->ka = 0.001;
    p->k1 = 0.0;
    p->k2 = 0.0;
    p->tau = 0.8;
    p->ts_from_tau = 1;
    p->base_pt = -0.08;
    p->wall_mode = CPMP_WALL_Z;
    p->lap_order = 5;
    p->complex_bc = 1;
    p->storage = CPMP_STORE_F32;
    p->scheme = CPMP_SCHEME_PLAIN;
    p->device = 0;
}

cpmp_status cpmp_coexistence(int model, double tr, double eos_a, double eos_b, double eos_omega,
                             const char *cocurve_dir, double *den_g, double *den_l, double *A, double *B,
                             double *Tc, double *Rc)
{
    double a, b, tc, rc;
    if (!eos_constants(model, tr, eos_a, eos_b, eos_omega, &a, &b, &tc, &rc))
        return fail(CPMP_ERR_PARAM, "unsupported model id " + std::to_string(model) +
                                        " (chemical-potential models 201..206)");
    if (!(tr > 0.0 && tr < 1.0)) return fail(CPMP_ERR_PARAM, "T/Tc must lie in (0, 1)");
    double g = 0, l = 0;
    if (cocurve_dir) {
        const int r = read_cocurve(cocurve_dir, model, tr, &g, &l);
        if (r != 0)
            return fail(CPMP_ERR_COCURVE, std::string("CoCurve table ") + (r == -2 ? "not found" : "has no row") +
                                              " for T/Tc=" + std::to_string(tr) + " in " + cocurve_dir);
        g *= rc;
        l *= rc;
    } else {
        if (maxwell(eos_of_model(model), a, b, tr * tc, &g, &l) != 0)
            return fail(CPMP_ERR_PARAM, "no coexistence at this temperature");
    }
    if (den_g) *den_g = g;
    if (den_l) *den_l = l;
    if (A) *A = a;
    if (B) *B = b;
    if (Tc) *Tc = tc;
    if (Rc) *Rc = rc;
    return CPMP_OK;
}

cpmp_status cpmp_create(const cpmp_params *pin, cpmp_handle **out)
{
    if (!pin || !out) return fail(CPMP_ERR_PARAM, "null argument");
    *out = nullptr;
    const cpmp_params &p = *pin;
    if (p.dx < 1 || p.dy < 1 || p.dz < 1) return fail(CPMP_ERR_PARAM, "grid dimensions must be positive");
    if ((long long)p.dx * p.dy * p.dz > (1LL << 34)) return fail(CPMP_ERR_PARAM, "grid too large");
    if (p.wall_mode != CPMP_WALL_NONE && p.wall_mode != CPMP_WALL_Z) return fail(CPMP_ERR_PARAM, "wall_mode");
    if (p.wall_mode == CPMP_WALL_Z && p.dz < 8) return fail(CPMP_ERR_PARAM, "walled box needs dz >= 8");
    if (p.lap_order != 5 && p.lap_order != 7) return fail(CPMP_ERR_PARAM, "lap_order must be 5 or 7");
    if (p.scheme == CPMP_SCHEME_PLAIN && p.storage != CPMP_STORE_F32 && p.storage != CPMP_STORE_F64)
        return fail(CPMP_ERR_UNSUPPORTED, "PLAIN scheme stores FP32 or FP64 populations");
    if (p.scheme == CPMP_SCHEME_FUSED && (long long)p.dx * p.dy * p.dz >= (1LL << 32))
        return fail(CPMP_ERR_UNSUPPORTED, "the FUSED scheme indexes nodes with 32 bits: N must be below 2^32");
    if (p.scheme == CPMP_SCHEME_FUSED && p.storage == CPMP_STORE_F64)
        return fail(CPMP_ERR_UNSUPPORTED, "FUSED scheme stores FP32, FP16 or BF16 populations");
    if (p.scheme != CPMP_SCHEME_PLAIN && p.scheme != CPMP_SCHEME_FUSED) return fail(CPMP_ERR_PARAM, "scheme");
    if (!(p.tau > 0.5)) return fail(CPMP_ERR_PARAM, "tau must exceed 0.5");

    std::unique_ptr<cpmp_handle> h(new cpmp_handle());
    h->p = p;
    if (p.cocurve_dir) {
        h->cocurve = p.cocurve_dir;
        h->p.cocurve_dir = h->cocurve.c_str();
    }
    h->eos = eos_of_model(p.model);
    if (h->eos < 0) return fail(CPMP_ERR_PARAM, "unsupported model id " + std::to_string(p.model));
    double g = 0, l = 0;
    cpmp_status s = cpmp_coexistence(p.model, p.tr, p.eos_a, p.eos_b, p.eos_omega,
                                     (p.den_g > 0 && p.den_l > 0) ? nullptr : h->p.cocurve_dir, &g, &l, &h->A,
                                     &h->B, &h->Tc, &h->Rc);
    if (s != CPMP_OK) return s;
    if (p.den_g > 0 && p.den_l > 0) {
        g = p.den_g;
        l = p.den_l;
    }
    h->den_g = g;
    h->den_l = l;
    h->T = p.tr * h->Tc;
    if (p.ts_from_tau) {
        for (int q = 0; q < CPMP_Q; ++q) h->ts[q] = 1.0;  // FluidCuda.cu:154-157
        h->ts[2] = h->ts[4] = h->ts[6] = h->ts[8] = 1.1;
        h->ts[9] = h->ts[11] = h->ts[13] = h->ts[14] = h->ts[15] = 1.0 / p.tau;
    } else {
        for (int q = 0; q < CPMP_Q; ++q) h->ts[q] = p.ts[q];
    }
    h->n = (long long)p.dx * p.dy * p.dz;
    h->plain = p.scheme == CPMP_SCHEME_PLAIN;
    h->f64 = h->plain && p.storage == CPMP_STORE_F64;
    const int wall_launches = p.wall_mode == CPMP_WALL_Z ? (p.complex_bc ? 3 : 1) : 0;
    h->launches_per_step = wall_launches + (h->plain ? 4 : 2);

    CK(cudaSetDevice(p.device));
    CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    const size_t n = (size_t)h->n, rs = real_size(h.get());
    const size_t np = (size_t)p.dx * p.dy;
    struct Guard {
        cpmp_handle *h;
        bool armed = true;
        ~Guard()
        {
            if (armed) free_all(h);
        }
    } guard{h.get()};
    if ((s = dalloc((void **)&h->type, n, "type")) != CPMP_OK) return s;
    if ((s = dalloc(&h->rho, n * rs, "rho")) != CPMP_OK) return s;
    if ((s = dalloc(&h->wall, 2 * np * rs, "wall")) != CPMP_OK) return s;
    if ((s = dalloc((void **)&h->partials, 3 * sizeof(double) * diag_partial_blocks(h->n), "partials")) != CPMP_OK)
        return s;
    if ((s = dalloc((void **)&h->dout, 32 * sizeof(double), "dout")) != CPMP_OK) return s;
    if (!h->plain) {
        if ((s = dalloc((void **)&h->sdiag, 2 * sizeof(unsigned), "mv max")) != CPMP_OK) return s;
        CK(cudaMemset(h->sdiag, 0, 2 * sizeof(unsigned)));
        if ((s = dalloc((void **)&h->kerr, sizeof(unsigned), "error word")) != CPMP_OK) return s;
        CK(cudaMemset(h->kerr, 0, sizeof(unsigned)));
    }
    if (h->plain) {
        if ((s = dalloc(&h->mu, n * rs, "mu")) != CPMP_OK) return s;
        if ((s = dalloc(&h->u, 3 * n * rs, "u")) != CPMP_OK) return s;
        if ((s = dalloc(&h->mv, 3 * n * rs, "mv")) != CPMP_OK) return s;
        if ((s = dalloc(&h->F, 3 * n * rs, "F")) != CPMP_OK) return s;
        if ((s = dalloc(&h->fb[0], CPMP_Q * n * rs, "f")) != CPMP_OK) return s;
        if ((s = dalloc(&h->fb[1], CPMP_Q * n * rs, "f")) != CPMP_OK) return s;
    } else {
        const size_t hs = p.storage == CPMP_STORE_F32 ? 4 : 2;
        if ((s = dalloc(&h->rho2, n * rs, "rho")) != CPMP_OK) return s;
        if ((s = dalloc(&h->h, (CPMP_Q - 1) * n * hs, "h")) != CPMP_OK) return s;
        if ((s = dalloc((void **)&h->f0[0], n * sizeof(float), "f0")) != CPMP_OK) return s;
        if ((s = dalloc((void **)&h->f0[1], n * sizeof(float), "f0")) != CPMP_OK) return s;
        CK(fused_setup_attributes());
        h->tile = default_tile(p);
        if (!fused_tile_usable(p.storage, p.lap_order, h->tile.ty, h->tile.tz, h->tile.np))
            h->tile = FusedTile{4, 32, h->tile.xl};
        if (!fused_tile_usable(p.storage, p.lap_order, h->tile.ty, h->tile.tz, h->tile.np))
            return fail(CPMP_ERR_UNSUPPORTED, "no fused tile fits this device's shared memory");
    }
    std::vector<double> w(2 * np, p.base_pt);
    if ((s = upload_wall(h.get(), w)) != CPMP_OK) return s;
    guard.armed = false;
    *out = h.release();
    return CPMP_OK;
}

void cpmp_destroy(cpmp_handle *h)
{
    if (!h) return;
    cudaSetDevice(h->p.device);
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->in_batch) h->st = nullptr;  // the batch owns the stream
    h->hook.reset();
    free_all(h);
    delete h;
}

cpmp_status cpmp_init_droplet(cpmp_handle *h, const cpmp_droplet *d)
{
    if (!h || !d) return fail(CPMP_ERR_PARAM, "null argument");
    if (!(d->width > 0)) return fail(CPMP_ERR_PARAM, "droplet width must be positive");
    CK(cudaSetDevice(h->p.device));
    DropletDev dd{d->cx, d->cy, d->cz, d->radius, d->width, h->den_g, h->den_l, d->ref_centre};
    const size_t n = (size_t)h->n, rs = real_size(h);
    if (h->plain) {
        CK(cudaMemsetAsync(h->F, 0, 3 * n * rs, h->st));
        CK(cudaMemsetAsync(h->mv, 0, 3 * n * rs, h->st));
        CK(cudaMemsetAsync(h->fb[1], 0, CPMP_Q * n * rs, h->st));
        if (h->f64)
            plain_launch_init<double, double>(make_kparams<double>(h), dd, h->type, (double *)h->rho,
                                              (double *)h->mu, (double *)h->u, (double *)h->fb[0], h->st);
        else
            plain_launch_init<float, float>(make_kparams<float>(h), dd, h->type, (float *)h->rho, (float *)h->mu,
                                            (float *)h->u, (float *)h->fb[0], h->st);
        h->cur = 0;
    } else {
        CK(cudaMemsetAsync(h->f0[1], 0, n * sizeof(float), h->st));
        fused_launch_init(h->p.storage, make_kparams<float>(h), dd, h->type, (float *)h->rho, h->f0[0], h->h,
                          h->st);
        CK(cudaMemcpyAsync(h->rho2, h->rho, n * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
    }
    h->launches += h->plain ? 1 : 2;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
    h->step = 0;
    h->initialised = true;
    return CPMP_OK;
}

cpmp_status cpmp_set_base_pt(cpmp_handle *h, double base_pt)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    CK(cudaSetDevice(h->p.device));
    h->p.base_pt = base_pt;
    std::vector<double> w(2 * (size_t)h->p.dx * h->p.dy, base_pt);
    return upload_wall(h, w);
}

cpmp_status cpmp_set_wall_field(cpmp_handle *h, const double *host, size_t count)
{
    if (!h || !host) return fail(CPMP_ERR_PARAM, "null argument");
    if (count != 2 * (size_t)h->p.dx * h->p.dy)
        return fail(CPMP_ERR_SIZE, "wall field needs 2*DX*DY values");
    CK(cudaSetDevice(h->p.device));
    std::vector<double> w(host, host + count);
    return upload_wall(h, w);
}

cpmp_status cpmp_step(cpmp_handle *h, int nsteps)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    if (nsteps < 0) return fail(CPMP_ERR_PARAM, "nsteps must be >= 0");
    if (!h->initialised) return fail(CPMP_ERR_PARAM, "cpmp_init_droplet or cpmp_set_field(DIST) first");
    if (h->in_batch) return fail(CPMP_ERR_PARAM, "boxes of a batch are stepped with cpmp_batch_step");
    CK(cudaSetDevice(h->p.device));
    LaunchHook *hook = h->timing ? h->hook.get() : nullptr;
    int left = nsteps;
    if (hook || nsteps < 2) {
        for (; left > 0; --left) launch_one_step(h, hook);
        CK(cudaGetLastError());
        return CPMP_OK;
    }
    if (!step_parity_even(h)) {
        launch_one_step(h, nullptr);
        --left;
    }
    if (left >= 2) {
        cpmp_status s = ensure_graph(h);
        if (s != CPMP_OK) return s;
        while (left >= 2) {
            CK(cudaGraphLaunch(h->gexec, h->st));
            h->step += 2;
            h->launches += 2LL * step_launches(h);
            left -= 2;  // two lattice swaps leave h->cur unchanged
        }
    }
    if (left == 1) launch_one_step(h, nullptr);
    CK(cudaGetLastError());
    return CPMP_OK;
}

cpmp_status cpmp_sync(cpmp_handle *h)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    CK(cudaSetDevice(h->p.device));
    CK(cudaStreamSynchronize(h->st));
    if (h->kerr) {
        unsigned e = 0;
        CK(cudaMemcpy(&e, h->kerr, sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (e) return fail(CPMP_ERR_TIMEOUT, "fused collide: a shared-memory copy did not complete in time");
    }
    return CPMP_OK;
}

cpmp_status cpmp_get_field(cpmp_handle *h, cpmp_field f, int dtype, void *dst, size_t bytes)
{
    if (!h || !dst) return fail(CPMP_ERR_PARAM, "null argument");
    CK(cudaSetDevice(h->p.device));
    const size_t n = (size_t)h->n;
    if (f == CPMP_FIELD_TYPE) {
        if (bytes != n) return fail(CPMP_ERR_SIZE, "TYPE needs N bytes");
        CK(cudaMemcpyAsync(dst, h->type, n, cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        return CPMP_OK;
    }
    if (dtype != CPMP_F64 && dtype != CPMP_F32) return fail(CPMP_ERR_PARAM, "dtype");
    const size_t es = dtype == CPMP_F64 ? 8 : 4;
    size_t comps;
    switch (f) {
    case CPMP_FIELD_RHO:
    case CPMP_FIELD_MU: comps = 1; break;
    case CPMP_FIELD_U:
    case CPMP_FIELD_MV:
    case CPMP_FIELD_FORCE: comps = 3; break;
    case CPMP_FIELD_DIST: comps = CPMP_Q; break;
    default: return fail(CPMP_ERR_PARAM, "unknown field");
    }
    if (bytes != comps * n * es) return fail(CPMP_ERR_SIZE, "buffer size does not match the field");
    CK(cudaStreamSynchronize(h->st));
    if (h->plain) {
        const void *src = f == CPMP_FIELD_RHO ? h->rho : f == CPMP_FIELD_MU ? h->mu : f == CPMP_FIELD_U ? h->u
                        : f == CPMP_FIELD_MV ? h->mv : f == CPMP_FIELD_FORCE ? h->F : h->fb[h->cur];
        return d2h_real(h, src, comps * n, dtype, dst);
    }
    // FUSED
    if (f == CPMP_FIELD_RHO) return d2h_real(h, h->rho, n, dtype, dst);
    if (f == CPMP_FIELD_DIST) {
        void *tmp = nullptr;
        cpmp_status s = dalloc(&tmp, CPMP_Q * n * es, "decode");
        if (s != CPMP_OK) return s;
        cudaMemsetAsync(tmp, 0, CPMP_Q * n * es, h->st);
        const int P = (int)(h->step & 1);
        fused_launch_decode(h->p.storage, make_kparams<float>(h), P, h->h, h->f0[P], tmp, dtype == CPMP_F64, h->st);
        h->launches += 1;
        cudaError_t e = cudaMemcpyAsync(dst, tmp, CPMP_Q * n * es, cudaMemcpyDeviceToHost, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        cudaFree(tmp);
        if (e != cudaSuccess) return fail(CPMP_ERR_CUDA, std::string("decode copy: ") + cudaGetErrorString(e));
        return CPMP_OK;
    }
    cpmp_status s = fused_diag_fields(h);
    if (s != CPMP_OK) return s;
    const void *src = f == CPMP_FIELD_MU ? h->mu : f == CPMP_FIELD_U ? h->u : f == CPMP_FIELD_MV ? h->mv : h->F;
    return d2h_real(h, src, comps * n, dtype, dst);
}

cpmp_status cpmp_set_field(cpmp_handle *h, cpmp_field f, int dtype, const void *src, size_t bytes)
{
    if (!h || !src) return fail(CPMP_ERR_PARAM, "null argument");
    if (dtype != CPMP_F64 && dtype != CPMP_F32) return fail(CPMP_ERR_PARAM, "dtype");
    CK(cudaSetDevice(h->p.device));
    const size_t n = (size_t)h->n, es = dtype == CPMP_F64 ? 8 : 4;
    if (!h->initialised) {
        // tags and wall values come from the initialiser; a flat state first
        cpmp_droplet d{0, 0, 0, 1, 1, 1};
        cpmp_status s = cpmp_init_droplet(h, &d);
        if (s != CPMP_OK) return s;
    }
    CK(cudaStreamSynchronize(h->st));
    if (f == CPMP_FIELD_RHO) {
        if (bytes != n * es) return fail(CPMP_ERR_SIZE, "RHO needs N values");
        return h2d_real(h, h->rho, n, dtype, src);
    }
    if (f == CPMP_FIELD_U) {
        if (!h->plain) return fail(CPMP_ERR_UNSUPPORTED, "FUSED scheme derives U from DIST");
        if (bytes != 3 * n * es) return fail(CPMP_ERR_SIZE, "U needs 3N values");
        return h2d_real(h, h->u, 3 * n, dtype, src);
    }
    if (f != CPMP_FIELD_DIST) return fail(CPMP_ERR_UNSUPPORTED, "settable fields: RHO, U, DIST");
    if (bytes != CPMP_Q * n * es) return fail(CPMP_ERR_SIZE, "DIST needs 19N values");
    if (h->plain) {
        cpmp_status s = h2d_real(h, h->fb[h->cur], CPMP_Q * n, dtype, src);
        if (s != CPMP_OK) return s;
        if (h->f64)
            plain_launch_macro<double, double>(make_kparams<double>(h), h->type, (const double *)h->fb[h->cur],
                                               (double *)h->rho, (double *)h->u, h->st);
        else
            plain_launch_macro<float, float>(make_kparams<float>(h), h->type, (const float *)h->fb[h->cur],
                                             (float *)h->rho, (float *)h->u, h->st);
        h->launches += 1;
    } else {
        // page-locked host memory is read by the encode kernels in place;
        // anything else goes through a device copy
        cudaPointerAttributes at{};
        const void *dsrc = nullptr;
        if (cudaPointerGetAttributes(&at, src) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
            dsrc = at.devicePointer;
        cudaGetLastError();
        void *tmp = nullptr;
        if (!dsrc) {
            cpmp_status s = dalloc(&tmp, CPMP_Q * n * es, "encode");
            if (s != CPMP_OK) return s;
            dsrc = tmp;
        }
        for (int P = 0; P < 2; ++P)
            if (h->sdiag) cudaMemsetAsync(h->sdiag + P * h->sdiag_stride, 0, sizeof(unsigned), h->st);
        cudaError_t e = tmp ? cudaMemcpyAsync(tmp, src, CPMP_Q * n * es, cudaMemcpyHostToDevice, h->st) : cudaSuccess;
        const int P = (int)(h->step & 1);
        auto k = make_kparams<float>(h);
        if (e == cudaSuccess) {
            fused_launch_encode(h->p.storage, k, P, h->h, h->f0[P], dsrc, dtype == CPMP_F64, h->st);
            fused_launch_density(h->p.storage, k, P, h->h, h->f0[P], (float *)h->rho, h->st, nullptr);
            h->launches += 3;
            e = cudaStreamSynchronize(h->st);
        }
        if (tmp) cudaFree(tmp);
        if (e != cudaSuccess) return fail(CPMP_ERR_CUDA, std::string("encode: ") + cudaGetErrorString(e));
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
    return CPMP_OK;
}

// A box's diagnostics from its kDiagStride result doubles and, for the FUSED
// scheme, the max |MV|^2 bits its last collision left.
static void diag_fill(const cpmp_handle *h, const double *r, unsigned mvbits, cpmp_diag *out)
{
    double m2 = r[1];
    if (!h->plain) {
        float f;
        std::memcpy(&f, &mvbits, sizeof(f));
        m2 = std::max(m2, (double)f);
    }
    out->mass = r[0];
    out->max_speed = std::sqrt(m2);
    out->nonfinite = r[2] != 0.0;
    if (h->p.dx >= 8 && h->p.dz >= 8) {
        out->ca_left = r[4];
        out->ca_right = r[5];
        out->ca_cap = r[6];
        out->x_left = r[7];
        out->x_right = r[8];
        out->cap_h = r[9];
        out->cap_l = r[10];
    }
    out->lap_r = r[12];
    out->lap_dp = r[13];
    out->lap_sigma = r[14];
    out->step = h->step;
}

cpmp_status cpmp_reduce(cpmp_handle *h, cpmp_diag *out)
{
    if (!h || !out) return fail(CPMP_ERR_PARAM, "null argument");
    CK(cudaSetDevice(h->p.device));
    std::memset(out, 0, sizeof(*out));
    // FUSED: max |MV| comes from the last collision (as the reference's MV
    // array, written by its collide kernel); the mass pass reads rho only
    const void *mv = h->plain ? h->mv : nullptr;
    const int tier = h->p.dy / 2;
    if (h->f64) {
        diag_launch_mass<double>(h->type, (const double *)h->rho, (const double *)mv, h->n, h->partials,
                                 h->dout, h->st);
        if (h->p.dx >= 8 && h->p.dz >= 8)
            diag_launch_contact_angle<double>((const double *)h->rho, h->p.dx, h->p.dy, h->p.dz, tier, h->den_g,
                                              h->den_l, h->dout + 4, h->st);
        diag_launch_laplace<double>((const double *)h->rho, h->p.dx, h->p.dy, h->p.dz, h->eos, h->A, h->B, h->T,
                                    h->p.k * h->p.k, h->dout + 12, h->st);
    } else {
        diag_launch_mass<float>(h->type, (const float *)h->rho, (const float *)mv, h->n, h->partials, h->dout,
                                h->st);
        if (h->p.dx >= 8 && h->p.dz >= 8)
            diag_launch_contact_angle<float>((const float *)h->rho, h->p.dx, h->p.dy, h->p.dz, tier, h->den_g,
                                             h->den_l, h->dout + 4, h->st);
        diag_launch_laplace<float>((const float *)h->rho, h->p.dx, h->p.dy, h->p.dz, h->eos, h->A, h->B, h->T,
                                   h->p.k * h->p.k, h->dout + 12, h->st);
    }
    h->launches += 4;
    double r[kDiagStride] = {0};
    unsigned mvbits = 0;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(r, h->dout, kDiagStride * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    if (h->sdiag && h->step > 0)
        CK(cudaMemcpyAsync(&mvbits, h->sdiag + ((h->step - 1) & 1) * h->sdiag_stride, sizeof(unsigned),
                           cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    diag_fill(h, r, mvbits, out);
    if (out->nonfinite) return fail(CPMP_ERR_NONFINITE, "NaN or negative density on a fluid node");
    return CPMP_OK;
}

cpmp_status cpmp_impact_diag(cpmp_handle *h, cpmp_impact *out)
{
    if (!h || !out) return fail(CPMP_ERR_PARAM, "null argument");
    CK(cudaSetDevice(h->p.device));
    std::memset(out, 0, sizeof(*out));
    if (!h->plain) {
        cpmp_status s = fused_diag_fields(h);
        if (s != CPMP_OK) return s;
    }
    const int nq = diag_impact_quantities();
    if (!h->impact_partials) {
        const size_t bytes = (size_t)nq * diag_partial_blocks(h->n) * sizeof(double) + 16 * sizeof(double);
        cpmp_status s = dalloc((void **)&h->impact_partials, bytes, "impact partials");
        if (s != CPMP_OK) return s;
    }
    double *dres = h->impact_partials + (size_t)nq * diag_partial_blocks(h->n);
    const double mid = (h->den_g + h->den_l) / 2;
    if (h->f64)
        diag_launch_impact<double>(h->type, (const double *)h->rho, (const double *)h->mv, h->p.dx, h->p.dy, h->p.dz,
                                   mid, h->impact_partials, dres, h->st);
    else
        diag_launch_impact<float>(h->type, (const float *)h->rho, (const float *)h->mv, h->p.dx, h->p.dy, h->p.dz,
                                  mid, h->impact_partials, dres, h->st);
    h->launches += 2;
    double r[16] = {0};
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(r, dres, nq * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    out->v = r[0];
    out->v_xy = r[1];
    out->v_z = r[2];
    out->mv = r[3];
    out->mv_xy = r[4];
    out->mv_z = r[5];
    out->energy = r[6];
    out->energy_xy = r[7];
    out->energy_z = r[8];
    out->tangential = r[9];
    out->m_tangential = r[10];
    out->drop_momentum = r[11];
    out->drop_mass = r[12];
    out->drop_velocity = r[12] > 0 ? r[11] / r[12] : 0.0;
    return CPMP_OK;
}

cpmp_status cpmp_get_eos(cpmp_handle *h, double *den_g, double *den_l, double *A, double *B, double *T, double *Rc)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    if (den_g) *den_g = h->den_g;
    if (den_l) *den_l = h->den_l;
    if (A) *A = h->A;
    if (B) *B = h->B;
    if (T) *T = h->T;
    if (Rc) *Rc = h->Rc;
    return CPMP_OK;
}

cpmp_status cpmp_autotune(cpmp_handle *h, int *tile_y, int *tile_z, int *march_x, double *ms_per_step)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    CK(cudaSetDevice(h->p.device));
    if (h->plain) return CPMP_OK;
    if (!h->initialised) return fail(CPMP_ERR_PARAM, "initialise the state before tuning");
    const size_t n = (size_t)h->n;
    const size_t hs = h->p.storage == CPMP_STORE_F32 ? 4 : 2;
    // scratch copy of the state: the in-place A-A kernel would otherwise advance it
    void *sh = nullptr, *sf0a = nullptr, *sf0b = nullptr, *srho = nullptr, *sF = nullptr;
    cpmp_status s;
    if ((s = dalloc(&sh, (CPMP_Q - 1) * n * hs, "tune h")) != CPMP_OK) return s;
    if ((s = dalloc(&sf0a, n * 4, "tune f0")) != CPMP_OK || (s = dalloc(&sf0b, n * 4, "tune f0")) != CPMP_OK ||
        (s = dalloc(&srho, n * 4, "tune rho")) != CPMP_OK || (s = dalloc(&sF, force_field_bytes(h), "tune F")) != CPMP_OK) {
        cudaFree(sh); cudaFree(sf0a); cudaFree(sf0b); cudaFree(srho); cudaFree(sF);
        return s;
    }
    const int P0 = (int)(h->step & 1);
    cudaMemcpyAsync(sh, h->h, (CPMP_Q - 1) * n * hs, cudaMemcpyDeviceToDevice, h->st);
    cudaMemcpyAsync(sf0a, h->f0[P0], n * 4, cudaMemcpyDeviceToDevice, h->st);
    cudaMemcpyAsync(srho, h->rho, n * 4, cudaMemcpyDeviceToDevice, h->st);
    auto k = make_kparams<float>(h);
    k.mvmax = nullptr;  // scratch launches leave the diagnostics alone
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    FusedTile best = h->tile;
    double best_ms = 1e30;
    const int xls[] = {8, 16, 32, 64, 128};
    for (int t = 0; t < fused_tile_count(); ++t) {
        for (int xi = 0; xi < 5; ++xi) {
            FusedTile ft = fused_tile(t, xls[xi]);
            // the two-pass form is slower in steady state on every workload
            // measured, while timing its two kernels back to back on the
            // scratch copy underestimates it; it is selected explicitly only
            if (ft.form != 0) continue;
            if (!fused_tile_usable(h->p.storage, h->p.lap_order, ft.ty, ft.tz, ft.np, ft.form)) continue;
            if (ft.np == 2 && !pair_grid_ok(h->p.dz)) continue;
            if (ft.xl > h->p.dx && xi > 0) continue;
            if (ft.ty > 2 * h->p.dy && ft.ty > 1) continue;
            if (ft.tz > 2 * h->p.dz) continue;
            ft.xl = std::min(ft.xl, h->p.dx);
            // warm-up, then time two launches (one of each parity)
            fused_launch_collide(h->p.storage, k, 0, ft, sh, (const float *)sf0a, (float *)sf0b,
                                 (const float *)srho, (float *)sF, h->st, nullptr);
            cudaEventRecord(e0, h->st);
            fused_launch_collide(h->p.storage, k, 1, ft, sh, (const float *)sf0b, (float *)sf0a,
                                 (const float *)srho, (float *)sF, h->st, nullptr);
            fused_launch_collide(h->p.storage, k, 0, ft, sh, (const float *)sf0a, (float *)sf0b,
                                 (const float *)srho, (float *)sF, h->st, nullptr);
            cudaEventRecord(e1, h->st);
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                cudaEventDestroy(e0); cudaEventDestroy(e1);
                cudaFree(sh); cudaFree(sf0a); cudaFree(sf0b); cudaFree(srho); cudaFree(sF);
                return fail(CPMP_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            h->launches += ft.form == 1 ? 6 : 3;
            if (ms / 2 < best_ms) {
                best_ms = ms / 2;
                best = ft;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sh);
    cudaFree(sf0a);
    cudaFree(sf0b);
    cudaFree(srho);
    cudaFree(sF);
    CK(cudaGetLastError());
    if (best.form == 1 && (s = ensure_force_field(h)) != CPMP_OK) return s;
    if (best.ty != h->tile.ty || best.tz != h->tile.tz || best.xl != h->tile.xl || best.np != h->tile.np ||
        best.form != h->tile.form) {
        h->tile = best;
        if (h->gexec) {
            cudaGraphExecDestroy(h->gexec);
            h->gexec = nullptr;
        }
    }
    if (tile_y) *tile_y = best.ty;
    if (tile_z) *tile_z = best.tz;
    if (march_x) *march_x = best.xl;
    if (ms_per_step) *ms_per_step = best_ms;
    return CPMP_OK;
}

cpmp_status cpmp_set_tile(cpmp_handle *h, int tile_y, int tile_z, int march_x)
{
    return cpmp_set_tile_ex(h, tile_y, tile_z, march_x, 1);
}

cpmp_status cpmp_set_tile_ex(cpmp_handle *h, int tile_y, int tile_z, int march_x, int nodes_per_thread)
{
    return cpmp_set_tile_form(h, tile_y, tile_z, march_x, nodes_per_thread, CPMP_FORM_ONE_PASS);
}

cpmp_status cpmp_get_form(cpmp_handle *h, int *form)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    if (h->plain) return fail(CPMP_ERR_UNSUPPORTED, "step forms apply to the FUSED scheme");
    if (form) *form = h->tile.form;
    return CPMP_OK;
}

cpmp_status cpmp_get_tile(cpmp_handle *h, int *tile_y, int *tile_z, int *march_x, int *nodes_per_thread)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    if (h->plain) return fail(CPMP_ERR_UNSUPPORTED, "tiles apply to the FUSED scheme");
    if (tile_y) *tile_y = h->tile.ty;
    if (tile_z) *tile_z = h->tile.tz;
    if (march_x) *march_x = h->tile.xl;
    if (nodes_per_thread) *nodes_per_thread = h->tile.np;
    return CPMP_OK;
}

cpmp_status cpmp_set_tile_form(cpmp_handle *h, int tile_y, int tile_z, int march_x, int nodes_per_thread, int form)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    if (h->plain) return fail(CPMP_ERR_UNSUPPORTED, "tiles apply to the FUSED scheme");
    if (march_x < 1) return fail(CPMP_ERR_PARAM, "march_x must be >= 1");
    if (nodes_per_thread != 1 && nodes_per_thread != 2) return fail(CPMP_ERR_PARAM, "nodes_per_thread must be 1 or 2");
    if (form != CPMP_FORM_ONE_PASS && form != CPMP_FORM_TWO_PASS) return fail(CPMP_ERR_PARAM, "unknown step form");
    if (form == CPMP_FORM_TWO_PASS && nodes_per_thread != 2)
        return fail(CPMP_ERR_PARAM, "the two-pass form runs node pairs (nodes_per_thread 2)");
    if (!fused_tile_usable(h->p.storage, h->p.lap_order, tile_y, tile_z, nodes_per_thread, form))
        return fail(CPMP_ERR_UNSUPPORTED, "tile not instantiated or too large for this device");
    if (nodes_per_thread == 2 && !pair_grid_ok(h->p.dz))
        return fail(CPMP_ERR_UNSUPPORTED, "the paired kernels need DZ a multiple of 4");
    CK(cudaSetDevice(h->p.device));
    if (form == CPMP_FORM_TWO_PASS) {
        const cpmp_status s = ensure_force_field(h);
        if (s != CPMP_OK) return s;
    }
    h->tile = FusedTile{tile_y, tile_z, std::min(march_x, h->p.dx), nodes_per_thread, form};
    if (h->gexec) {
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    return CPMP_OK;
}

void *cpmp_stream(cpmp_handle *h) { return h ? (void *)h->st : nullptr; }

cpmp_status cpmp_set_kernel_timing(cpmp_handle *h, int on)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    CK(cudaSetDevice(h->p.device));
    if (on) {
        if (!h->hook) h->hook.reset(new LaunchHook());
        h->hook->reset();
        h->timing = true;
    } else {
        if (h->hook) h->hook->fold();
        h->timing = false;
    }
    return CPMP_OK;
}

int cpmp_kernel_times(cpmp_handle *h, const char **names, long long *launches, double *ms, int cap)
{
    if (!h || !h->hook) return 0;
    cudaSetDevice(h->p.device);
    h->hook->fold();
    int k = 0;
    for (int c = 0; c < K_CLASSES; ++c) {
        if (h->hook->launches[c] == 0) continue;
        if (k < cap) {
            if (names) names[k] = kernel_class_name(c);
            if (launches) launches[k] = h->hook->launches[c];
            if (ms) ms[k] = h->hook->ms[c];
        }
        ++k;
    }
    return k;
}

long long cpmp_launch_count(cpmp_handle *h) { return h ? h->launches : 0; }

}  // extern "C"

// ------------------------------------------------------------------ batches --
namespace {

cpmp_status batch_upload(cpmp_batch *b)
{
    const int nb = (int)b->boxes.size();
    std::vector<KParams<float>> kp(nb);
    std::vector<BatchBox> bx(nb);
    long long item = 0, wblk = 0, dblk = 0;
    b->nodes = 0;
    for (int i = 0; i < nb; ++i) {
        cpmp_handle *h = b->boxes[i];
        kp[i] = make_kparams<float>(h);
        const bool even = (h->step & 1) == 0;
        bx[i].h = h->h;
        bx[i].f0[0] = h->f0[0];
        bx[i].f0[1] = h->f0[1];
        bx[i].rho[0] = (float *)(even ? h->rho : h->rho2);
        bx[i].rho[1] = (float *)(even ? h->rho2 : h->rho);
        bx[i].tiles_z = (h->p.dz + b->tile.tz - 1) / b->tile.tz;
        bx[i].tiles_y = (h->p.dy + b->tile.ty - 1) / b->tile.ty;
        bx[i].item0 = item;
        item += (long long)bx[i].tiles_z * bx[i].tiles_y * ((h->p.dx + b->tile.xl - 1) / b->tile.xl);
        // flattened wall and density grids: the box's blocks follow the previous box's
        bx[i].wblk0 = wblk;
        if (h->p.wall_mode == 1) wblk += ((long long)h->p.dx * h->p.dy + BATCH_WALL_BLOCK - 1) / BATCH_WALL_BLOCK;
        bx[i].dblk0 = dblk;
        dblk += (((long long)h->p.dy * pairs_per_column(h->p.dz) + BATCH_DENSITY_BLOCK - 1) / BATCH_DENSITY_BLOCK) *
                h->p.dx;
        b->nodes += h->n;
    }
    b->total_items = item;
    b->wall_blocks = wblk;
    b->density_blocks = dblk;
    b->ref_rates = std::all_of(kp.begin(), kp.end(), [](const KParams<float> &k) { return reference_rates(k); });
    // the batched diagnostics: each box's mass blocks follow the previous box's
    std::vector<DiagBox> dg(nb);
    long long mblk = 0;
    for (int i = 0; i < nb; ++i) {
        const cpmp_handle *h = b->boxes[i];
        DiagBox &d = dg[i];
        d.type = h->type;
        d.rho[0] = bx[i].rho[0];
        d.rho[1] = bx[i].rho[1];
        d.part = h->partials;
        d.n = h->n;
        d.blk0 = mblk;
        d.nb = diag_partial_blocks(h->n);
        d.vec = diag_mass_vec_flags(h->type, d.rho[0], nullptr, h->n) & diag_mass_vec_flags(h->type, d.rho[1], nullptr, h->n);
        mblk += d.nb;
        d.dx = h->p.dx;
        d.dy = h->p.dy;
        d.dz = h->p.dz;
        d.tier = h->p.dy / 2;
        d.angle = (h->p.dx >= 8 && h->p.dz >= 8) ? 1 : 0;
        d.eos = h->eos;
        d.mid = (h->den_g + h->den_l) / 2;
        d.A = h->A;
        d.B = h->B;
        d.T = h->T;
        d.kk = h->p.k * h->p.k;
    }
    b->mass_blocks = mblk;
    CK(cudaMemcpyAsync(b->d_params, kp.data(), nb * sizeof(KParams<float>), cudaMemcpyHostToDevice, b->st));
    CK(cudaMemcpyAsync(b->d_boxes, bx.data(), nb * sizeof(BatchBox), cudaMemcpyHostToDevice, b->st));
    CK(cudaMemcpyAsync(b->d_diag, dg.data(), nb * sizeof(DiagBox), cudaMemcpyHostToDevice, b->st));
    CK(cudaStreamSynchronize(b->st));
    return CPMP_OK;
}

void batch_one_step(cpmp_batch *b, LaunchHook *hook, bool bookkeeping)
{
    const int P = (int)(b->boxes[0]->step & 1);
    const size_t nb = b->boxes.size();
    cudaMemsetAsync(b->d_mvmax + P * nb, 0, nb * sizeof(unsigned), b->st);
    fused_batch_step(b->storage, b->lap_order, b->wall_mode, b->complex_bc, b->tile, b->d_params, b->d_boxes,
                     (int)b->boxes.size(), b->total_items, b->wall_blocks, b->density_blocks, P, b->d_counter,
                     b->ref_rates, b->st, hook);
    if (!bookkeeping) return;
    for (cpmp_handle *h : b->boxes) {
        h->step += 1;
        std::swap(h->rho, h->rho2);
    }
    b->launches += (b->wall_mode == 1 ? 1 : 0) + 2;
}

cpmp_status batch_check(cpmp_batch *b)
{
    const long long s0 = b->boxes[0]->step;
    for (cpmp_handle *h : b->boxes) {
        if (!h->initialised) return fail(CPMP_ERR_PARAM, "initialise every box of the batch first");
        if ((h->step & 1) != (s0 & 1)) return fail(CPMP_ERR_PARAM, "boxes of a batch must share the step parity");
    }
    return CPMP_OK;
}

}  // namespace

extern "C" {

cpmp_status cpmp_batch_create(const cpmp_params *params, int count, cpmp_batch **out)
{
    if (!params || !out || count < 1) return fail(CPMP_ERR_PARAM, "need count >= 1 parameter sets");
    if (count > 65535) return fail(CPMP_ERR_PARAM, "at most 65535 boxes per batch");
    *out = nullptr;
    const cpmp_params &p0 = params[0];
    for (int i = 0; i < count; ++i) {
        const cpmp_params &p = params[i];
        if (p.scheme != CPMP_SCHEME_FUSED) return fail(CPMP_ERR_UNSUPPORTED, "batches run the FUSED scheme");
        if (p.dx > 65535) return fail(CPMP_ERR_PARAM, "batch boxes have dx <= 65535");
        if (p.storage != p0.storage || p.lap_order != p0.lap_order || p.wall_mode != p0.wall_mode ||
            p.complex_bc != p0.complex_bc || p.device != p0.device)
            return fail(CPMP_ERR_PARAM, "boxes of a batch share storage, lap_order, wall_mode, complex_bc, device");
    }
    std::unique_ptr<cpmp_batch> b(new cpmp_batch());
    b->device = p0.device;
    b->storage = p0.storage;
    b->lap_order = p0.lap_order;
    b->wall_mode = p0.wall_mode;
    b->complex_bc = p0.complex_bc;
    CK(cudaSetDevice(b->device));
    CK(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    auto cleanup = [&]() {
        for (cpmp_handle *h : b->boxes) cpmp_destroy(h);
        b->boxes.clear();
        if (b->d_params) cudaFree(b->d_params);
        if (b->d_boxes) cudaFree(b->d_boxes);
        if (b->d_counter) cudaFree(b->d_counter);
        if (b->d_mvmax) cudaFree(b->d_mvmax);
        if (b->d_diag) cudaFree(b->d_diag);
        if (b->d_dout) cudaFree(b->d_dout);
        cudaStreamDestroy(b->st);
    };
    for (int i = 0; i < count; ++i) {
        cpmp_handle *h = nullptr;
        cpmp_status s = cpmp_create(&params[i], &h);
        if (s != CPMP_OK) {
            cleanup();
            return s;
        }
        cudaStreamDestroy(h->st);
        h->st = b->st;
        h->in_batch = true;
        b->boxes.push_back(h);
    }
    // one tile for every box: the first box's heuristic choice (one node per
    // thread, the batched collide's form), refined by cpmp_batch_autotune
    b->tile = b->boxes[0]->tile;
    if (b->tile.np != 1) b->tile = FusedTile{8, 32, b->tile.xl, 1};
    // (a march longer than a box's x extent covers that box in one chunk)
    for (cpmp_handle *h : b->boxes) h->tile = b->tile;
    cpmp_status s;
    if ((s = dalloc((void **)&b->d_params, count * sizeof(KParams<float>), "batch params")) != CPMP_OK ||
        (s = dalloc((void **)&b->d_boxes, count * sizeof(BatchBox), "batch boxes")) != CPMP_OK ||
        (s = dalloc((void **)&b->d_counter, sizeof(unsigned), "batch counter")) != CPMP_OK ||
        (s = dalloc((void **)&b->d_mvmax, 2 * count * sizeof(unsigned), "batch mv max")) != CPMP_OK ||
        (s = dalloc((void **)&b->d_diag, count * sizeof(DiagBox), "batch diagnostics table")) != CPMP_OK ||
        (s = dalloc((void **)&b->d_dout, (size_t)count * kDiagStride * sizeof(double), "batch diagnostics")) !=
            CPMP_OK) {
        cleanup();
        return s;
    }
    CK(cudaMemset(b->d_mvmax, 0, 2 * count * sizeof(unsigned)));
    for (int i = 0; i < count; ++i) {  // the boxes' diagnostics live in the batch's array
        cpmp_handle *h = b->boxes[i];
        if (h->sdiag && h->sdiag_owned) cudaFree(h->sdiag);
        h->sdiag = b->d_mvmax + i;
        h->sdiag_stride = count;
        h->sdiag_owned = false;
    }
    if ((s = batch_upload(b.get())) != CPMP_OK) {
        cleanup();
        return s;
    }
    *out = b.release();
    return CPMP_OK;
}

cpmp_status cpmp_batch_handle(cpmp_batch *b, int index, cpmp_handle **h)
{
    if (!b || !h || index < 0 || index >= (int)b->boxes.size()) return fail(CPMP_ERR_PARAM, "box index");
    *h = b->boxes[index];
    return CPMP_OK;
}

int cpmp_batch_count(cpmp_batch *b) { return b ? (int)b->boxes.size() : 0; }

long long cpmp_batch_nodes(cpmp_batch *b) { return b ? b->nodes : 0; }

cpmp_status cpmp_batch_step(cpmp_batch *b, int nsteps)
{
    if (!b) return fail(CPMP_ERR_PARAM, "null batch");
    if (nsteps < 0) return fail(CPMP_ERR_PARAM, "nsteps must be >= 0");
    cpmp_status s;
    if ((s = batch_check(b)) != CPMP_OK) return s;
    CK(cudaSetDevice(b->device));
    // the device tables name each box's even- and odd-step density buffers,
    // so they stay valid whatever the parity
    LaunchHook *hook = b->timing ? b->hook.get() : nullptr;
    int left = nsteps;
    if (hook || nsteps < 2) {
        for (; left > 0; --left) batch_one_step(b, hook, true);
        CK(cudaGetLastError());
        return CPMP_OK;
    }
    if (b->boxes[0]->step & 1) {
        batch_one_step(b, nullptr, true);
        --left;
    }
    if (left >= 2) {
        if (!b->gexec) {
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
            batch_one_step(b, nullptr, false);
            // the second step of the pair runs at odd parity on the same tables
            {
                const int P = 1;
                const size_t nb = b->boxes.size();
                cudaMemsetAsync(b->d_mvmax + P * nb, 0, nb * sizeof(unsigned), b->st);
                fused_batch_step(b->storage, b->lap_order, b->wall_mode, b->complex_bc, b->tile, b->d_params,
                                 b->d_boxes, (int)b->boxes.size(), b->total_items, b->wall_blocks, b->density_blocks, P,
                                 b->d_counter, b->ref_rates, b->st, nullptr);
            }
            cudaError_t e = cudaStreamEndCapture(b->st, &g);
            if (e != cudaSuccess) return fail(CPMP_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&b->gexec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                b->gexec = nullptr;
                return fail(CPMP_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e));
            }
        }
        while (left >= 2) {
            CK(cudaGraphLaunch(b->gexec, b->st));
            for (cpmp_handle *h : b->boxes) h->step += 2;  // two swaps: rho pointers unchanged
            b->launches += 2LL * ((b->wall_mode == 1 ? 1 : 0) + 2);
            left -= 2;
        }
    }
    if (left == 1) batch_one_step(b, nullptr, true);
    CK(cudaGetLastError());
    return CPMP_OK;
}

cpmp_status cpmp_batch_sync(cpmp_batch *b)
{
    if (!b) return fail(CPMP_ERR_PARAM, "null batch");
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->st));
    return CPMP_OK;
}

cpmp_status cpmp_batch_reduce(cpmp_batch *b, cpmp_diag *out, int count)
{
    if (!b || !out) return fail(CPMP_ERR_PARAM, "null argument");
    const int nb = (int)b->boxes.size();
    if (count != nb) return fail(CPMP_ERR_PARAM, "out must hold one cpmp_diag per box of the batch");
    cpmp_status s;
    if ((s = batch_check(b)) != CPMP_OK) return s;
    CK(cudaSetDevice(b->device));
    std::memset(out, 0, (size_t)nb * sizeof(cpmp_diag));
    const long long step = b->boxes[0]->step;
    diag_launch_batch(b->d_diag, nb, b->mass_blocks, (int)(step & 1), b->d_dout, b->st);
    b->launches += 4;
    std::vector<double> r((size_t)nb * kDiagStride);
    std::vector<unsigned> mv(nb, 0u);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(r.data(), b->d_dout, r.size() * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    if (step > 0)
        CK(cudaMemcpyAsync(mv.data(), b->d_mvmax + ((step - 1) & 1) * nb, nb * sizeof(unsigned),
                           cudaMemcpyDeviceToHost, b->st));
    CK(cudaStreamSynchronize(b->st));
    int bad = -1;
    for (int i = 0; i < nb; ++i) {
        diag_fill(b->boxes[i], r.data() + (size_t)i * kDiagStride, mv[i], out + i);
        if (out[i].nonfinite && bad < 0) bad = i;
    }
    if (bad >= 0)
        return fail(CPMP_ERR_NONFINITE, "NaN or negative density on a fluid node of box " + std::to_string(bad));
    return CPMP_OK;
}

cpmp_status cpmp_batch_set_tile(cpmp_batch *b, int tile_y, int tile_z, int march_x)
{
    return cpmp_batch_set_tile_ex(b, tile_y, tile_z, march_x, 1);
}

cpmp_status cpmp_batch_get_tile(cpmp_batch *b, int *tile_y, int *tile_z, int *march_x, int *nodes_per_thread)
{
    if (!b) return fail(CPMP_ERR_PARAM, "null batch");
    if (tile_y) *tile_y = b->tile.ty;
    if (tile_z) *tile_z = b->tile.tz;
    if (march_x) *march_x = b->tile.xl;
    if (nodes_per_thread) *nodes_per_thread = b->tile.np;
    return CPMP_OK;
}

cpmp_status cpmp_batch_set_tile_ex(cpmp_batch *b, int tile_y, int tile_z, int march_x, int nodes_per_thread)
{
    if (!b) return fail(CPMP_ERR_PARAM, "null batch");
    if (march_x < 1) return fail(CPMP_ERR_PARAM, "march_x must be >= 1");
    if (nodes_per_thread != 1) return fail(CPMP_ERR_UNSUPPORTED, "batches step one node per thread");
    if (!fused_tile_usable(b->storage, b->lap_order, tile_y, tile_z, nodes_per_thread))
        return fail(CPMP_ERR_UNSUPPORTED, "tile not instantiated or too large for this device");
    b->tile = FusedTile{tile_y, tile_z, march_x, nodes_per_thread};
    for (cpmp_handle *h : b->boxes) h->tile = b->tile;
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return batch_upload(b);
}

cpmp_status cpmp_batch_autotune(cpmp_batch *b, int *tile_y, int *tile_z, int *march_x, double *ms_per_step)
{
    if (!b) return fail(CPMP_ERR_PARAM, "null batch");
    cpmp_status s;
    if ((s = batch_check(b)) != CPMP_OK) return s;
    CK(cudaSetDevice(b->device));
    // scratch copies of every box's lattice so the state is not advanced
    const size_t hs = b->storage == CPMP_STORE_F32 ? 4 : 2;
    std::vector<void *> scratch;
    auto free_scratch = [&]() {
        for (void *q : scratch) cudaFree(q);
        scratch.clear();
    };
    struct Saved { void *h, *rho, *rho2; float *f0[2]; };
    std::vector<Saved> saved;
    for (cpmp_handle *h : b->boxes) {
        const size_t n = (size_t)h->n;
        void *sh = nullptr, *sa = nullptr, *sb = nullptr, *sr = nullptr, *sr2 = nullptr;
        if ((s = dalloc(&sh, (CPMP_Q - 1) * n * hs, "tune h")) != CPMP_OK) { free_scratch(); return s; }
        scratch.push_back(sh);
        if ((s = dalloc(&sa, n * 4, "tune f0")) != CPMP_OK) { free_scratch(); return s; }
        scratch.push_back(sa);
        if ((s = dalloc(&sb, n * 4, "tune f0")) != CPMP_OK) { free_scratch(); return s; }
        scratch.push_back(sb);
        if ((s = dalloc(&sr, n * 4, "tune rho")) != CPMP_OK) { free_scratch(); return s; }
        scratch.push_back(sr);
        if ((s = dalloc(&sr2, n * 4, "tune rho")) != CPMP_OK) { free_scratch(); return s; }
        scratch.push_back(sr2);
        cudaMemcpyAsync(sh, h->h, (CPMP_Q - 1) * n * hs, cudaMemcpyDeviceToDevice, b->st);
        cudaMemcpyAsync(sa, h->f0[0], n * 4, cudaMemcpyDeviceToDevice, b->st);
        cudaMemcpyAsync(sb, h->f0[1], n * 4, cudaMemcpyDeviceToDevice, b->st);
        cudaMemcpyAsync(sr, h->rho, n * 4, cudaMemcpyDeviceToDevice, b->st);
        cudaMemcpyAsync(sr2, h->rho2, n * 4, cudaMemcpyDeviceToDevice, b->st);
        saved.push_back(Saved{h->h, h->rho, h->rho2, {h->f0[0], h->f0[1]}});
        h->h = sh;
        h->f0[0] = (float *)sa;
        h->f0[1] = (float *)sb;
        h->rho = sr;
        h->rho2 = sr2;
    }
    const FusedTile keep = b->tile;
    const long long step_keep = b->boxes[0]->step;
    std::vector<unsigned> mv_keep(2 * b->boxes.size());  // the scratch steps overwrite the diagnostics
    cudaMemcpyAsync(mv_keep.data(), b->d_mvmax, mv_keep.size() * sizeof(unsigned), cudaMemcpyDeviceToHost, b->st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    FusedTile best = keep;
    double best_ms = 1e30;
    int maxx = 0;
    for (cpmp_handle *h : b->boxes) maxx = std::max(maxx, h->p.dx);
    const int xls[] = {8, 16, 32, 64, 128};
    cudaError_t err = cudaSuccess;
    for (int t = 0; t < fused_tile_count() && err == cudaSuccess; ++t) {
        for (int xi = 0; xi < 5; ++xi) {
            FusedTile ft = fused_tile(t, xls[xi]);
            if (ft.np != 1 || !fused_tile_usable(b->storage, b->lap_order, ft.ty, ft.tz, ft.np)) continue;
            if (xi > 0 && xls[xi - 1] >= maxx) continue;  // every box already in one chunk
            b->tile = ft;
            if (batch_upload(b) != CPMP_OK) break;
            batch_one_step(b, nullptr, false);
            cudaEventRecord(e0, b->st);
            batch_one_step(b, nullptr, false);
            batch_one_step(b, nullptr, false);
            cudaEventRecord(e1, b->st);
            err = cudaEventSynchronize(e1);
            if (err != cudaSuccess) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            b->launches += 3LL * ((b->wall_mode == 1 ? 1 : 0) + 2);
            if (ms / 2 < best_ms) {
                best_ms = ms / 2;
                best = b->tile;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (size_t i = 0; i < b->boxes.size(); ++i) {
        cpmp_handle *h = b->boxes[i];
        h->h = saved[i].h;
        h->rho = saved[i].rho;
        h->rho2 = saved[i].rho2;
        h->f0[0] = saved[i].f0[0];
        h->f0[1] = saved[i].f0[1];
        h->step = step_keep;
    }
    cudaStreamSynchronize(b->st);
    free_scratch();
    if (err != cudaSuccess) return fail(CPMP_ERR_CUDA, std::string("batch autotune: ") + cudaGetErrorString(err));
    CK(cudaMemcpy(b->d_mvmax, mv_keep.data(), mv_keep.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
    b->tile = best;
    for (cpmp_handle *h : b->boxes) h->tile = best;
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if ((s = batch_upload(b)) != CPMP_OK) return s;
    if (tile_y) *tile_y = best.ty;
    if (tile_z) *tile_z = best.tz;
    if (march_x) *march_x = best.xl;
    if (ms_per_step) *ms_per_step = best_ms;
    return CPMP_OK;
}

cpmp_status cpmp_batch_set_kernel_timing(cpmp_batch *b, int on)
{
    if (!b) return fail(CPMP_ERR_PARAM, "null batch");
    if (on) {
        if (!b->hook) b->hook.reset(new LaunchHook());
        b->hook->reset();
        b->timing = true;
    } else {
        if (b->hook) b->hook->fold();
        b->timing = false;
    }
    return CPMP_OK;
}

int cpmp_batch_kernel_times(cpmp_batch *b, const char **names, long long *launches, double *ms, int cap)
{
    if (!b || !b->hook) return 0;
    cudaSetDevice(b->device);
    b->hook->fold();
    int k = 0;
    for (int c = 0; c < K_CLASSES; ++c) {
        if (b->hook->launches[c] == 0) continue;
        if (k < cap) {
            if (names) names[k] = kernel_class_name(c);
            if (launches) launches[k] = b->hook->launches[c];
            if (ms) ms[k] = b->hook->ms[c];
        }
        ++k;
    }
    return k;
}

long long cpmp_batch_launch_count(cpmp_batch *b) { return b ? b->launches : 0; }

void *cpmp_batch_stream(cpmp_batch *b) { return b ? (void *)b->st : nullptr; }

void cpmp_batch_destroy(cpmp_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->st);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (cpmp_handle *h : b->boxes) cpmp_destroy(h);
    cudaFree(b->d_params);
    cudaFree(b->d_boxes);
    cudaFree(b->d_counter);
    cudaFree(b->d_mvmax);
    cudaFree(b->d_diag);
    cudaFree(b->d_dout);
    cudaStreamDestroy(b->st);
    b->hook.reset();
    delete b;
}

}  // extern "C"

// ------------------------------------------------------------------ adjoint --
namespace {

// Forward run with sqrt(T) checkpoints, loss, reverse sweep (PLAIN scheme).
template <class R>
cpmp_status adjoint_run(cpmp_handle *h, int T, int S, const double *target_host, double *loss_out,
                        double *gwall_out, double *gka_out)
{
    const size_t n = (size_t)h->n, np = (size_t)h->p.dx * h->p.dy;
    const size_t state = 23 * n;    // checkpoint: f (19N) | rho (N) | u (3N)
    const size_t sstate = 29 * n;   // segment state: f | rho | u | grad mu (3N) | F (3N)
    const int nck = (T + S - 1) / S;
    std::vector<void *> mem;
    cudaStream_t rs = nullptr;  // replay stream
    cudaEvent_t replayed[2] = {nullptr, nullptr}, reversed[2] = {nullptr, nullptr}, fwd = nullptr;
    auto alloc = [&](void **p, size_t bytes, const char *what) -> cpmp_status {
        cpmp_status s = dalloc(p, bytes, what);
        if (s == CPMP_OK) mem.push_back(*p);
        return s;
    };
    auto release = [&]() {
        if (rs) cudaStreamSynchronize(rs);
        for (void *q : mem) cudaFree(q);
        mem.clear();
        for (cudaEvent_t e : {replayed[0], replayed[1], reversed[0], reversed[1], fwd})
            if (e) cudaEventDestroy(e);
        if (rs) cudaStreamDestroy(rs);
        rs = nullptr;
    };
    R *ck = nullptr, *seg[2] = {nullptr, nullptr}, *mvr = nullptr, *mus = nullptr;
    double *target = nullptr;
    AdjBufs<R> b{};
    const KParams<R> kp = make_kparams<R>(h);
    const dim3 g3((unsigned)((h->p.dz + 127) / 128), (unsigned)h->p.dy, (unsigned)h->p.dx);
    const size_t nblocks = (size_t)g3.x * g3.y * g3.z;
    cpmp_status s;
#define ALLOC(ptr, bytes, what)                                           \
    if ((s = alloc((void **)&(ptr), (bytes), (what))) != CPMP_OK) {       \
        release();                                                        \
        return s;                                                         \
    }
    ALLOC(ck, (size_t)nck * state * sizeof(R), "adjoint checkpoints");
    ALLOC(seg[0], (size_t)S * sstate * sizeof(R), "adjoint segment");
    ALLOC(mvr, 3 * n * sizeof(R), "adjoint mv");
    ALLOC(mus, n * sizeof(R), "adjoint mu");
    ALLOC(target, n * sizeof(double), "adjoint target");
    ALLOC(b.lamp, 19 * n * sizeof(R), "lambda partial");
    ALLOC(b.lamp_next, 19 * n * sizeof(R), "lambda partial");
    ALLOC(b.lamF, 4 * n * sizeof(R), "lambda F");
    ALLOC(b.lammu, n * sizeof(R), "lambda mu");
    ALLOC(b.lmr, 2 * n * sizeof(R), "lambda mu (fluid), rho");
    ALLOC(b.lamrho, n * sizeof(R), "lambda rho");
    ALLOC(b.lamrho_next, n * sizeof(R), "lambda rho");
    ALLOC(b.ka_part, nblocks * sizeof(double), "loss partials");
    ALLOC(b.ka_acc, (size_t)adj_tiled_blocks(h->p.dx, h->p.dy, h->p.dz) * sizeof(double), "kappa partials");
    ALLOC(b.gka, sizeof(double), "kappa gradient");
    ALLOC(b.gwall, 2 * np * sizeof(double), "wall gradient");
    ALLOC(b.loss, sizeof(double), "loss");
#undef ALLOC
    // A second segment buffer lets the replay of segment k-1 run on its own
    // stream while the reverse sweep of segment k runs; without the room for
    // it the two alternate on one buffer.
    int nbuf = 1;
    if (nck > 1 && cudaMalloc((void **)&seg[1], (size_t)S * sstate * sizeof(R)) == cudaSuccess) {
        mem.push_back(seg[1]);
        nbuf = 2;
    }
    cudaGetLastError();
    {
        cudaError_t e = cudaStreamCreateWithFlags(&rs, cudaStreamNonBlocking);
        for (cudaEvent_t *ev : {&replayed[0], &replayed[1], &reversed[0], &reversed[1], &fwd})
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            release();
            return fail(CPMP_ERR_CUDA, std::string("adjoint streams: ") + cudaGetErrorString(e));
        }
    }
    cudaStream_t st = h->st;
#define CKR(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            release();                                                                             \
            return fail(CPMP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
        }                                                                                          \
    } while (0)
    CKR(cudaMemcpyAsync(target, target_host, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CKR(cudaMemsetAsync(b.gka, 0, sizeof(double), st));
    CKR(cudaMemsetAsync(b.gwall, 0, 2 * np * sizeof(double), st));
    auto save = [&](R *dst) {
        cudaMemcpyAsync(dst, h->fb[h->cur], 19 * n * sizeof(R), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(dst + 19 * n, h->rho, n * sizeof(R), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(dst + 20 * n, h->u, 3 * n * sizeof(R), cudaMemcpyDeviceToDevice, st);
    };
    LaunchHook *hook = h->timing ? h->hook.get() : nullptr;
    // Replay segment k on the replay stream into buffer k % nbuf: the step
    // from state m-1 to m extrapolates the wall layers of state m-1's density
    // in place and leaves its grad mu and F in its slot, so each slot ends up
    // holding what the reverse step needs (walled rho, u, grad mu, F).
    auto replay = [&](int k) {
        const int n0 = k * S, len = std::min(n0 + S, T) - n0, bi = k % nbuf;
        if (k + nbuf < nck) cudaStreamWaitEvent(rs, reversed[bi], 0);  // the buffer's previous segment is done
        R *sg = seg[bi];
        cudaMemcpyAsync(sg, ck + (size_t)k * state, state * sizeof(R), cudaMemcpyDeviceToDevice, rs);
        for (int m = 1; m < len; ++m) {
            R *prev = sg + (size_t)(m - 1) * sstate, *cur = sg + (size_t)m * sstate;
            plain_launch_step_split<R, R>(kp, h->type, prev + 19 * n, mus, prev + 20 * n, prev + 26 * n, mvr, prev,
                                          cur, cur + 19 * n, cur + 20 * n, prev + 23 * n, rs, hook);
        }
        R *last = sg + (size_t)(len - 1) * sstate;  // never stepped from
        plain_launch_mu_force<R>(kp, h->type, last + 19 * n, mus, last + 26 * n, rs, last + 23 * n);
        cudaEventRecord(replayed[bi], rs);
    };
    auto reverse = [&](int k) {
        const int n0 = k * S, n1 = std::min(n0 + S, T), bi = k % nbuf;
        cudaStreamWaitEvent(st, replayed[bi], 0);
        for (int t = n1 - 1; t >= n0; --t) {
            const R *stt = seg[bi] + (size_t)(t - n0) * sstate;
            adj_launch_step<R>(kp, h->type, stt + 19 * n, stt + 20 * n, stt + 23 * n, stt + 26 * n, b, st, hook);
            std::swap(b.lamp, b.lamp_next);
            std::swap(b.lamrho, b.lamrho_next);
        }
        cudaEventRecord(reversed[bi], st);
    };
    // forward, checkpoint every S steps (the handle's own state advances to
    // T); the last segment's replay starts as soon as its checkpoint exists
    for (int t = 0; t < T; ++t) {
        if (t % S == 0) {
            save(ck + (size_t)(t / S) * state);
            if (t / S == nck - 1) {
                cudaEventRecord(fwd, st);
                cudaStreamWaitEvent(rs, fwd, 0);
                replay(nck - 1);
            }
        }
        launch_one_step(h, hook);
    }
    adj_launch_loss<R>(kp, h->type, (const R *)h->rho, target, b, st);
    CKR(cudaGetLastError());
    // reverse sweep, one segment at a time, the next segment's replay ahead
    for (int k = nck - 1; k >= 0; --k) {
        if (nbuf == 2 && k > 0) replay(k - 1);
        reverse(k);
        if (nbuf == 1 && k > 0) replay(k - 1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            release();
            return fail(CPMP_ERR_CUDA, std::string("adjoint sweep: ") + cudaGetErrorString(e));
        }
    }
#undef CKR
    adj_launch_finish<R>(kp, b, st);
    std::vector<double> gw(2 * np);
    double loss = 0, gka = 0;
    cudaMemcpyAsync(&loss, b.loss, sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&gka, b.gka, sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(gw.data(), b.gwall, 2 * np * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    release();
    if (e != cudaSuccess) return fail(CPMP_ERR_CUDA, std::string("adjoint: ") + cudaGetErrorString(e));
    h->launches += (long long)T * h->launches_per_step * 2 + (long long)T * 12;
    if (loss_out) *loss_out = loss;
    if (gka_out) *gka_out = gka;
    if (gwall_out) std::memcpy(gwall_out, gw.data(), 2 * np * sizeof(double));
    return CPMP_OK;
}

}  // namespace

extern "C" {

cpmp_status cpmp_get_dims(cpmp_handle *h, int *dims)
{
    if (!h || !dims) return fail(CPMP_ERR_PARAM, "null argument");
    dims[0] = h->p.dx;
    dims[1] = h->p.dy;
    dims[2] = h->p.dz;
    return CPMP_OK;
}

cpmp_status cpmp_set_kappa(cpmp_handle *h, double ka)
{
    if (!h) return fail(CPMP_ERR_PARAM, "null handle");
    h->p.ka = ka;
    if (h->gexec) {  // captured launches carry the parameters by value
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    return CPMP_OK;
}

cpmp_status cpmp_adjoint(cpmp_handle *h, int steps, int checkpoint_every, const double *target_rho,
                         double *loss, double *grad_wall, double *grad_kappa)
{
    if (!h || !target_rho) return fail(CPMP_ERR_PARAM, "null argument");
    if (!h->plain) return fail(CPMP_ERR_UNSUPPORTED, "the adjoint runs on the PLAIN scheme");
    if (h->p.k1 != 0.0 || h->p.k2 != 0.0)
        return fail(CPMP_ERR_UNSUPPORTED, "the K1/K2 pressure-tensor term is not differentiated");
    if (!h->initialised) return fail(CPMP_ERR_PARAM, "initialise the state first");
    if (steps < 1) return fail(CPMP_ERR_PARAM, "steps must be >= 1");
    int S = checkpoint_every;
    if (S <= 0) S = (int)std::ceil(std::sqrt((double)steps));
    S = std::max(1, std::min(S, steps));
    CK(cudaSetDevice(h->p.device));
    CK(cudaStreamSynchronize(h->st));
    if (h->f64) return adjoint_run<double>(h, steps, S, target_rho, loss, grad_wall, grad_kappa);
    return adjoint_run<float>(h, steps, S, target_rho, loss, grad_wall, grad_kappa);
}

}  // extern "C"
