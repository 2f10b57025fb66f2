// mtg_api.cu -- the extern "C" boundary (include/mtcode_gb300.h): argument checks, error
// conversion, and dispatch to the FP32 or FP64 implementation.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mtcode_gb300.h"
#include "mtg_sys_base.h"

using namespace mtg_impl;

namespace {

thread_local std::string g_create_error;

// ------------------------------------------------------------------ model / replica tables

void check_model(const mtg_patch_model &m, int n) {
    MTG_REQUIRE(m.n_types >= 1 && m.n_types <= MTG_MAX_TYPES, "patch model: n_types out of range");
    int nor = 0, npots = 0, prev = 0;
    for (int k = 0; k < m.n_types; k++) {
        MTG_REQUIRE(m.patches_per_type[k] >= 0, "patch model: negative patch count");
        MTG_REQUIRE(m.count_per_type[k] >= prev, "patch model: count_per_type must be cumulative");
        prev = m.count_per_type[k];
        nor += m.patches_per_type[k];
    }
    MTG_REQUIRE(prev == n, "patch model: count_per_type[last] must equal the replica's particle count");
    MTG_REQUIRE(nor <= MTG_MAX_ORIENT, "patch model: too many patch vectors");
    for (int a = 0; a < m.n_types; a++)
        for (int b = a; b < m.n_types; b++) npots += m.patches_per_type[a] * m.patches_per_type[b];
    MTG_REQUIRE(npots <= MTG_MAX_POTS, "patch model: too many potentials");
    for (int i = 0; i < nor; i++) {
        double s = m.orient[i][0] * m.orient[i][0] + m.orient[i][1] * m.orient[i][1] + m.orient[i][2] * m.orient[i][2];
        // KernFrenkelOnePatch2 constructor check (potentialtheta.h:409-416)
        MTG_REQUIRE(std::fabs(s - 1) <= 1e-5, "patch model: patch vectors must be unit vectors");
    }
    for (int q = 0; q < npots; q++)
        MTG_REQUIRE(m.params[q][1] > 0 && m.params[q][2] > 0, "patch model: dis and thetam must be positive");
}

}  // namespace

struct mtg_system {
    std::unique_ptr<SysBase> impl;
    int device = 0;
    std::string err;
};

#define MTG_GUARD(h, ...)                                    \
    do {                                                      \
        if (!(h)) return MTG_ERR_ARG;                         \
        try {                                                 \
            cudaSetDevice((h)->device);                       \
            __VA_ARGS__;                                      \
        } catch (const Fail &f_) {                            \
            (h)->err = f_.msg;                                \
            return f_.st;                                     \
        } catch (const std::exception &e_) {                  \
            (h)->err = e_.what();                             \
            return MTG_ERR_ARG;                               \
        }                                                     \
    } while (0)

// the single-bond capacity that failed, from the reason bits latched with MTG_FLAG_BIND
static std::string bind_failure(uint32_t f) {
    std::string m = "single-bond mode:";
    if (f & MTG_BIND_WHY_ADJ) m += " a patch had more than 8 candidate partners;";
    if (f & MTG_BIND_WHY_CLUSTER) m += " a patch cluster exceeded 128 patches;";
    if (f & MTG_BIND_WHY_LIST) m += " a list of the force pass was full;";
    if (f & MTG_BIND_WHY_REF) m += " a cluster reached one of the reference's error() paths;";
    if (f & MTG_BIND_WHY_SPIN) m += " an atomic retry loop reached its bound;";
    return m;
}

extern "C" {

int mtg_api_version(void) { return MTG_API_VERSION; }

const char *mtg_status_string(int s) {
    switch (s) {
        case MTG_OK: return "ok";
        case MTG_ERR_ARG: return "invalid argument";
        case MTG_ERR_CUDA: return "CUDA runtime error";
        case MTG_ERR_NOMEM: return "device allocation failed";
        case MTG_ERR_STATE: return "call order violated";
        case MTG_ERR_NONFINITE: return "non-finite state on the device";
        case MTG_ERR_CAPACITY: return "caller buffer too small";
        case MTG_ERR_TIMEOUT: return "bounded device wait expired";
        case MTG_ERR_NODEVICE: return "no usable sm_103 device";
        default: return "unknown status";
    }
}

void mtg_model_tetrahedral(mtg_patch_model *m, double att, double dis, double thetam) {
    std::memset(m, 0, sizeof(*m));
    m->n_types = 1;
    m->patches_per_type[0] = 4;
    m->count_per_type[0] = 0;  // set to n by the caller (or mtg_create fills a 0 with n)
    const double v[4][3] = {{std::sqrt(8. / 9.), 0., -1. / 3.},
                            {-std::sqrt(2. / 9.), std::sqrt(2. / 3.), -1. / 3.},
                            {-std::sqrt(2. / 9.), -std::sqrt(2. / 3.), -1. / 3.},
                            {0., 0., 1.}};
    for (int i = 0; i < 4; i++)
        for (int c = 0; c < 3; c++) m->orient[i][c] = v[i][c];
    for (int q = 0; q < 16; q++) {
        m->params[q][0] = att;
        m->params[q][1] = dis;
        m->params[q][2] = thetam;
    }
}

void mtg_model_bivalent(mtg_patch_model *m, double att, double dis, double thetam) {
    std::memset(m, 0, sizeof(*m));
    m->n_types = 1;
    m->patches_per_type[0] = 2;
    m->orient[0][0] = -1.0;
    m->orient[1][0] = 1.0;
    for (int q = 0; q < 4; q++) {
        m->params[q][0] = att;
        m->params[q][1] = dis;
        m->params[q][2] = thetam;
    }
}

void mtg_replica_defaults(mtg_replica_desc *r) {
    std::memset(r, 0, sizeof(*r));
    r->periodic = 1;
    r->dt = 0.005;
    r->kT = 1.0;
    r->gamma = 1.0;
    r->gammar = 1.0;
    r->mass = 1.0;
    r->inertia = 0.25 * 2.0 / 5.0;
    r->hs_eps = 1.0;
    r->hs_sigma = 1.0;
    r->max_dist2 = 2.4;
    r->seed = 0;
}

mtg_status mtg_create(const mtg_config *cfg, mtg_system **out) {
    if (!cfg || !out || cfg->n_replicas < 1 || cfg->n_replicas >= (1 << 30) || !cfg->replicas) {
        g_create_error = "mtg_create: null config/output, or replica count outside [1, 2^30)";
        return MTG_ERR_ARG;
    }
    *out = nullptr;
    try {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
            cudaGetLastError();
            g_create_error = "mtg_create: no CUDA device with that ordinal";
            return MTG_ERR_NODEVICE;
        }
        cudaDeviceProp prop;
        MTG_CUDA(cudaGetDeviceProperties(&prop, cfg->device));
        if (prop.major * 10 + prop.minor != 103) {
            g_create_error = "mtg_create: this build targets sm_103a (GB300); device is sm_" +
                             std::to_string(prop.major) + std::to_string(prop.minor);
            return MTG_ERR_NODEVICE;
        }
        std::vector<mtg_replica_desc> reps(cfg->replicas, cfg->replicas + cfg->n_replicas);
        for (auto &d : reps) {
            MTG_REQUIRE(d.n >= 1, "replica: n must be >= 1");
            MTG_REQUIRE(d.box > 0 && d.dt > 0 && d.mass > 0 && d.inertia > 0 && d.kT >= 0, "replica: bad parameters");
            MTG_REQUIRE(d.gamma >= 0 && d.gammar >= 0 && d.hs_sigma > 0 && d.max_dist2 > 0, "replica: bad parameters");
            if (d.model.n_types == 1 && d.model.count_per_type[0] == 0) d.model.count_per_type[0] = d.n;
            check_model(d.model, d.n);
        }
        MTG_REQUIRE(std::isfinite(cfg->neighbor_skin) && cfg->neighbor_skin >= 0 && cfg->neighbor_skin <= 10,
                    "mtg_create: neighbor_skin must lie in [0, 10] sigma");
        mtg_config c = *cfg;
        c.replicas = reps.data();
        std::unique_ptr<mtg_system> h(new mtg_system);
        h->device = cfg->device;
        if (cfg->precision == MTG_FP64) h->impl.reset(make_sys_f64(c));
        else if (cfg->precision == MTG_FP32) h->impl.reset(make_sys_f32(c));
        else throw Fail{MTG_ERR_ARG, "mtg_create: precision must be MTG_FP32 or MTG_FP64"};
        *out = h.release();
        return MTG_OK;
    } catch (const Fail &f) {
        g_create_error = f.msg;
        return f.st;
    }
}

void mtg_destroy(mtg_system *h) { delete h; }

int64_t mtg_num_particles(const mtg_system *h) { return h ? h->impl->ntot() : 0; }
int64_t mtg_replica_offset(const mtg_system *h, int r) { return h ? h->impl->offset(r) : 0; }

mtg_status mtg_set_state(mtg_system *h, const double *x, const double *p, const double *Lb, const double *Q,
                         const double *Ft, const double *Tt) {
    MTG_GUARD(h, h->impl->set_state(x, p, Lb, Q, Ft, Tt));
    return MTG_OK;
}

mtg_status mtg_get_state(mtg_system *h, double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt) {
    MTG_GUARD(h, return h->impl->get_state(x, p, Lb, Q, Ft, Tt));
    return MTG_OK;
}

mtg_status mtg_init_forces(mtg_system *h) {
    MTG_GUARD(h, h->impl->init_forces(nullptr));
    return MTG_OK;
}

mtg_status mtg_init_forces_noise(mtg_system *h, const double *noise) {
    if (h && !noise) return MTG_ERR_ARG;
    MTG_GUARD(h, h->impl->init_forces(noise));
    return MTG_OK;
}

mtg_status mtg_set_bonds(mtg_system *h, const int32_t *bonds, int64_t nbonds, double k, double r0) {
    MTG_GUARD(h, h->impl->set_bonds(bonds, nbonds, k, r0));
    return MTG_OK;
}

int64_t mtg_neighbor_rebuilds(mtg_system *h) {
    if (!h) return 0;
    try {
        cudaSetDevice(h->device);
        return h->impl->rebuilds();
    } catch (const Fail &f) {
        h->err = f.msg;
        return 0;
    }
}

mtg_status mtg_gr(mtg_system *h, int replica, double rmax, double dr, int64_t *hist, int cap, int *nbins) {
    MTG_GUARD(h, h->impl->gr(replica, rmax, dr, hist, cap, nbins));
    return MTG_OK;
}

mtg_status mtg_clusters(mtg_system *h, int replica, double cut, int32_t *labels) {
    MTG_GUARD(h, h->impl->clusters(replica, cut, labels));
    return MTG_OK;
}

mtg_status mtg_step_profile(mtg_system *h, int nsteps, double *kernel_ms) {
    MTG_GUARD(h, h->impl->step_profile(nsteps, kernel_ms));
    return MTG_OK;
}

mtg_status mtg_step(mtg_system *h, int nsteps) {
    MTG_GUARD(h, h->impl->step(nsteps, nullptr));
    return MTG_OK;
}

mtg_status mtg_step_noise(mtg_system *h, int nsteps, const double *noise) {
    if (h && !noise) return MTG_ERR_ARG;
    MTG_GUARD(h, h->impl->step(nsteps, noise));
    return MTG_OK;
}

mtg_status mtg_forces(mtg_system *h, double *F, double *T, double *E) {
    MTG_GUARD(h, h->impl->forces(F, T, E));
    return MTG_OK;
}

mtg_status mtg_pairs(mtg_system *h, int replica, double rc, int32_t *pairs, int64_t cap, int64_t *npairs) {
    MTG_GUARD(h, return h->impl->pairs(replica, rc, pairs, cap, npairs));
    return MTG_OK;
}

mtg_status mtg_temperature(mtg_system *h, double *out) {
    MTG_GUARD(h, {
        if (!out) throw Fail{MTG_ERR_ARG, "mtg_temperature: null output"};
        if (h->impl->temperature(out) & MTG_FLAG_NONFINITE) return MTG_ERR_NONFINITE;
    });
    return MTG_OK;
}

mtg_status mtg_step_temperatures(mtg_system *h, int nsteps, double *out) {
    MTG_GUARD(h, {
        if (nsteps < 0) throw Fail{MTG_ERR_ARG, "mtg_step_temperatures: nsteps must be >= 0"};
        if (!out && nsteps > 0) throw Fail{MTG_ERR_ARG, "mtg_step_temperatures: null output"};
        if (h->impl->step_temperatures(nsteps, out) & MTG_FLAG_NONFINITE) return MTG_ERR_NONFINITE;
    });
    return MTG_OK;
}

mtg_status mtg_observables(mtg_system *h, double *out) {
    MTG_GUARD(h, {
        if (!out) throw Fail{MTG_ERR_ARG, "mtg_observables: null output"};
        h->impl->observables(out);
    });
    return MTG_OK;
}

mtg_status mtg_get_displacement(mtg_system *h, double *disp) {
    MTG_GUARD(h, {
        if (!disp) throw Fail{MTG_ERR_ARG, "mtg_get_displacement: null output"};
        h->impl->displacement(disp);
    });
    return MTG_OK;
}

uint64_t mtg_get_draw(const mtg_system *h) { return h ? h->impl->get_draw() : 0; }

mtg_status mtg_set_draw(mtg_system *h, uint64_t d) {
    MTG_GUARD(h, h->impl->set_draw(d));
    return MTG_OK;
}

mtg_status mtg_sync(mtg_system *h) {
    MTG_GUARD(h, {
        MTG_CUDA(cudaStreamSynchronize(h->impl->stream()));
        const uint32_t f = h->impl->flags();
        if (f & MTG_FLAG_TIMEOUT) throw Fail{MTG_ERR_TIMEOUT, "a bounded device wait expired"};
        if (f & MTG_FLAG_BINNING) throw Fail{MTG_ERR_STATE, "cell binning incomplete: a step was skipped"};
        if (f & MTG_FLAG_BIND) throw Fail{MTG_ERR_CAPACITY, bind_failure(f)};
        if (f & MTG_FLAG_NONFINITE) return MTG_ERR_NONFINITE;
    });
    return MTG_OK;
}

mtg_status mtg_set_single_bond(mtg_system *h, const mtg_single_bond *sb) {
    MTG_GUARD(h, h->impl->set_single_bond(sb));
    return MTG_OK;
}

int64_t mtg_num_patches(const mtg_system *h) { return h ? h->impl->num_patches() : 0; }

int64_t mtg_patch_offset(const mtg_system *h, int replica) { return h ? h->impl->patch_offset(replica) : 0; }

mtg_status mtg_set_bind_state(mtg_system *h, const int32_t *boundto, const uint8_t *isbound) {
    MTG_GUARD(h, h->impl->set_bind_state(boundto, isbound));
    return MTG_OK;
}

mtg_status mtg_get_bind_state(mtg_system *h, int32_t *boundto, uint8_t *isbound) {
    MTG_GUARD(h, h->impl->get_bind_state(boundto, isbound));
    return MTG_OK;
}

// ---- the step's phases one at a time (host arrays by global index, all replicas)

mtg_status mtg_calculateforces(mtg_system *h, double *F) {
    MTG_GUARD(h, h->impl->phase_forces(1, F, nullptr));
    return MTG_OK;
}

mtg_status mtg_calculate_forces_and_torques3D(mtg_system *h, double *F, double *T) {
    MTG_GUARD(h, {
        MTG_REQUIRE(F && T, "mtg_calculate_forces_and_torques3D: F and T are required");
        const size_t n = (size_t)h->impl->ntot();
        std::vector<double> pf(3 * n), pt(3 * n);
        h->impl->phase_forces(2, pf.data(), pt.data());
        // the reference adds the patch terms to the caller's F and T (LangevinR.cpp:1015-1030)
        for (size_t i = 0; i < 3 * n; i++) {
            F[i] += pf[i];
            T[i] += pt[i];
        }
    });
    return MTG_OK;
}

mtg_status mtg_create_forces_and_torques_sphere(mtg_system *h, double *F, double *T, const double *R) {
    MTG_GUARD(h, h->impl->phase_langevin(F, T, R));
    return MTG_OK;
}

mtg_status mtg_advancemom_halfstep(mtg_system *h, const double *F, const double *T) {
    MTG_GUARD(h, h->impl->phase_halfkick(F, T));
    return MTG_OK;
}

mtg_status mtg_advance_pos(mtg_system *h) {
    MTG_GUARD(h, h->impl->phase_drift());
    return MTG_OK;
}

mtg_status mtg_set_wait_limit(mtg_system *h, int64_t limit) {
    MTG_GUARD(h, {
        MTG_REQUIRE(limit >= 0, "mtg_set_wait_limit: limit must be >= 0");
        h->impl->set_wait_limit(limit);
    });
    return MTG_OK;
}

mtg_status mtg_get_launch_config(mtg_system *h, mtg_launch_config *out) {
    MTG_GUARD(h, {
        MTG_REQUIRE(out, "mtg_get_launch_config: out is required");
        h->impl->get_launch_config(out);
    });
    return MTG_OK;
}

mtg_status mtg_set_launch_config(mtg_system *h, const mtg_launch_config *cfg) {
    MTG_GUARD(h, {
        MTG_REQUIRE(cfg, "mtg_set_launch_config: cfg is required");
        h->impl->set_launch_config(cfg);
    });
    return MTG_OK;
}

mtg_status mtg_autotune(mtg_system *h, int steps_per_trial, mtg_launch_config *best, double *ms_per_step) {
    MTG_GUARD(h, {
        MTG_REQUIRE(best && ms_per_step, "mtg_autotune: best and ms_per_step are required");
        h->impl->autotune(steps_per_trial, best, ms_per_step);
        const uint32_t f = h->impl->flags();
        if (f & MTG_FLAG_NONFINITE) throw Fail{MTG_ERR_NONFINITE, "mtg_autotune: non-finite state during the trials"};
    });
    return MTG_OK;
}

mtg_status mtg_rotate(mtg_system *h) {
    MTG_GUARD(h, h->impl->phase_rotate());
    return MTG_OK;
}

mtg_status mtg_bind_update(mtg_system *h, double *F, double *T) {
    MTG_GUARD(h, {
        h->impl->bind_update(F, T);
        const uint32_t f = h->impl->flags();
        if (f & MTG_FLAG_BIND) throw Fail{MTG_ERR_CAPACITY, bind_failure(f)};
    });
    return MTG_OK;
}

mtg_status mtg_setup_random_binding(mtg_system *h, uint64_t seed) {
    MTG_GUARD(h, {
        h->impl->setup_random_binding(seed);
        const uint32_t f = h->impl->flags();
        if (f & MTG_FLAG_BIND) throw Fail{MTG_ERR_CAPACITY, bind_failure(f)};
    });
    return MTG_OK;
}

uint32_t mtg_flags(mtg_system *h) {
    if (!h) return 0;
    try {
        cudaSetDevice(h->device);
        return h->impl->flags();
    } catch (const Fail &f) {
        h->err = f.msg;
        return 0;
    }
}

void mtg_clear_flags(mtg_system *h) {
    if (!h) return;
    try {
        cudaSetDevice(h->device);
        h->impl->clear_flags();
    } catch (const Fail &f) {
        h->err = f.msg;
    }
}

void *mtg_stream(mtg_system *h) { return h ? (void *)h->impl->stream() : nullptr; }

int64_t mtg_launch_count(const mtg_system *h) { return h ? h->impl->launches() : 0; }

const char *mtg_last_error(const mtg_system *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

}  // extern "C"
