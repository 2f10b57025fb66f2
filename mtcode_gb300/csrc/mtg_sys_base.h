// mtg_sys_base.h -- host-side interface between the extern "C" layer and the precision-specific
// implementations (mtg_sys_f32.cu / mtg_sys_f64.cu), so each precision compiles in its own unit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mtcode_gb300.h"

namespace mtg_impl {

struct Fail {
    mtg_status st;
    std::string msg;
};

#define MTG_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            throw Fail{e_ == cudaErrorMemoryAllocation ? MTG_ERR_NOMEM : MTG_ERR_CUDA,         \
                       std::string(#call) + ": " + cudaGetErrorString(e_)};                   \
    } while (0)

#define MTG_REQUIRE(cond, msg) \
    do {                       \
        if (!(cond)) throw Fail{MTG_ERR_ARG, msg}; \
    } while (0)

struct SysBase {
    virtual ~SysBase() {}
    virtual void set_state(const double *, const double *, const double *, const double *, const double *,
                           const double *) = 0;
    virtual mtg_status get_state(double *, double *, double *, double *, double *, double *) = 0;
    virtual void init_forces(const double *noise) = 0;
    virtual void step_profile(int nsteps, double *kernel_ms) = 0;
    virtual void step(int nsteps, const double *noise) = 0;
    virtual void forces(double *, double *, double *) = 0;
    virtual void set_bonds(const int32_t *, int64_t, double, double) = 0;
    virtual void gr(int, double, double, int64_t *, int, int *) = 0;
    virtual void clusters(int, double, int32_t *) = 0;
    virtual int64_t rebuilds() = 0;
    virtual mtg_status pairs(int, double, int32_t *, int64_t, int64_t *) = 0;
    virtual uint32_t temperature(double *) = 0;   // returns the status flags, read with the result
    virtual uint32_t step_temperatures(int, double *) = 0;   // likewise
    virtual void observables(double *) = 0;
    virtual void displacement(double *) = 0;
    virtual void set_draw(uint64_t) = 0;
    virtual uint64_t get_draw() const = 0;
    virtual uint32_t flags() = 0;
    virtual void clear_flags() = 0;
    virtual cudaStream_t stream() const = 0;
    virtual int64_t launches() const = 0;
    virtual int64_t ntot() const = 0;
    virtual int64_t offset(int r) const = 0;
    virtual void set_single_bond(const mtg_single_bond *) = 0;
    virtual int64_t num_patches() const = 0;
    virtual int64_t patch_offset(int r) const = 0;
    virtual void set_bind_state(const int32_t *, const uint8_t *) = 0;
    virtual void get_bind_state(int32_t *, uint8_t *) = 0;
    virtual void bind_update(double *, double *) = 0;
    virtual void setup_random_binding(uint64_t seed) = 0;
    virtual void phase_forces(int, double *, double *) = 0;
    virtual void phase_langevin(double *, double *, const double *) = 0;
    virtual void phase_halfkick(const double *, const double *) = 0;
    virtual void phase_drift() = 0;
    virtual void phase_rotate() = 0;
    virtual void set_wait_limit(int64_t) = 0;
    virtual void get_launch_config(mtg_launch_config *) const = 0;
    virtual void set_launch_config(const mtg_launch_config *) = 0;
    virtual void autotune(int, mtg_launch_config *, double *) = 0;
};


SysBase *make_sys_f32(const mtg_config &cfg);
SysBase *make_sys_f64(const mtg_config &cfg);

}  // namespace mtg_impl
