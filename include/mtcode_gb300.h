/*
 * mtcode_gb300.h -- C ABI of the GB300 (sm_103a) rotational-Langevin step for patchy spheres.
 *
 * This is the drop-in boundary for the per-timestep hot path of osmanovicdino/mtcode: cell-list
 * construction, the WCA-core + Kern-Frenkel patch force/torque loop, and the translational and
 * rotational Langevin update.  The reference has no FFI of its own (every executable #includes the
 * C++ sources); the entry points below are what its C++ classes forward to through the header-only
 * adapter include/LangevinNVTRGPU.hpp.  Each entry point names the reference routine it replaces.
 *
 * Conventions (identical to the reference's row-major matrix<double> layout, DataStructures/matrix2.h:24-40):
 *   x, p, F   n x 3 doubles, lab frame
 *   Lb, T~    n x 3 doubles, BODY frame (angular momentum / carried torque)
 *   Q         n x 9 doubles, lab -> body rotation; patch direction in the lab frame = Q^T n_body
 *   noise     n x 6 doubles, mean 0, variance 1 (matrix2.cpp:1807-1821)
 * Several independent replicas ("systems") live in one handle; host arrays for all replicas are
 * concatenated replica after replica, each replica's rows in its own particle order.
 *
 * Errors: every call returns an mtg_status; nothing exits or reads stdin (the reference's error()
 * and pausel(), Basic/basic.h:61-99, block on stdin).  Device-side conditions (non-finite state,
 * a |pair force| above the reference's 1e4 pause threshold) are latched on the device and reported
 * by the next synchronising call (mtg_sync, mtg_get_state, mtg_temperature, ...).
 * Threading: one host thread per handle; calls are ordered on the handle's CUDA stream.
 */
#ifndef MTCODE_GB300_H
#define MTCODE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MTG_API_VERSION 5

typedef enum {
    MTG_OK = 0,
    MTG_ERR_ARG = 1,          /* invalid argument */
    MTG_ERR_CUDA = 2,         /* CUDA runtime failure (mtg_last_error has the text) */
    MTG_ERR_NOMEM = 3,        /* device allocation failed */
    MTG_ERR_STATE = 4,        /* call order violated (e.g. a step before any state was set) */
    MTG_ERR_NONFINITE = 5,    /* a position, force or torque became NaN/Inf on the device */
    MTG_ERR_CAPACITY = 6,     /* a caller buffer is too small; the size needed is returned */
    MTG_ERR_TIMEOUT = 7,      /* a bounded device-side wait expired */
    MTG_ERR_NODEVICE = 8      /* no usable sm_103 device */
} mtg_status;

typedef enum { MTG_FP32 = 0, MTG_FP64 = 1 } mtg_precision;

/* device-latched condition bits, read with mtg_flags() */
#define MTG_FLAG_NONFINITE   0x1u   /* see MTG_ERR_NONFINITE */
#define MTG_FLAG_FORCE_LIMIT 0x2u   /* some |pair force| > 1e4: where MD.cpp:1711-1749 would pausel() */
#define MTG_FLAG_TIMEOUT     0x4u   /* a bounded device wait expired (see MTG_ERR_TIMEOUT) */
#define MTG_FLAG_OVERFLOW    0x8u   /* a tile's pair list overflowed: handled by the per-particle path */
#define MTG_FLAG_BINNING     0x10u  /* the cell histogram disagreed with the particle count: step skipped */
#define MTG_FLAG_BIND        0x20u  /* single-bond mode: a capacity was exceeded or a cluster reached one of
                                       the reference's error() paths; one of the reasons below is set too */
#define MTG_BIND_WHY_ADJ     0x10000u  /* a patch had more than 8 candidate partners in one update */
#define MTG_BIND_WHY_CLUSTER 0x20000u  /* a patch cluster had more than 128 patches */
#define MTG_BIND_WHY_LIST    0x40000u  /* a list of the force pass (pairs, patches, bound pairs) was full */
#define MTG_BIND_WHY_REF     0x80000u  /* a cluster reached one of the reference's error() paths */
#define MTG_BIND_WHY_SPIN    0x100000u /* an atomic retry loop reached its bound */

typedef struct mtg_system mtg_system;

/* Patch model in GeneralPatch form (MDBase/Potentials/ComboPatch/GeneralPatch.cpp:7-121).
 * TetrahedralPatch(att, dis, thetam) (TetrahedralPatch.cpp:4-44) and BivalentPatch
 * (BivalentPatch.cpp:4-34) are one-type special cases; mtg_model_tetrahedral / mtg_model_bivalent
 * fill this struct for them.  Potentials are ordered type pair (k1 <= k2), then patch of k1, then
 * patch of k2, exactly as GeneralPatch enumerates potential_bundle. */
#define MTG_MAX_TYPES 4
#define MTG_MAX_ORIENT 16
#define MTG_MAX_POTS 64
typedef struct {
    int n_types;
    int patches_per_type[MTG_MAX_TYPES];
    int count_per_type[MTG_MAX_TYPES];    /* cumulative particle counts (GeneralPatch num_per_type) */
    double orient[MTG_MAX_ORIENT][3];     /* body-frame patch unit vectors, types contiguous */
    double params[MTG_MAX_POTS][3];       /* (att, dis, thetam) per potential (KernFrenkelOnePatch2) */
} mtg_patch_model;

/* One independent system: cube(box, pb, 3) + LangevinNVTR parameters + HSPotential + ComboPatch. */
typedef struct {
    int n;                 /* particles */
    double box;            /* cube::l */
    int periodic;          /* 1: periodic (all three axes); 0: reflecting walls */
    double dt;             /* LangevinNVTR::setdt */
    double kT;             /* setkT */
    double gamma;          /* setgamma   (translational friction) */
    double gammar;         /* setgammar  (rotational friction) */
    double mass;           /* LangevinNVT::m (reference default 1) */
    double inertia;        /* isotropic moment of inertia (reference default 0.25*2/5 = 0.1) */
    double hs_eps;         /* HSPotential(eps, sigma): WCA core, potential.h:79-162 */
    double hs_sigma;
    double max_dist2;      /* LangevinNVTR::max_distance_check (reference default 2.4) */
    uint64_t seed;         /* Philox key of this replica's noise stream */
    mtg_patch_model model;
} mtg_replica_desc;

typedef struct {
    int precision;                     /* mtg_precision */
    int n_replicas;
    const mtg_replica_desc *replicas;
    int device;                        /* CUDA device ordinal */
    int track_displacement;            /* 1: keep FP64 unwrapped-displacement accumulators */
    int force_kernel;                  /* 0 = pair pipeline (default, both precisions: pair list, one thread
                                              per pair, per-particle epilogue; FP32 sums in order-independent
                                              fixed point, FP64 sums by double atomics), 1 = one thread per
                                              particle, 2 = tiled shared-memory kernel (FP32 only; an FP64
                                              handle asking for it gets MTG_ERR_ARG) */
    double neighbor_skin;              /* 0 (default): the cell list is rebuilt every step.  > 0: Verlet
                                          skin (sigma): cells and per-particle candidate lists are built at
                                          force range + skin and reused until some particle has moved more
                                          than skin / 2 since the build -- the reference's pair reuse
                                          (Condensate.cpp:344-350) with an exactness check instead of a
                                          fixed 20-step schedule.  The force set is the same either way. */
} mtg_config;

/* Fill `m` with TetrahedralPatch(att, dis, thetam) / BivalentPatch(att, dis, thetam). */
void mtg_model_tetrahedral(mtg_patch_model *m, double att, double dis, double thetam);
void mtg_model_bivalent(mtg_patch_model *m, double att, double dis, double thetam);
/* Reference defaults: dt 0.005, kT 1, gamma = gammar = 1, m 1, I 0.1, HS(1,1), max_dist2 2.4. */
void mtg_replica_defaults(mtg_replica_desc *r);

/* Create / destroy a handle.  Replaces constructing LangevinNVTR(cube&) + setdt/setkT/setgamma/
 * setgammar (LangevinR.cpp:41-69, LangevinR.h:109-134) and binding a ComboPatch. */
mtg_status mtg_create(const mtg_config *cfg, mtg_system **out);
void mtg_destroy(mtg_system *h);

/* Total particles over all replicas; particle offset of replica r. */
int64_t mtg_num_particles(const mtg_system *h);
int64_t mtg_replica_offset(const mtg_system *h, int replica);

/* LangevinNVTR::initialize(x, p, Q, Lb) (LangevinR.cpp:309-325) for all replicas at once.
 * Ft/Tt (the carried F~ lab / T~ body of Condensate::run) may be NULL: they are then zero and
 * mtg_init_forces() should be called before the first step. */
mtg_status mtg_set_state(mtg_system *h, const double *x, const double *p, const double *Lb, const double *Q,
                         const double *Ft, const double *Tt);
/* getdat/getmom/getangmom/getorientation (LangevinR.h:190-196) + the carried F~, T~; any may be NULL. */
mtg_status mtg_get_state(mtg_system *h, double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt);

/* Condensate.cpp:312-334: F = calculateforces(HS) + calculate_forces_and_torques3D(ComboPatch),
 * then create_forces_and_torques_sphere(F, T, one noise draw) -> carried F~, T~. */
mtg_status mtg_init_forces(mtg_system *h);
/* Same, with the noise of that draw supplied by the caller (total particles x 6, host memory):
 * create_forces_and_torques_sphere(F, T, RT) with the caller's RT (LangevinR.cpp:580-592). */
mtg_status mtg_init_forces_noise(mtg_system *h, const double *noise);

/* nsteps of the Condensate::run loop body (Condensate.cpp:335-378) with counter-based Philox noise:
 * advancemom_halfstep -> advance_pos -> rotate -> cell list -> forces+torques -> noise+friction
 * (create_forces_and_torques_sphere) -> advancemom_halfstep.  The cell list is rebuilt every step
 * and covers every pair within the force range exactly.  Asynchronous. */
mtg_status mtg_step(mtg_system *h, int nsteps);
/* Same, with the noise supplied by the caller instead of Philox: noise holds nsteps blocks of
 * (total particles x 6) values, replaces generate_uniform_random_matrix (matrix2.cpp:1807-1821). */
mtg_status mtg_step_noise(mtg_system *h, int nsteps, const double *noise);

/* Forces at the current state without advancing it:
 * F = MD::calculateforces(pairs, HSPotential) (MD.cpp:1684-1764) plus the patch forces, and
 * T = the lab-frame torques of LangevinNVTR::calculate_forces_and_torques3D (LangevinR.cpp:911-1047).
 * energy (nullable): per-particle potential energy, half of every pair energy (WCA + KF2). */
mtg_status mtg_forces(mtg_system *h, double *F, double *T, double *energy);

/* The loop body one phase at a time, for a driver that keeps Condensate::run's loop (Condensate.cpp:335-378)
 * and swaps its calls one by one.  Host arrays hold all replicas by global index (n x 3 doubles unless
 * stated); each call runs on the handle's state, synchronises, and matches the fused mtg_step's arithmetic.
 * The force calls take no pair list: the handle's cell list finds every pair within the force range, which is
 * the pair set of a caller's list that covers that range.
 *
 * MD::calculateforces(pairs, HSPotential) (MD.cpp:1684-1764): F = the WCA core forces (plus the harmonic
 * bonds of mtg_set_bonds), overwritten. */
mtg_status mtg_calculateforces(mtg_system *h, double *F);
/* LangevinNVTR::calculate_forces_and_torques3D(pairs, ComboPatch, F, T) (LangevinR.cpp:911-1047): ADDS the
 * Kern-Frenkel patch forces to F and the lab-frame torques to T, as the reference does (in single-bond mode:
 * the bound pairs' forces and torques). */
mtg_status mtg_calculate_forces_and_torques3D(mtg_system *h, double *F, double *T);
/* LangevinNVTR::create_forces_and_torques_sphere(F, T, R) (LangevinR.cpp:474-592): F (lab) and T (lab) in,
 * F~ = F + friction + noise (lab) and T~ (BODY frame) out, in place.  R: n x 6 noise (matrix2.cpp:1807-1821),
 * or NULL for the handle's Philox noise of the next draw.  F~ and T~ also become the handle's carried
 * forces, which mtg_step's first half-kick uses. */
mtg_status mtg_create_forces_and_torques_sphere(mtg_system *h, double *F, double *T, const double *R);
/* LangevinNVTR::advancemom_halfstep(F, T) (LangevinR.cpp:327-347): p += dt/2 F (F lab), L += dt/2 T (T body). */
mtg_status mtg_advancemom_halfstep(mtg_system *h, const double *F, const double *T);
/* LangevinNVT::advance_pos() (Langevin.cpp:205-222): x += (dt/m) p, then wrap (periodic) or reflect with p
 * negated (walls), cube::correct_position_and_momentum (geometry.h:403-446). */
mtg_status mtg_advance_pos(mtg_system *h);
/* LangevinNVTR::rotate() (LangevinR.cpp:594-695): the free-rotor propagator genfullmat (:392-461) applied to
 * L (L <- R L) and the orientation (Q <- R^T Q). */
mtg_status mtg_rotate(mtg_system *h);

/* Fixed bonds with HarmonicPotential(k, r0) (MDBase/Potentials/potential.h:265-297): from now on every
 * force pass adds MD::calculateforces(bonds, pot) (MD.cpp:1684-1764), f = -k (r - r0) along the
 * minimum-image separation, to the central forces -- the bonded term of the polymer drivers
 * (mainActivePolymer.cpp:390-402).  bonds: nbonds x 2 host-order (global) particle indices, both ends
 * in one replica; nbonds = 0 removes them.  mtg_forces' energy then includes 0.5 k (r - r0)^2 per bond
 * (half to each end); mtg_observables does not.  Call mtg_init_forces after changing bonds mid-run. */
mtg_status mtg_set_bonds(mtg_system *h, const int32_t *bonds, int64_t nbonds, double k, double r0);

/* MD::calculatepairs_parallel(boxlist, rc) (MD.cpp:1100-1176) for one replica: every pair (i < j,
 * local indices) with minimum-image distance < rc, sorted by (i, j).  The cell grid is rebuilt at
 * side >= rc for this call.  If *npairs > cap on return, nothing beyond cap was written and the call
 * returns MTG_ERR_CAPACITY. */
mtg_status mtg_pairs(mtg_system *h, int replica, double rc, int32_t *pairs, int64_t cap, int64_t *npairs);

/* LangevinNVTR::measured_temperature (LangevinR.cpp:170-193), per replica: 6 doubles
 * (<p_k^2/2m>, <L_k^2/2I>, k = x,y,z).  out: n_replicas x 6. Synchronising. */
mtg_status mtg_temperature(mtg_system *h, double *out);

/* nsteps steps of mtg_step, each followed by mtg_temperature's per-replica sums of that step, as
 * Condensate::run measures the temperature every step (Condensate.cpp:335-378).  Every step's sums stay
 * on the device (a ring of at most 32 MB) and are copied to pinned host memory once per chunk of steps (no
 * host round trip between steps); the call synchronises once at the end.  out: nsteps x n_replicas x 6,
 * step-major.  The copies land in a pinned staging buffer of the same size (kept for later calls): for
 * long runs, call it in blocks of steps.  A failed allocation returns MTG_ERR_CUDA. */
mtg_status mtg_step_temperatures(mtg_system *h, int nsteps, double *out);

/* Per-replica FP64 observables at the current state, out: n_replicas x MTG_OBS_COUNT:
 *  [0] KF2 patch energy, [1] WCA energy (+eps shifted, r < 1.12246 sigma), [2] virial sum r.f,
 *  [3] bonded patch pairs (LangevinNVTR::calculate_bound_pairs criterion, LangevinR.cpp:1854-1998),
 *  [4] pairs within the force range.  Synchronising. */
#define MTG_OBS_COUNT 5
mtg_status mtg_observables(mtg_system *h, double *out);

/* calcg1(data, geo, rmax, dr) (MDBase/Analysis/PairCorrelation.cpp:9-153) for one replica at the
 * current state: counts of unordered pair distances (cube::distance, geometry.h:107-121, FP64) in bins
 * floor(r / dr) < nbins = floor(rmax / dr).  *nbins receives the bin count; hist (cap >= nbins
 * entries, or null to ask for the count) the counts.  rmax must not exceed the box side.  Synchronising. */
mtg_status mtg_gr(mtg_system *h, int replica, double rmax, double dr, int64_t *hist, int cap, int *nbins);

/* distance_graph(pos, boxes, geo, cut, index_test) (MDBase/Analysis/AnalyzeGrowth.cpp:136-171) for one
 * replica: labels[i] (local index i) = the smallest local index of i's connected component in the graph
 * of pairs closer than cut, the labels ConnectedComponentsParallel_Old (Bindings/GraphAlgorithms.cpp:
 * 672-800) converges to.  Synchronising. */
mtg_status mtg_clusters(mtg_system *h, int replica, double cut, int32_t *labels);

/* Launch shapes of the pair pipeline (force_kernel 0).  Every shape computes the same FP32 forces bit for bit
 * (the sums are fixed point), so the shapes only change speed.  The reference has no counterpart: its one
 * tuning knob is the pair-list rebuild interval (Condensate.cpp:344-350). */
typedef struct {
    int pairfind_threads;          /* pair finding, one thread per particle: 128, 256 (default) or 512 */
    int pairforce_blocks_per_sm;   /* grid of the grid-stride pair-force kernel, blocks of 256 per SM: 1..64 (16) */
    int patch_blocks_per_sm;       /* grid of the patch-pair (single-bond: edge) kernel per SM: 1..64 (8) */
    int epilogue_threads;          /* per-particle epilogue: 128, 256 (default) or 512 */
    int fused_pairs;               /* 1 (default): pair finding also evaluates the WCA core and the cone pre-test
                                      of the pairs it finds, in the same kernel, and writes no pair list (steps
                                      without a neighbour skin; in single-bond mode also the bond pass's pair
                                      stage); 0: separate pair list and pair-force kernel */
} mtg_launch_config;
mtg_status mtg_get_launch_config(mtg_system *h, mtg_launch_config *out);
/* Sets the shapes; the step graphs are captured again at the next step. */
mtg_status mtg_set_launch_config(mtg_system *h, const mtg_launch_config *cfg);
/* Autotuner: coordinate descent over the shapes above (two sweeps), each candidate timed with CUDA events on
 * steps_per_trial steps of the current state -- the trials are real steps and advance the simulation (about
 * 20 x steps_per_trial steps in all).  The fastest shape stays set and is returned with its time per step.
 * A handle without the pair pipeline returns its time per step and the unchanged shapes.  Synchronising. */
mtg_status mtg_autotune(mtg_system *h, int steps_per_trial, mtg_launch_config *best, double *ms_per_step);

/* Bound on the device loops of mtg_clusters that wait on other threads' progress (each union-find parent walk
 * and the compare-and-swap retries of one hook): at most `limit` iterations.  0 (the default) restores their
 * own bound, n + 1, which always suffices.  A loop that reaches its bound stops and latches MTG_FLAG_TIMEOUT,
 * its kernel returns normally, and mtg_clusters reports MTG_ERR_TIMEOUT; the handle stays usable.  (The tile
 * kernel's pipeline waits keep their own fixed bound.) */
mtg_status mtg_set_wait_limit(mtg_system *h, int64_t limit);

/* FP64 unwrapped displacement accumulated since the last mtg_set_state (total particles x 3). */
mtg_status mtg_get_displacement(mtg_system *h, double *disp);

/* Number of noise draws consumed so far (mtg_init_forces and every step each consume one);
 * set it to resume a run bit-reproducibly. */
uint64_t mtg_get_draw(const mtg_system *h);
mtg_status mtg_set_draw(mtg_system *h, uint64_t draw);

/* Waits for the handle's stream and reports latched device conditions. */
mtg_status mtg_sync(mtg_system *h);
uint32_t mtg_flags(mtg_system *h);
void mtg_clear_flags(mtg_system *h);

/* The handle's cudaStream_t (as void*). */
void *mtg_stream(mtg_system *h);

/* Kernel launches issued on this handle so far (every entry point counts its own launches). */
int64_t mtg_launch_count(const mtg_system *h);

/* Instrumented steps: nsteps of mtg_step launched one kernel at a time (no graph) with CUDA events
 * around every launch on the handle's stream.  kernel_ms[k] receives the summed device time of
 * kernel k over the nsteps, for k = 0 scan_reduce, 1 scan_top, 2 scan_down, 3 scatter (reorder +
 * first half-step), 4 force (force/torque + Langevin epilogue + next binning), and in single-bond mode
 * 5 bind_begin (the update's start; the edges are part of the force pass), 6 bind_decide (clusters and
 * bond decisions).  With a neighbour skin: 0 = rebuild decision + binning + scan_reduce, 1 scan_top,
 * 2 scan_down, 3 scatter + copy-back (rebuild steps) + in-place first half-step (other steps), 4 force.
 * With the FP32 pair pipeline, 7..10 split slot 4 by kernel: 7 pair reset + pairfind, 8 pairforce,
 * 9 patch pairs (single-bond mode: edges + bound pairs, without slot 6's decisions), 10 epilogue; zero
 * otherwise.  Slots 5 and 6 are zero outside single-bond mode.  Synchronising. */
#define MTG_PROFILE_KERNELS 11
mtg_status mtg_step_profile(mtg_system *h, int nsteps, double *kernel_ms);

/* With a neighbour skin: list rebuilds since mtg_create (each initial force pass and each step that
 * rebuilt); 0 without a skin.  Synchronising. */
int64_t mtg_neighbor_rebuilds(mtg_system *h);

/* Text of the last error on this handle (or of the last failed mtg_create when h is NULL). */
const char *mtg_last_error(const mtg_system *h);
const char *mtg_status_string(int status);
int mtg_api_version(void);

/* ---------------------------------------------------------------- single-bond-per-patch mode
 * Condensate::run_singlebond (Condensate/Condensate.cpp:422-618): every patch holds at most one bond.  Each
 * force pass runs LangevinNVTR::calculate_forces_and_torques3D_onlyone_nonlets (MDBase/Rotational/
 * LangevinRforce.cpp:2874-4030): candidate patch pairs that pass the distance and cone tests become edges,
 * bonds whose partner is no longer a candidate break, and each connected cluster of patches is resolved by
 * the binding model (one bond per patch); only bound pairs then exert the Kern-Frenkel force and torque,
 * on top of the WCA core (and any harmonic bonds).  The candidate list (LangevinNVTR::calculate_patch_list,
 * LangevinR.cpp:1702-1852) is rebuilt every patch_every steps.  Patches are numbered per replica as
 * GeneralPatch numbers them (GeneralPatch.cpp:285-320; TetrahedralPatch: 4 i + k).
 * Binding decisions draw counter-based Philox numbers keyed by (replica seed, draw index, cluster's
 * smallest patch, decision number), the same draw index as the step's noise. */

/* Binding model in table form (MDBase/Bindings).  species_rule: the species of a patch index --
 *   0 one species (BindingModelSingle), 1 index < div1 ? 1 : 2 (BindingModelBinary),
 *   2 SortingFunctionUniform (1 below div1, 2 below div2, else 3), 3 SortingFunctionNonUniform
 *   (as 2, but past div2 only every np-th patch, (index - div2) % np == np - 1, is species 3, the rest 1)
 *   (BindingModelTernary.h:6-30).
 * drate rows: species pairs 11, 12, 13, 22, 23, 33 (doubr**): [before * 2 + 0] = rate to unbound,
 *   [before * 2 + 1] = rate to bound, before = the pair was bound to each other.
 * trate rows: sorted species triples 111, 112, 113, 122, 123, 133, 222, 223, 233, 333 (tripr***):
 *   [state * 4 + k], state 0..3 = bound 12 / 23 / 13 / none, k = to 12 / 23 / 13 / none.
 * A BindingModelTernary's tables are its own rate vectors; mtg_binding_single and
 * mtg_binding_binary_equilibrium fill the table form of the other two models. */
typedef struct {
    int species_rule;
    int div1, div2, np;
    double drate[6][4];
    double trate[10][16];
} mtg_binding_model;

/* BindingModelSingle(on_rate, off_rate) (Bindings/BindingModelSingle.cpp). */
void mtg_binding_single(mtg_binding_model *m, double on_rate, double off_rate);
/* BindingModelBinary(div) + setup_equilibrium() (Bindings/BindingModelBinary.cpp); its 122 and 222 triplets
 * take the rate to none-bound from tripr111, as the reference's triplet does. */
void mtg_binding_binary_equilibrium(mtg_binding_model *m, int div);

typedef struct {
    mtg_binding_model model;
    double max_ang;     /* ComboPatch::max_ang of the candidate cone test; NAN: GeneralPatch's value,
                           min(0.6, cos thetam) over the potentials (TetrahedralPatch / BivalentPatch keep
                           0.6, combopatch.h:15) */
    double list_cut;    /* candidates come from particle pairs closer than min(list_cut, max_check + 1);
                           run_singlebond builds its pair list at 2.5 sigma */
    int patch_every;    /* candidate list rebuilt every patch_every steps (run_singlebond: 10) */
} mtg_single_bond;

/* max_ang NAN, list_cut 2.5, patch_every 10, model = BindingModelSingle(1, 0). */
void mtg_single_bond_defaults(mtg_single_bond *sb);

/* Switch a handle to single-bond mode (sb non-null) or back to the full Kern-Frenkel force (sb null).
 * Needs the pair pipeline or the per-particle force kernel and no neighbour skin.  The bond state starts
 * all unbound; mtg_init_forces (or the first step) then runs the initial force pass of run_singlebond,
 * which also decides the first bonds. */
mtg_status mtg_set_single_bond(mtg_system *h, const mtg_single_bond *sb);
/* Patches over all replicas, and the first patch of a replica (bond-state arrays are concatenated
 * replica after replica, each replica's patches in its own numbering). */
int64_t mtg_num_patches(const mtg_system *h);
int64_t mtg_patch_offset(const mtg_system *h, int replica);
/* BinaryBindStore (Bindings/BinaryBindStore.h): boundto (replica-local patch index of the partner) and
 * isbound (0 / 1) of every patch.  Setting it marks the candidate list for a rebuild at the next pass. */
mtg_status mtg_set_bind_state(mtg_system *h, const int32_t *boundto, const uint8_t *isbound);
mtg_status mtg_get_bind_state(mtg_system *h, int32_t *boundto, uint8_t *isbound);
/* One calculate_forces_and_torques3D_onlyone_nonlets pass at the current state, as run_singlebond's first
 * call makes it: candidate list rebuilt, bonds decided (consuming one draw index), then F = WCA core
 * (+ harmonic bonds) + bound-pair forces and T = bound-pair torques (lab), either nullable.  The state
 * does not move.  Synchronising. */
mtg_status mtg_bind_update(mtg_system *h, double *F, double *T);
/* LangevinNVTR::setup_random_binding(pairs, divs, iny, bo, bm) (MDBase/Rotational/LangevinRforceUtil.cpp:749-1010,
 * called by run_singlebond before its loop, Condensate.cpp:484): the candidate list of the current state, every
 * candidate that passes the edge test as an edge with score scr1 + scr2 + scr3 - log(1e-10 + calculate_score),
 * and the edges taken in a random order, each binding both patches when both are unbound and its score is below
 * 4.  The reference draws the order from std::random_device; here it is ascending Philox4x32-10 priority of the
 * replica-local patch pair (counter (lower patch, higher patch, replica, 0x53455455), key seed), ties by the
 * lower then the higher patch -- reproducible for a seed.  Bonds already in the state stay.  The state does not
 * move; the next force pass recomputes the forces.  Synchronising. */
mtg_status mtg_setup_random_binding(mtg_system *h, uint64_t seed);

/* Neighbour-pair build that allocates no device memory.  It has no counterpart in the reference.
 * It is for callers that cannot allocate device memory when they need the pair list: code that runs
 * inside another framework's memory pool or allocator hooks, or a host application that reserves the
 * device memory up front and forbids allocations inside its step loop.  Inputs and outputs are the
 * caller's DEVICE buffers: x_dev (n x 3 doubles, row-major), pairs_dev (room for cap pairs of two
 * int32, i < j, unordered) and npairs_dev (one int64: the number of pairs within rc, which may exceed
 * cap; only the first cap are written).  Work is queued on `stream` (a cudaStream_t, NULL for the
 * default stream); results are ready when the stream is.  The inclusion test is the reference's
 * cube::distance_less_than, so the set equals mtg_pairs on the same coordinates.
 * Scratch lives in one fixed array inside the library (a file-scope device array, held by every GPU
 * that loads the library until the process exits), which limits a call to
 * n <= MTG_NOALLOC_MAX_PARTICLES and (floor(box / rc))^3 <= MTG_NOALLOC_MAX_CELLS; larger calls return
 * MTG_ERR_ARG without touching the device.  The array takes 1,836,544 bytes of device memory.  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress) and should come before any
 * stream capture; the address is kept, so do not call this across cudaDeviceReset of that device.  Every
 * call shares the one array: calls that overlap on the GPU (different streams, or host threads sharing a
 * device) race. */
#define MTG_NOALLOC_MAX_PARTICLES 65536
#define MTG_NOALLOC_MAX_CELLS 65536
mtg_status mtg_pairs_noalloc(const double *x_dev, int n, double box, int periodic, double rc, int32_t *pairs_dev,
                             int64_t cap, int64_t *npairs_dev, void *stream);

/* Host-side seeded synthetic inputs (no GPU use).
 * mtg_random_positions: uniform in [0, box)^3 with non-overlap rejection at min_dist (minimum image
 * when periodic); returns MTG_ERR_ARG if the packing cannot be reached in 1000*n attempts.
 * mtg_random_rotations: uniform random rotations, the construction of LangevinR.cpp:239-267. */
mtg_status mtg_random_positions(int n, double box, int periodic, double min_dist, uint64_t seed, double *x);
void mtg_random_rotations(int n, uint64_t seed, double *Q);
/* mtg_random_chains: n_chains self-avoiding random-walk chains of `beads` beads (bond length step,
 * every bead at least min_dist from all others, minimum image), chain c's bead b at row c*beads + b of
 * x: the random-walk start of the bonded-polymer workloads.  MTG_ERR_ARG if a chain cannot be placed. */
mtg_status mtg_random_chains(int n_chains, int beads, double box, int periodic, double step, double min_dist,
                             uint64_t seed, double *x);

/* Frame files in the reference's format (no GPU use).
 * mtg_csv_write: rows x cols row-major doubles as matrix::operator<<= writes them (matrix2.cpp:898-912):
 *   ',' between values, '\n' after each row, each value as an ostream prints a double (%g).
 * mtg_csv_read: importcsv (matrix2.cpp:1597-1640): rows from lines, atof per ','-cell, short rows padded
 *   with 0.  *rows / *cols receive the shape; with a null a only the shape is read; MTG_ERR_CAPACITY if
 *   rows * cols > cap.
 * mtg_frame_name: Condensate::run's frame names (Condensate.cpp:296-300, 383-405), e.g. kind "pos" or
 *   "orientation": kind + strbase + "_i=" + frame zero-padded to the digits of ceil(runtime/every)
 *   + ".csv".  Writes at most cap bytes (snprintf) and returns the full length, -1 on bad arguments. */
mtg_status mtg_csv_write(const char *path, const double *a, int64_t rows, int cols);
mtg_status mtg_csv_read(const char *path, double *a, int64_t cap, int64_t *rows, int *cols);
int mtg_frame_name(char *out, int cap, const char *kind, const char *strbase, int frame, int runtime, int every);

#ifdef __cplusplus
}
#endif
#endif /* MTCODE_GB300_H */
