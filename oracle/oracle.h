/*
 * oracle.h -- CPU restatement (FP64) of the mtcode rotational-Langevin step for patchy spheres.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may load it.  The product
 * (mtcode_gb300/) never calls into it and has no CPU fallback.
 *
 * Parity pinning: every routine here is compared, bit for bit on x86-64, against the reference's own
 * routines compiled from the reference sources (oracle/ref_driver.cpp -> oracle/_ref/libmtref.so) on
 * the golden inputs committed under tests/golden/ (see tests/test_oracle_golden.py).
 *
 * Conventions follow the reference (units sigma = epsilon = m = 1):
 *   x, p, Lb, F, T : row-major n x 3 doubles (Lb and the carried torque are BODY frame)
 *   Q              : row-major n x 9 doubles, lab -> body rotation (patch in lab frame = Q^T n_body)
 *   pairs          : row-major np x 2 ints
 */
#ifndef MTG_ORACLE_H
#define MTG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_TYPES 8
#define ORC_MAX_ORIENT 64
#define ORC_MAX_POTS 2048

/* GeneralPatch-shaped patch model (MDBase/Potentials/ComboPatch/GeneralPatch.cpp:7-121).
 * TetrahedralPatch (TetrahedralPatch.cpp:4-44) is one type with the four tetrahedral vectors and 16
 * identical potentials; BivalentPatch (BivalentPatch.cpp:4-34) is one type with -x/+x and 4 potentials.
 * Potentials are enumerated type pair (k1 <= k2), then patch of k1, then patch of k2. */
typedef struct {
    int n_types;
    int patches_per_type[ORC_MAX_TYPES];
    int num_per_type[ORC_MAX_TYPES];      /* cumulative particle counts (particle i has type k if i < num_per_type[k]) */
    double orient[ORC_MAX_ORIENT][3];     /* body-frame patch unit vectors, types contiguous */
    int n_pots;
    double att[ORC_MAX_POTS];             /* KernFrenkelOnePatch2::att */
    double dis[ORC_MAX_POTS];             /* KernFrenkelOnePatch2::dis */
    double thetam[ORC_MAX_POTS];          /* KernFrenkelOnePatch2::thetam */
} orc_model;

typedef struct {
    int n;
    double box;          /* cube::l */
    int periodic;        /* cube::periodic */
    double dt, kT, gamma, gammar, mass, inertia;
    double hs_eps, hs_sigma;   /* HSPotential(eps, sigma) */
    double max_dist2;          /* LangevinNVTR::max_distance_check (squared distance) */
    const orc_model *model;
    /* fixed bond list (nbonds x 2 particle indices) with HarmonicPotential(bond_k, bond_r0)
     * (MDBase/Potentials/potential.h:265-297); nbonds = 0 for none */
    const int *bonds;
    long nbonds;
    double bond_k, bond_r0;
} orc_params;

/* geometry.h:508-520 */
int orc_assign_box(const double *xrow, int n, double box);
/* geometry.h:523-608: sorted, de-duplicated 27-cell stencil of cell c; returns its length */
int orc_neighbor_cells(int c, int n, int *out);
/* MD.cpp:1035-1098 + 715-869 (serial order). Returns the number of pairs (may exceed cap: then
 * only the first cap pairs are written). */
long orc_pairs(const orc_params *P, const double *x, int ncell, double rc, int *pairs, long cap);

/* MD.cpp:1684-1764 with HSPotential::force (potential.h:106-118). F is overwritten. */
void orc_hs_forces(const orc_params *P, const double *x, const int *pairs, long np, double *F);
/* MD.cpp:1684-1764 over the bond list with HarmonicPotential::force (potential.h:274-276):
 * f = -k (r - r0) along x_p1 - x_p2.  F is overwritten. */
void orc_bond_forces(const orc_params *P, const double *x, const int *bonds, long nb, double k, double r0, double *F);
/* The central forces a bonded driver sums (mainActivePolymer.cpp:390-402 pattern): F = bond forces,
 * then F += HS forces over the pairs (the HS part alone when P has no bonds).  F is overwritten. */
void orc_central_forces(const orc_params *P, const double *x, const int *pairs, long np, double *F);
/* LangevinR.cpp:911-1047 with KernFrenkelOnePatch2::force_and_torque (potentialtheta.h:517-750).
 * Adds into F and T (lab frame). */
void orc_patch_forces(const orc_params *P, const double *x, const double *Q, const int *pairs, long np,
                      double *F, double *T);
/* one KernFrenkelOnePatch2::force_and_torque evaluation, exposed for unit tests */
void orc_kf2_force_torque(const double nb1[3], const double nb2[3], double att, double dis, double thetam,
                          const double un[3], double rij, const double *Qi, const double *Qj, double out9[9]);

/* LangevinR.cpp:474-592: F <- F + Q^T(-(gamma/m) Q p + Rt xi[0:3]);  T <- -(gammar/I) Lb + Rr xi[3:6] + Q T */
void orc_langevin_forces(const orc_params *P, const double *p, const double *Lb, const double *Q,
                         const double *noise, double *F, double *T);
/* LangevinR.cpp:327-347 */
void orc_halfkick(int n, double dt, double *p, double *Lb, const double *F, const double *T);
/* Langevin.cpp:205-222 then geometry.h:403-446 */
void orc_drift(const orc_params *P, double *x, double *p);
/* LangevinR.cpp:392-461 (genfullmat) and 594-695 (rotate) */
void orc_rotation_matrix(double dt, double inertia, const double L[3], double R[9]);
void orc_rotate(const orc_params *P, double *Lb, double *Q);
/* LangevinR.cpp:170-193: per-axis <p^2/2m>, <L^2/2I> */
void orc_temperature(const orc_params *P, const double *p, const double *Lb, double out6[6]);

/* Philox4x32-10 (Salmon et al., SC'11 "Parallel random numbers: as easy as 1, 2, 3"). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* The noise draw the CUDA path uses: for particle i (local index), replica r, draw d:
 *   ctr = {i, d_lo, d_hi, 2r + blk}, key = {seed_lo, seed_hi}, 8 words -> the first 6 give
 *   xi = 3.464101615 * u - 1.732050808 with u = (w >> 8) * 2^-24   (matrix2.cpp:1807-1821 shape) */
void orc_philox_noise(int n, uint64_t seed, uint32_t replica, uint64_t draw, double *noise);

/* Energy and bookkeeping observables over all pairs within range:
 *   out[0] = KF2 patch energy (potentialtheta.h:448-515 form),
 *   out[1] = WCA energy 4e[(s/r)^12-(s/r)^6]+e for r < 1.12246 s (HSPotential force range),
 *   out[2] = virial sum r_ij . f_ij (central + patch forces),
 *   out[3] = number of bonded patch pairs (LangevinR.cpp:1854-1998 criterion, max_check = max 1.4 dis). */
void orc_observables(const orc_params *P, const double *x, const double *Q, const int *pairs, long np,
                     double out[4]);

/* calcg1(data, geo, max, dx) (MDBase/Analysis/PairCorrelation.cpp:9-153): histogram of the distances
 * of all unordered pairs, cube::distance (geometry.h:107-121), bin floor(r / dx) for the
 * floor(max / dx) bins.  Returns the bin count (hist receives at most cap bins). */
int orc_gr(const orc_params *P, const double *x, double max, double dx, long *hist, int cap);
/* distance_graph(pos, boxes, geo, cut, index_test) (MDBase/Analysis/AnalyzeGrowth.cpp:136-171):
 * connected components of the graph of pairs closer than cut (the calculatepairs_parallel set);
 * ConnectedComponentsParallel_Old (Bindings/GraphAlgorithms.cpp:672-800) converges to the smallest
 * particle index of each component, which labels[i] receives. */
void orc_clusters(const orc_params *P, const double *x, double cut, int *labels);

/* Full forces as the driver computes them: F = (bond forces +) HS forces + patch forces;
 * T = patch torques (lab). */
void orc_forces(const orc_params *P, const double *x, const double *Q, int ncell, double rc,
                double *F, double *T);

/* Condensate.cpp:312-334: initial F~, T~ from the current state and one noise draw. */
void orc_init_forces(const orc_params *P, const double *x, const double *p, const double *Lb, const double *Q,
                     int ncell, double rc, const double *noise, double *Ft, double *Tt);

/* Condensate.cpp:335-378 loop body, nsteps times, pairs rebuilt every `rebuild` steps at (ncell, rc)
 * from the positions at the start of the step.  noise_mode: 0 = xi = 0, 1 = external array
 * (nsteps x n x 6), 2 = Philox(seed, replica, draw0 + step).  With check_skin, returns -1 if a pair
 * came within the force range without being in the (stale) pair list -- the skin was too small. */
int orc_run(const orc_params *P, double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt,
            int nsteps, int ncell, double rc, int rebuild, int noise_mode, const double *noise,
            uint64_t seed, uint32_t replica, uint64_t draw0, int check_skin);

/* ---------------------------------------------------------------- single-bond-per-patch mode
 * Condensate::run_singlebond (Condensate/Condensate.cpp:422-618). */

/* Binding model in table form.  rule: species of a patch index -- 0: one species (BindingModelSingle),
 * 1: index < div1 ? 1 : 2 (BindingModelBinary), 2: SortingFunctionUniform, 3: SortingFunctionNonUniform
 * (Bindings/BindingModelTernary.h:6-30).  drate rows: species pairs 11, 12, 13, 22, 23, 33, each
 * [before * 2 + 0] = rate to unbound, [before * 2 + 1] = rate to bound (doubr**).  trate rows: sorted
 * species triples 111, 112, 113, 122, 123, 133, 222, 223, 233, 333, each [state * 4 + k] (tripr***). */
typedef struct {
    int rule;
    int div1, div2, np;
    double drate[6][4];
    double trate[10][16];
} orc_binding;

/* patchint (LangevinR.cpp:1790-1800): one candidate patch pair */
typedef struct { int p1, p2, potn, wp1, wp2; } orc_patchint;

double orc_max_check(const orc_model *M);
int orc_total_patches(const orc_model *M, int n);

/* LangevinNVTR::calculate_patch_list(pairs, iny) (LangevinR.cpp:1702-1852).  max_ang = ComboPatch::max_ang
 * (0.6, combopatch.h:15; GeneralPatch lowers it to the smallest cos(thetam), GeneralPatch.cpp:99).
 * Returns the count (entries beyond cap are not written). */
long orc_patch_list(const orc_params *P, const double *x, const double *Q, const int *pairs, long np,
                    double max_ang, orc_patchint *out, long cap);

/* uniform [0, 1) of the GPU path's binding decisions: Philox4x32-10 with counter (root, draw, replica),
 * key (seed_lo + 0x2545F491 (iter + 1), seed_hi ^ 0x6A09E667), 53 bits of the first two words */
double orc_bind_uniform(uint64_t seed, uint32_t replica, uint64_t draw, uint32_t root, uint32_t iter);

/* LangevinNVTR::calculate_forces_and_torques3D_onlyone_nonlets (LangevinRforce.cpp:2874-4030) on the
 * candidate list: edges, bond breaking, patch clusters, binding decisions, then the KF2 force and torque
 * of every bound pair added to F, T.  boundto / isbound (total patches) are updated in place.
 * rng 1: random numbers from the C library's rand() in the reference's order (Generate_Random_Numbers_Needed,
 * then generate_random_matrix for the larger clusters); rng 0: orc_bind_uniform(seed, replica, draw, root
 * patch of the cluster, decision number inside it).  Returns 0, or -2 / -3 where the reference calls error(). */
int orc_bind_update(const orc_params *P, const double *x, const double *Q, const orc_patchint *list, long nl,
                    const orc_binding *B, int rng, uint64_t seed, uint32_t replica, uint64_t draw, int *boundto,
                    unsigned char *isbound, double *F, double *T);

/* LangevinNVTR::setup_random_binding(pairs, divs, iny, bo, bm) (LangevinRforceUtil.cpp:749-1010) on the
 * candidate list: edges as the bond update's edge test finds them, score scr1 + scr2 + scr3 - log(1e-10 +
 * calculate_score), then the greedy walk that binds two unbound patches when the score is below 4.  The
 * reference walks the edges in a std::random_device shuffle; here in ascending (orc_setup_priority(seed,
 * replica, lower patch, higher patch), lower patch, higher patch), the library's seeded order. */
uint32_t orc_setup_priority(uint64_t seed, uint32_t replica, uint32_t lo, uint32_t hi);
/* its edges (wp1, wp2 pairs into ab, 2 per edge) with their scores; returns the count (at most nl) */
long orc_setup_edges(const orc_params *P, const double *x, const double *Q, const orc_patchint *list, long nl,
                     const orc_binding *B, const int *boundto, const unsigned char *isbound, int *ab, double *scr);
int orc_setup_random_binding(const orc_params *P, const double *x, const double *Q, const orc_patchint *list, long nl,
                             const orc_binding *B, uint64_t seed, uint32_t replica, int *boundto,
                             unsigned char *isbound);

/* The run_singlebond loop (Condensate.cpp:422-560) on one system, nsteps from loop index i0:
 * pairs within pair_cut rebuilt when i > 0 and i % pair_every == 0 (and at the start), the candidate
 * list when i > 0 and i % patch_every == 0 (and at the start); F = central forces, T = 0, then
 * orc_bind_update (rng 0, draw0 + s), noise (noise_mode as orc_run), half-kick.  With init, the
 * initial pass before the loop runs first (F, T, bind update and noise of draw init_draw -> Ft, Tt). */
int orc_run_singlebond(const orc_params *P, double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt,
                       int *boundto, unsigned char *isbound, const orc_binding *B, double max_ang, int nsteps, int i0,
                       int ncell, double pair_cut, int pair_every, int patch_every, int init, uint64_t init_draw,
                       int noise_mode, const double *noise, uint64_t seed, uint32_t replica, uint64_t draw0);

/* ---------------------------------------------------------------- seeded synthetic inputs
 * The test and benchmark inputs, generated here as well so that the CPU baselines need nothing from the
 * product library.  They are the same algorithms, draw for draw, as the library's mtg_random_positions /
 * mtg_random_rotations / mtg_random_chains (tests/test_oracle_generators.py checks the outputs are
 * identical): splitmix64 uniforms; random sequential addition with a cell hash at side >= min_dist;
 * uniform rotations by the construction of LangevinNVTR::initialize (LangevinR.cpp:239-267); self-avoiding
 * random-walk chains with directions from cube rejection.  Return 0, or -1 where the library returns
 * MTG_ERR_ARG. */
int orc_random_positions(int n, double box, int periodic, double min_dist, uint64_t seed, double *x);
void orc_random_rotations(int n, uint64_t seed, double *Q);
int orc_random_chains(int n_chains, int beads, double box, int periodic, double step, double min_dist,
                      uint64_t seed, double *x);

#ifdef __cplusplus
}
#endif
#endif
