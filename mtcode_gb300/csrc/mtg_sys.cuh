// mtg_sys.cuh -- one handle's device buffers and the launch sequence of every C-ABI operation,
// templated on the arithmetic type (float: the batched path; double: the plain FP64 path).
//
// A step is five kernels (scan x3, scatter, force) captured once into a CUDA graph per buffer
// parity and replayed.
#pragma once

#include <algorithm>
#include <memory>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "mtg_kernels.cuh"
#include "mtg_pairs.cuh"
#include "mtg_sys_base.h"
#include "mtg_tile.cuh"
#include "mtg_pipe.cuh"
#include "mtg_bind.cuh"

namespace mtg_impl {

// the reference's `pi` is a long double holding pi rounded to double (Basic/basic.h:31)
const long double kPiL = (long double)3.1415926535897932384626433832795028841971693993751;

inline int n_pots_of(const mtg_patch_model &m) {
    int npots = 0;
    for (int a = 0; a < m.n_types; a++)
        for (int b = a; b < m.n_types; b++) npots += m.patches_per_type[a] * m.patches_per_type[b];
    return npots;
}

template <class real>
mtg::Model<real> make_model(const mtg_patch_model &m) {
    mtg::Model<real> M;
    std::memset(&M, 0, sizeof(M));
    M.n_types = m.n_types;
    int oo = 0;
    for (int k = 0; k < m.n_types; k++) {
        M.np[k] = m.patches_per_type[k];
        M.ncum[k] = m.count_per_type[k];
        M.ooff[k] = oo;
        oo += m.patches_per_type[k];
    }
    for (int i = 0; i < oo; i++)
        for (int c = 0; c < 3; c++) M.orient[i][c] = (real)m.orient[i][c];
    int ps = 0;
    for (int a = 0; a < m.n_types; a++)
        for (int b = a; b < m.n_types; b++) {
            M.pstart[a][b] = ps;
            double mc = 2.0;
            for (int q = ps; q < ps + m.patches_per_type[a] * m.patches_per_type[b]; q++) {
                double att = m.params[q][0], dis = m.params[q][1], th = m.params[q][2];
                M.att[q] = (real)att;
                M.dis[q] = (real)dis;
                M.inv_dis[q] = (real)(1.0 / dis);
                M.rmax[q] = (real)(1.4 * dis);
                M.costm[q] = (real)std::cos(th);
                M.kfac[q] = (real)(double)(kPiL / (2.0L * (long double)th));
                mc = std::min(mc, std::cos(th));
            }
            M.mincos[a][b] = M.mincos[b][a] = (real)mc;
            ps += m.patches_per_type[a] * m.patches_per_type[b];
        }
    for (int a = 0; a < m.n_types; a++) {
        M.mincos_any[a] = (real)2;
        for (int b = 0; b < m.n_types; b++) M.mincos_any[a] = std::min(M.mincos_any[a], M.mincos[a][b]);
    }
    return M;
}

struct ReplicaGeometry {
    double rc;        // force range
    double patch_r;   // patch force range
    double bond_r;    // ComboPatch::max_check
};

inline ReplicaGeometry geometry_of(const mtg_replica_desc &d) {
    ReplicaGeometry g;
    double hs = 1.12246 * d.hs_sigma;
    double dmax = 0;
    bool patches = false;
    for (int k = 0; k < d.model.n_types; k++) patches |= d.model.patches_per_type[k] > 0;
    int np = n_pots_of(d.model);
    for (int q = 0; q < np; q++) dmax = std::max(dmax, 1.4 * d.model.params[q][1]);
    g.patch_r = patches ? std::min(std::sqrt(d.max_dist2), dmax) : 0.0;
    g.rc = std::max(hs, g.patch_r);
    g.bond_r = std::max(1.0, dmax);
    return g;
}

// skin lists: the list (and cell) range, force range + skin, padded by 1e-3 sigma so that an FP32
// rounding of the displacement test can never lose a pair
inline double list_range(double rc, double skin) { return skin > 0 ? rc + skin + 1e-3 : rc; }

// Pair finding forms a shifted separation as (x_a - x_b) - shift, which may differ from the pair kernels'
// min_image_sep by a rounding at the box length's scale plus the float box's own error; it takes every pair
// within the range widened by that slack (squared here), and the pair kernels drop the extra ones with the
// exact test.
inline double find_range2(double range, double box) {
    const double ulp_box = std::ldexp(1.0, std::ilogb(std::max(box, 1.0)) - 23);
    const double slack = 2.0 * ulp_box + std::fabs(box - (double)(float)box) + 1e-6;
    return (range + slack) * (range + slack) * (1 + 1e-6);
}

// Division by a cell count without an integer divide: n / nc = floor(n m / 2^(32+k)) with k the largest
// integer such that 2^k < nc and m = ceil(2^(32+k) / nc) < 2^32.  With m = 2^(32+k) / nc + e (0 <= e < 1), the
// product overshoots n / nc by n e / 2^(32+k) < 1 / nc whenever n nc < 2^(32+k), which cannot carry it past the
// next integer; since 2^(k+1) >= nc, that holds for every n < nc^3 while nc^3 <= 2^31 (nc <= 1290; cell keys
// are ints).  nc = 1: every key is 0, m = 0.
inline void nc_magic(int nc, uint32_t &mul, int &sh) {
    if (nc <= 1) {
        mul = 0;
        sh = 0;
        return;
    }
    int k = 0;
    while ((2ll << k) < nc) k++;
    mul = (uint32_t)(((1ull << (32 + k)) + (uint64_t)nc - 1) / (uint64_t)nc);
    sh = k;
}

template <class real>
mtg::Replica<real> make_replica(const mtg_replica_desc &d, int off, int cell_off, int nc, int model,
                                double skin = 0.0) {
    mtg::Replica<real> R;
    std::memset(&R, 0, sizeof(R));
    ReplicaGeometry g = geometry_of(d);
    R.n = d.n;
    R.off = off;
    R.cell_off = cell_off;
    R.nc = nc;
    nc_magic(nc, R.nc_mul, R.nc_sh);
    R.periodic = d.periodic ? 1 : 0;
    R.model = model;
    R.seed_lo = (uint32_t)d.seed;
    R.seed_hi = (uint32_t)(d.seed >> 32);
    R.box = (real)d.box;
    R.box_lo = (real)(d.box - (double)R.box);
    R.half_box = (real)(d.box * 0.5);
    R.l2s = (real)((d.box / 2.) * (d.box / 2.));
    R.cell_scale = (real)((double)nc / d.box);
    R.dt = (real)d.dt;
    R.half_dt = (real)(d.dt / 2.);
    R.c1 = (real)(d.dt / d.mass);
    R.fric_t = (real)(-d.gamma / d.mass);
    R.fric_r = (real)(-d.gammar / d.inertia);
    R.Rt = (real)std::sqrt(2 * d.gamma * d.kT / d.dt);
    R.Rr = (real)std::sqrt(2 * d.gammar * d.kT / d.dt);
    R.inertia = (real)d.inertia;
    double s6 = std::pow(d.hs_sigma, 6);
    R.hs_limit = (real)(1.12246 * d.hs_sigma);
    R.hs_4eps = (real)(4 * d.hs_eps);
    R.hs_s6 = (real)s6;
    R.hs_s12 = (real)(s6 * s6);
    R.hs_eps = (real)d.hs_eps;
    R.max_dist2 = (real)d.max_dist2;
    R.rc2 = (real)(g.rc * g.rc);
    R.patch_r2 = (real)(g.patch_r * g.patch_r);
    R.bond_r = (real)g.bond_r;
    const double rl = list_range(g.rc, skin);
    R.rc2_list = (real)(rl * rl);
    R.rc2_find = (real)find_range2(g.rc, d.box);
    R.rc2_list_find = (real)find_range2(rl, d.box);
    R.half_skin2 = (real)(0.25 * skin * skin);
    return R;
}

// cells per side so that side >= range (with room for rounding of the cell assignment), at most 1,024: cells
// only grow beyond the range, which keeps every pair, and nc^3 keys stay within nc_magic's exact range
inline int cells_per_side(double box, double range) {
    const double f = std::floor(box / (range * 1.0001));
    return !(f >= 1) ? 1 : (f > 1024 ? 1024 : (int)f);
}

// Cells per side of an analysis grid (pair export, g(r), clusters) for a cut rc: side >= rc, so the
// 27-cell stencil holds every pair closer than rc.  The count is capped (in 64-bit arithmetic) at the
// smaller of 512 and about twice the cube root of n: cells only grow beyond rc, which keeps the pair set
// exact, and nc^3 and every cell key stay far inside int even for a tiny rc.
inline int analysis_cells(double box, double rc, int n) {
    const double f = std::floor(box / (rc * (1 + 1e-12)));
    int64_t nc = !(f >= 1) ? 1 : (f > 512 ? 512 : (int64_t)f);
    int64_t cap = 2;
    while (cap * cap * cap < 8 * (int64_t)std::max(n, 1) && cap < 512) cap++;
    return (int)std::max<int64_t>(1, std::min(nc, cap));
}

inline int grid_for(int64_t n, int block, int per_sm, int sms) {
    int64_t need = (n + block - 1) / block;
    int64_t cap = (int64_t)per_sm * sms;
    return (int)std::max<int64_t>(1, std::min(need, cap));
}

// Tile plan of one replica for the FP32 tile kernel: whole x-rows or chunks of 30/16/8 cells, times
// T x T rows (T = 4, 2, 1).  Warps take 32-particle units of a tile, so larger tiles only lower the
// halo share; the choice is the largest tile whose expected staged count (tile + one-cell halo, from
// the mean cell occupancy) is at most half the staging buffer, leaving room for density fluctuations.
inline void plan_tiles(int rep, int nc, int periodic, int cell_off, double per_cell, std::vector<int4> &out) {
    const int rep_word = rep | ((periodic ? 1 : 0) << 30);
    if (nc < 3 || nc > 1023) {
        out.push_back(make_int4(rep_word, 0, 1 << 21, cell_off));
        return;
    }
    struct Cand { bool whole; int tx, T; double home, staged; };
    std::vector<Cand> cands;
    for (int T : {4, 2, 1}) {
        if (nc <= mtg::kTileXMax) cands.push_back({true, nc, T, nc * T * T * per_cell, nc * (T + 2.0) * (T + 2.0) * per_cell});
        for (int tx : {30, 16, 8})  // a staged row (tx + 2 cells) spans at most one warp's lanes
            if (tx + 2 <= nc) cands.push_back({false, tx, T, tx * T * T * per_cell, (tx + 2.0) * (T + 2.0) * (T + 2.0) * per_cell});
    }
    const Cand *best = nullptr;
    for (const Cand &c : cands) {
        if (c.staged > 0.5 * mtg::kStageCap) continue;
        if (!best || c.home > best->home * 1.05 ||
            (c.home > best->home * 0.95 && c.staged / c.home < best->staged / best->home))
            best = &c;
    }
    if (!best)
        for (const Cand &c : cands)
            if (!best || c.staged < best->staged) best = &c;
    const int T = best->T, tx = best->whole ? nc : best->tx;
    for (int z0 = 0; z0 < nc; z0 += T)
        for (int y0 = 0; y0 < nc; y0 += T)
            for (int x0 = 0; x0 < nc; x0 += tx) {
                const int ty = std::min(T, nc - y0), tz = std::min(T, nc - z0);
                const int sx = best->whole ? nc : std::min(tx, nc - x0) + 2;
                out.push_back(make_int4(rep_word, x0 | (y0 << 10) | (z0 << 20),
                                        sx | (ty << 10) | (tz << 15) | ((best->whole ? 1 : 0) << 20) | (nc << 22),
                                        cell_off));
            }
}

template <class real>
struct Sys : SysBase {
    int device = 0;
    int sms = 0;
    cudaStream_t st = nullptr;
    int nrep = 0;
    int ntot_ = 0;
    bool track_disp = true;
    std::vector<mtg_replica_desc> desc;
    std::vector<mtg::Replica<real>> reps, reps_obs;
    std::vector<mtg::Model<real>> models;
    std::vector<int> rep_slot;
    int ncells = 0, ncells_obs = 0, ncells_alloc = 0;

    mtg::Replica<real> *d_reps = nullptr, *d_reps_obs = nullptr;
    int reps_uniform = 0, reps_obs_uniform = 0;   // see pair_uniform()
    mtg::Model<real> *d_models = nullptr;
    int *d_rep_slot = nullptr;
    unsigned short *d_slot_rep = nullptr;   // replica of every slot (fewer than 65,536 replicas)
    mtg::Buffers<real> buf[2] = {};
    int cur = 0;
    int2 *d_bin = nullptr;
    int *d_count = nullptr, *d_start = nullptr, *d_block = nullptr;
    unsigned *d_flags = nullptr;
    unsigned long long *d_draw = nullptr;
    double *d_stage = nullptr;   // 24 x ntot doubles: host-order state in / out
    double *d_noise = nullptr;   // ntot x 6 (external noise)
    double *d_obs = nullptr;     // nrep x 6
    unsigned *h_flags = nullptr; // pinned
    double *h_obs = nullptr;     // pinned: temperature read-backs (one slot of 6 x nrep per step)
    size_t h_obs_cap = 0;
    double *d_tring = nullptr;   // device ring of per-step temperature sums (mtg_step_temperatures)
    size_t d_tring_cap = 0;
    uint64_t draw = 0;
    bool have_state = false, cells_valid = false, bins_valid = false, forces_ready = false;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_kernels[2] = {0, 0};   // kernel launches of one step (kernel nodes of its graph)
    bool capturing = false;          // a step graph is being captured: its launches are counted per replay
    // fixed bonds (CSR by global index) and the id -> slot map the bond pass needs
    int *d_bond_start = nullptr, *d_bond_partner = nullptr, *d_slot_of = nullptr;
    int *d_gather_map = nullptr;   // slot of each global index, built by get_state when d_slot_of is not kept
    int64_t nbonds = 0;
    double bond_k = 0, bond_r0 = 0;
    int64_t nlaunch = 0;
    cudaEvent_t *prof_ev = nullptr;  // set by step_profile: events around the pair pipeline's kernels
    int64_t wait_limit = 0;          // mtg_set_wait_limit: 0 = each bounded loop's own bound
    // launch shapes of the pair pipeline (mtg_set_launch_config / mtg_autotune); every shape gives the same
    // FP32 results bit for bit (fixed-point sums), so the tuner may time them on the live state
    mtg_launch_config lc = {256, 16, 8, 256, 1};
    // FP32 tile kernel
    bool use_tiles = false;
    int4 *d_tiles = nullptr;
    int ntiles = 0, occ_tile = 1;
    // pair pipeline (force_kernel 0): pair list, its length, force/torque sums per slot (FP32: fixed point)
    bool use_pipe = false;
    int2 *d_pairs = nullptr;
    unsigned long long *d_npairs = nullptr;
    using acc_t = typename mtg::PairAcc<real>::type;
    acc_t *d_acc = nullptr;
    long long pair_cap = 0;
    // pairs with a patch near a cone on both sides, for the patch-pair kernel (segmented list)
    int2 *d_patch_list = nullptr;
    unsigned long long *d_patch_ctr = nullptr;
    long long patch_cap = 0;
    // skin lists (null without a skin): state flags, candidate lists and lengths, build positions / cells
    double skin = 0;
    int *d_skin = nullptr, *d_list_n = nullptr, *d_home_cell = nullptr;
    unsigned *d_list = nullptr;
    real *d_xref = nullptr;
    size_t tile_smem = 0;
    // occupancy-derived grid caps
    int occ_force = 1, occ_stream = 1;
    // single-bond-per-patch mode (Condensate::run_singlebond): patch numbering, binding model, candidate
    // list, per-update adjacency, bond state (global patch indices), large-cluster queue and scratch
    bool single_bond = false;
    int ptot = 0, patch_every = 10, scratch_threads = 0;
    std::vector<int> patch_slot;
    mtg::BindModel bind_model_h;   // the binding model's tables (host copy)
    std::vector<mtg::Replica<real>> reps_full;   // replica constants with the full patch force
    mtg::BindRep *d_brep = nullptr;
    mtg::BindModel *d_bmodel = nullptr;
    int *d_patch_slot = nullptr, *d_boundto = nullptr, *d_large = nullptr, *d_scratch = nullptr;
    int *d_touched = nullptr;
    int2 *d_bind_pairs = nullptr;   // pairs the FP32 pipeline lists for the edge pass
    int2 *d_bound = nullptr;        // pairs bound by the decisions (FP32 pipeline)
    long long tcap = 0, bcap = 0, lcap = 0;   // segment capacities: touched, bound, listed pairs
    int2 *d_recheck = nullptr;                 // patch pairs for the FP64 tests of the float edge pass
    long long rcap = 0;
    int ncells_full = 0;                         // the force grid's cells outside single-bond mode
    unsigned long long *d_bctr = nullptr, *d_deg = nullptr;
    int2 *d_adj = nullptr;
    unsigned char *d_isbound = nullptr;

    Sys(const mtg_config &cfg) {
        device = cfg.device;
        MTG_CUDA(cudaSetDevice(device));
        cudaDeviceProp prop;
        MTG_CUDA(cudaGetDeviceProperties(&prop, device));
        sms = prop.multiProcessorCount;
        MTG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        nrep = cfg.n_replicas;
        track_disp = cfg.track_displacement != 0;
        skin = cfg.neighbor_skin;
        desc.assign(cfg.replicas, cfg.replicas + nrep);
        int64_t off = 0, coff = 0, coff_obs = 0;
        rep_slot.push_back(0);
        for (int r = 0; r < nrep; r++) {
            const mtg_replica_desc &d = desc[r];
            ReplicaGeometry g = geometry_of(d);
            int nc = cells_per_side(d.box, list_range(g.rc, skin));
            int nco = cells_per_side(d.box, std::max(g.rc, g.bond_r));
            models.push_back(make_model<real>(d.model));
            reps.push_back(make_replica<real>(d, (int)off, (int)coff, nc, r, skin));
            reps_obs.push_back(make_replica<real>(d, (int)off, (int)coff_obs, nco, r));
            off += d.n;
            coff += (int64_t)nc * nc * nc;
            coff_obs += (int64_t)nco * nco * nco;
            if (off > 0x7fffffff || coff > 0x7fffffff) throw Fail{MTG_ERR_ARG, "too many particles or cells"};
            rep_slot.push_back((int)off);
        }
        ntot_ = (int)off;
        ncells = (int)coff;
        ncells_obs = (int)coff_obs;
        ncells_alloc = std::max(ncells, ncells_obs);
        size_t n = (size_t)std::max(ntot_, 1);
        MTG_CUDA(cudaMalloc(&d_reps, sizeof(mtg::Replica<real>) * nrep));
        MTG_CUDA(cudaMalloc(&d_reps_obs, sizeof(mtg::Replica<real>) * nrep));
        MTG_CUDA(cudaMalloc(&d_models, sizeof(mtg::Model<real>) * nrep));
        MTG_CUDA(cudaMalloc(&d_rep_slot, sizeof(int) * (nrep + 1)));
        MTG_CUDA(cudaMemcpy(d_reps, reps.data(), sizeof(mtg::Replica<real>) * nrep, cudaMemcpyHostToDevice));
        reps_uniform = pair_uniform(reps);
        MTG_CUDA(cudaMemcpy(d_reps_obs, reps_obs.data(), sizeof(mtg::Replica<real>) * nrep, cudaMemcpyHostToDevice));
        reps_obs_uniform = pair_uniform(reps_obs);
        MTG_CUDA(cudaMemcpy(d_models, models.data(), sizeof(mtg::Model<real>) * nrep, cudaMemcpyHostToDevice));
        MTG_CUDA(cudaMemcpy(d_rep_slot, rep_slot.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice));
        if (nrep < 65536) {
            std::vector<unsigned short> sr((size_t)std::max(ntot_, 1), 0);
            for (int r = 0; r < nrep; r++)
                for (int i = rep_slot[r]; i < rep_slot[r + 1]; i++) sr[(size_t)i] = (unsigned short)r;
            MTG_CUDA(cudaMalloc(&d_slot_rep, sizeof(unsigned short) * sr.size()));
            MTG_CUDA(cudaMemcpy(d_slot_rep, sr.data(), sizeof(unsigned short) * sr.size(), cudaMemcpyHostToDevice));
        }

        for (int b = 0; b < 2; b++) {
            MTG_CUDA(cudaMalloc(&buf[b].pos, sizeof(real) * 4 * n));
            MTG_CUDA(cudaMalloc(&buf[b].rota, sizeof(real) * 4 * n));
            MTG_CUDA(cudaMalloc(&buf[b].rotb, sizeof(real) * 4 * n));
            MTG_CUDA(cudaMalloc(&buf[b].motion, sizeof(real) * mtg::kRow * n));
            MTG_CUDA(cudaMalloc(&buf[b].ident, sizeof(int) * n));
            if (track_disp) {
                MTG_CUDA(cudaMalloc(&buf[b].dx, sizeof(double) * n));
                MTG_CUDA(cudaMalloc(&buf[b].dy, sizeof(double) * n));
                MTG_CUDA(cudaMalloc(&buf[b].dz, sizeof(double) * n));
            }
        }
        if (skin > 0) {
            MTG_CUDA(cudaMalloc(&d_skin, sizeof(int) * 4));
            MTG_CUDA(cudaMemset(d_skin, 0, sizeof(int) * 4));
            MTG_CUDA(cudaMalloc(&d_list, sizeof(unsigned) * mtg::kListCap * n));
            MTG_CUDA(cudaMalloc(&d_list_n, sizeof(int) * n));
            MTG_CUDA(cudaMemset(d_list_n, 0, sizeof(int) * n));
            MTG_CUDA(cudaMalloc(&d_home_cell, sizeof(int) * n));
            MTG_CUDA(cudaMalloc(&d_xref, sizeof(real) * 4 * n));
            for (int b = 0; b < 2; b++) {
                buf[b].xref = d_xref;
                buf[b].home_cell = d_home_cell;
            }
        }
        MTG_CUDA(cudaMalloc(&d_bin, sizeof(int2) * n));
        MTG_CUDA(cudaMalloc(&d_count, sizeof(int) * (ncells_alloc + 1)));
        // + 8: the tile kernel copies cell starts in aligned 16-byte chunks, up to 3 entries past the end
        MTG_CUDA(cudaMalloc(&d_start, sizeof(int) * (ncells_alloc + 8)));
        MTG_CUDA(cudaMemset(d_start, 0, sizeof(int) * (ncells_alloc + 8)));
        int nblk = (ncells_alloc + mtg::kScanTile - 1) / mtg::kScanTile + 1;
        MTG_CUDA(cudaMalloc(&d_block, sizeof(int) * nblk));
        MTG_CUDA(cudaMalloc(&d_flags, sizeof(unsigned)));
        MTG_CUDA(cudaMalloc(&d_draw, sizeof(unsigned long long) * 2));
        MTG_CUDA(cudaMalloc(&d_stage, sizeof(double) * 24 * n));
        MTG_CUDA(cudaMalloc(&d_obs, sizeof(double) * 6 * std::max(nrep, 1)));
        MTG_CUDA(cudaMallocHost(&h_flags, sizeof(unsigned)));
        MTG_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int) * (ncells_alloc + 1), st));
        MTG_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(unsigned), st));
        MTG_CUDA(cudaMemsetAsync(d_draw, 0, sizeof(unsigned long long) * 2, st));
        int occ = 0;
        MTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mtg::force_kernel<real, mtg::kModeStep>, 128, 0));
        occ_force = std::max(occ, 1);
        MTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mtg::scatter_kernel<real, true>, 256, 0));
        occ_stream = std::max(occ, 1);
        MTG_REQUIRE(cfg.force_kernel >= 0 && cfg.force_kernel <= 2, "mtg_create: force_kernel must be 0, 1 or 2");
        MTG_REQUIRE((cfg.force_kernel != 2 || std::is_same<real, float>::value),
                    "mtg_create: the tiled force kernel (force_kernel 2) is FP32 only");
        use_pipe = cfg.force_kernel == 0;
        if (use_pipe) {
            pair_cap = (long long)mtg::kPairsPerParticle * (long long)n;
            MTG_CUDA(cudaMalloc(&d_pairs, sizeof(int2) * (size_t)pair_cap));
            MTG_CUDA(cudaMalloc(&d_npairs, sizeof(unsigned long long)));
            MTG_CUDA(cudaMemset(d_npairs, 0, sizeof(unsigned long long)));
            MTG_CUDA(cudaMalloc(&d_acc, sizeof(acc_t) * 6 * n));
            MTG_CUDA(cudaMemset(d_acc, 0, sizeof(acc_t) * 6 * n));
            patch_cap = std::max<long long>(1024, 2 * (pair_cap + mtg::kSegs - 1) / mtg::kSegs);
            MTG_CUDA(cudaMalloc(&d_patch_list, sizeof(int2) * (size_t)patch_cap * mtg::kSegs));
            MTG_CUDA(cudaMalloc(&d_patch_ctr, sizeof(unsigned long long) * mtg::kSegs));
            MTG_CUDA(cudaMemset(d_patch_ctr, 0, sizeof(unsigned long long) * mtg::kSegs));
            if (!d_home_cell) {
                MTG_CUDA(cudaMalloc(&d_home_cell, sizeof(int) * n));
                MTG_CUDA(cudaMemset(d_home_cell, 0, sizeof(int) * n));
                buf[0].home_cell = buf[1].home_cell = d_home_cell;
            }
        }
        if constexpr (std::is_same<real, float>::value) {
            use_tiles = cfg.force_kernel == 2;
            if (use_tiles) {
                std::vector<int4> tiles;
                for (int r = 0; r < nrep; r++)
                    plan_tiles(r, reps[r].nc, reps[r].periodic, reps[r].cell_off, (double)desc[r].n / ((double)reps[r].nc * reps[r].nc * reps[r].nc), tiles);
                ntiles = (int)tiles.size();
                MTG_CUDA(cudaMalloc(&d_tiles, sizeof(int4) * ntiles));
                MTG_CUDA(cudaMemcpy(d_tiles, tiles.data(), sizeof(int4) * ntiles, cudaMemcpyHostToDevice));
                tile_smem = sizeof(mtg::TileShared);
                MTG_CUDA(cudaFuncSetAttribute(mtg::tile_force_kernel<mtg::kModeStep>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem));
                MTG_CUDA(cudaFuncSetAttribute(mtg::tile_force_kernel<mtg::kModeInit>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem));
                MTG_CUDA(cudaFuncSetAttribute(mtg::tile_force_kernel<mtg::kModeForces>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem));
                MTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mtg::tile_force_kernel<mtg::kModeStep>,
                                                                       mtg::kTileThreads, tile_smem));
                occ_tile = std::max(occ, 1);
            }
        }
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    ~Sys() override {
        cudaSetDevice(device);
        if (st) cudaStreamSynchronize(st);
        for (int b = 0; b < 2; b++) {
            if (graph[b]) cudaGraphExecDestroy(graph[b]);
            cudaFree(buf[b].pos); cudaFree(buf[b].rota); cudaFree(buf[b].rotb); cudaFree(buf[b].motion); cudaFree(buf[b].ident);
            cudaFree(buf[b].dx); cudaFree(buf[b].dy); cudaFree(buf[b].dz);
        }
        cudaFree(d_reps); cudaFree(d_reps_obs); cudaFree(d_models); cudaFree(d_rep_slot); cudaFree(d_slot_rep);
        cudaFree(d_bin); cudaFree(d_count); cudaFree(d_start); cudaFree(d_block);
        cudaFree(d_flags); cudaFree(d_draw); cudaFree(d_stage); cudaFree(d_noise); cudaFree(d_obs);
        cudaFree(d_tring);
        cudaFree(d_tiles);
        cudaFree(d_bond_start); cudaFree(d_bond_partner); cudaFree(d_slot_of); cudaFree(d_gather_map);
        cudaFree(d_skin); cudaFree(d_list); cudaFree(d_list_n); cudaFree(d_home_cell); cudaFree(d_xref);
        cudaFree(d_pairs); cudaFree(d_npairs); cudaFree(d_acc); cudaFree(d_patch_list); cudaFree(d_patch_ctr);
        free_bind();
        if (h_flags) cudaFreeHost(h_flags);
        if (h_obs) cudaFreeHost(h_obs);
        if (st) cudaStreamDestroy(st);
    }

    mtg::Tables<real> tables(bool obs = false) const {
        mtg::Tables<real> t;
        t.reps = obs ? d_reps_obs : d_reps;
        t.rep_slot = d_rep_slot;
        t.models = d_models;
        t.nrep = nrep;
        t.ntot = ntot_;
        t.ncells = obs ? ncells_obs : ncells;
        t.uniform = obs ? reps_obs_uniform : reps_uniform;
        t.slot_rep = d_slot_rep;
        return t;
    }

    // 1 when every replica has replica 0's pair constants (box, boundary, ranges, HSPotential, patch range)
    // and a model equal to replica 0's with one particle type: a pair's constants then do not depend on
    // its replica (per-replica fields -- offsets, counts, seeds, cell grid -- are not compared)
    int pair_uniform(const std::vector<mtg::Replica<real>> &rs) const {
        if (rs.empty()) return 0;
        const mtg::Replica<real> &a = rs[0];
        const mtg::Model<real> &ma = models[a.model];
        if (ma.n_types != 1) return 0;
        auto same = [](const void *x, const void *y, size_t n) { return std::memcmp(x, y, n) == 0; };
        for (const mtg::Replica<real> &b : rs) {
            if (b.periodic != a.periodic || b.box != a.box || b.box_lo != a.box_lo || b.half_box != a.half_box ||
                b.l2s != a.l2s ||
                b.hs_limit != a.hs_limit || b.hs_4eps != a.hs_4eps || b.hs_s6 != a.hs_s6 || b.hs_s12 != a.hs_s12 ||
                b.hs_eps != a.hs_eps || b.max_dist2 != a.max_dist2 || b.rc2 != a.rc2 || b.patch_r2 != a.patch_r2 ||
                b.rc2_list != a.rc2_list || b.rc2_find != a.rc2_find || b.rc2_list_find != a.rc2_list_find ||
                b.half_skin2 != a.half_skin2 || b.bond_r != a.bond_r)
                return 0;
            const mtg::Model<real> &mb = models[b.model];
            if (mb.n_types != 1 || !same(mb.np, ma.np, sizeof ma.np) || !same(mb.ooff, ma.ooff, sizeof ma.ooff) ||
                !same(mb.pstart, ma.pstart, sizeof ma.pstart) || !same(mb.orient, ma.orient, sizeof ma.orient) ||
                !same(mb.att, ma.att, sizeof ma.att) || !same(mb.dis, ma.dis, sizeof ma.dis) ||
                !same(mb.inv_dis, ma.inv_dis, sizeof ma.inv_dis) || !same(mb.rmax, ma.rmax, sizeof ma.rmax) ||
                !same(mb.costm, ma.costm, sizeof ma.costm) || !same(mb.kfac, ma.kfac, sizeof ma.kfac) ||
                !same(mb.mincos, ma.mincos, sizeof ma.mincos) ||
                !same(mb.mincos_any, ma.mincos_any, sizeof ma.mincos_any))
                return 0;
        }
        return 1;
    }

    int64_t ntot() const override { return ntot_; }
    int64_t offset(int r) const override { return rep_slot[r]; }
    cudaStream_t stream() const override { return st; }
    int64_t launches() const override { return nlaunch; }

    void check_launch() { MTG_CUDA(cudaGetLastError()); }
    // k kernels enqueued (outside a graph capture; a replayed step graph adds its own kernel count)
    void counted(int k) {
        if (!capturing) nlaunch += k;
    }

    // counting sort of the current buffer by cell (no motion), result in the other buffer
    void rebuild_cells(bool obs) {
        mtg::Tables<real> tb = tables(obs);
        int nc = obs ? ncells_obs : ncells;
        MTG_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int) * (ncells_alloc + 1), st));
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::bin_kernel<real, false><<<g, 256, 0, st>>>(tb, buf[cur], d_bin, d_count, d_flags);
        check_launch();
        scan(nc, false);
        mtg::scatter_kernel<real, false><<<g, 256, 0, st>>>(tb, buf[cur], buf[cur ^ 1], d_bin, d_start, d_flags);
        check_launch();
        cur ^= 1;
        nlaunch += 2;  // bin and scatter (the scan counts its own)
        cells_valid = !obs;
        bins_valid = false;
    }

    void scan(int n, bool consume_draw) {
        int nblk = (n + mtg::kScanTile - 1) / mtg::kScanTile;
        if (nblk < 1) nblk = 1;
        mtg::scan_reduce_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, n, d_block);
        mtg::scan_top_kernel<<<1, mtg::kScanThreads, 0, st>>>(d_block, nblk, d_start, n, d_draw, consume_draw ? 1 : 0);
        mtg::scan_down_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, n, d_block, d_start);
        check_launch();
        counted(3);
    }

    mtg::ForceArgs<real> force_args(int b, int do_kick) {
        mtg::ForceArgs<real> a;
        std::memset(&a, 0, sizeof(a));
        a.tb = tables();
        a.buf = buf[b];
        a.start = d_start;
        a.bin = d_bin;
        a.count = d_count;
        a.flags = d_flags;
        a.draw = d_draw;
        a.do_kick = do_kick;
        a.parts = 3;
        if (skin > 0) {
            a.skin = d_skin;
            a.skin_next = d_skin + 1;
            a.list = d_list;
            a.list_n = d_list_n;
        }
        if (nbonds > 0) {
            a.bond_start = d_bond_start;
            a.bond_partner = d_bond_partner;
            a.bond_k = (real)bond_k;
            a.bond_r0 = (real)bond_r0;
        }
        if (single_bond) {
            a.bind_reps = d_brep;
            a.bind_on = d_isbound;
            a.bind_to = d_boundto;
        }
        return a;
    }

    // ---------------------------------------------------------------- single-bond-per-patch mode

    mtg::BindState bind_state() const {
        mtg::BindState S;
        std::memset(&S, 0, sizeof(S));
        S.reps = d_brep;
        S.model = d_bmodel;
        S.patch_slot = d_patch_slot;
        S.nrep = nrep;
        S.ptot = ptot;
        S.patch_every = patch_every;
        S.ctr = d_bctr;
        S.deg = d_deg;
        S.adj = d_adj;
        S.boundto = d_boundto;
        S.isbound = d_isbound;
        S.large = d_large;
        S.touched = d_touched;
        S.tcap = tcap;
        S.bound = nullptr;
        S.bcap = bcap;
        S.scratch = d_scratch;
        S.scratch_threads = scratch_threads;
        S.flags = d_flags;
        S.draw = d_draw;
        return S;
    }

    // this update's stamp and whether the candidate list is due; a forced list (a pass that does not move
    // the particles) takes its snapshot from buffer b at once, a step's from the scatter
    void enqueue_bind_begin(int b, int force, int advance) {
        mtg::bind_begin_kernel<<<1, 32, 0, st>>>(bind_state(), force, advance);
        counted(1);
        if (force) {
            const int g = grid_for(ntot_, 256, occ_stream, sms);
            mtg::bind_snapshot_kernel<real><<<g, 256, 0, st>>>(ntot_, buf[b]);
            counted(1);
        }
    }

    // clusters and bond decisions from this update's edges (positions reached through slot_of)
    void enqueue_bind_decide(const mtg::ForceArgs<real> &a, bool listed) {
        mtg::BindState S = bind_state();
        if (listed) S.bound = d_bound;
        mtg::bind_unbind_kernel<<<grid_for((ptot + 15) / 16, 256, occ_stream, sms), 256, 0, st>>>(S);  // 16 patches a thread
        mtg::bind_decide_kernel<<<grid_for(ptot, 256, 4, sms), 256, 0, st>>>(S);
        mtg::bind_large_kernel<real><<<scratch_threads / mtg::kLargeThreads, mtg::kLargeThreads, 0, st>>>(a, S);
        counted(3);
    }

    void free_bind() {
        cudaFree(d_brep); cudaFree(d_bmodel); cudaFree(d_patch_slot); cudaFree(d_boundto); cudaFree(d_large);
        cudaFree(d_scratch); cudaFree(d_bctr); cudaFree(d_deg); cudaFree(d_adj); cudaFree(d_isbound);
        cudaFree(d_touched); cudaFree(d_bind_pairs); cudaFree(d_bound); cudaFree(d_recheck);
        d_recheck = nullptr;
        d_touched = nullptr;
        d_bind_pairs = nullptr;
        d_bound = nullptr;
        d_brep = nullptr; d_bmodel = nullptr; d_patch_slot = d_boundto = d_large = d_scratch = nullptr;
        d_bctr = d_deg = nullptr; d_adj = nullptr; d_isbound = nullptr;
        cudaFree(buf[0].snap_a); cudaFree(buf[0].snap_b); cudaFree(buf[0].snap_c);  // one set, shared
        for (int b = 0; b < 2; b++) buf[b].snap_a = buf[b].snap_b = buf[b].snap_c = nullptr;
    }

    void drop_graphs() {
        for (int b = 0; b < 2; b++) {
            if (graph[b]) cudaGraphExecDestroy(graph[b]);
            graph[b] = nullptr;
            graph_kernels[b] = 0;
        }
    }

    void ensure_slot_of() {
        if (d_slot_of) return;
        MTG_CUDA(cudaMalloc(&d_slot_of, sizeof(int) * (size_t)std::max(ntot_, 1)));
        buf[0].slot_of = buf[1].slot_of = d_slot_of;
        if (have_state) {
            const int g = grid_for(ntot_, 256, occ_stream, sms);
            mtg::slot_map_kernel<<<g, 256, 0, st>>>(ntot_, buf[cur].ident, d_slot_of);
            check_launch();
            nlaunch += 1;
        }
    }

    void set_single_bond(const mtg_single_bond *sb) override {
        MTG_CUDA(cudaStreamSynchronize(st));
        if (!sb) {
            if (!single_bond) return;
            drop_graphs();
            free_bind();
            single_bond = false;
            reps = reps_full;
            ncells = ncells_full;
            MTG_CUDA(cudaMemcpy(d_reps, reps.data(), sizeof(mtg::Replica<real>) * nrep, cudaMemcpyHostToDevice));
            reps_uniform = pair_uniform(reps);
        reps_uniform = pair_uniform(reps);
            forces_ready = false;
            cells_valid = bins_valid = false;
            return;
        }
        MTG_REQUIRE(skin <= 0, "mtg_set_single_bond: not available with a neighbour skin");
        MTG_REQUIRE(!use_tiles, "mtg_set_single_bond: needs the pair pipeline or the per-particle force kernel");
        const mtg_binding_model &bm = sb->model;
        MTG_REQUIRE(bm.species_rule >= 0 && bm.species_rule <= 3, "mtg_set_single_bond: species_rule must be 0..3");
        MTG_REQUIRE(bm.species_rule != 3 || bm.np >= 1, "mtg_set_single_bond: SortingFunctionNonUniform needs np >= 1");
        for (int r = 0; r < 6; r++)
            for (int k = 0; k < 4; k++) MTG_REQUIRE(std::isfinite(bm.drate[r][k]), "mtg_set_single_bond: rates must be finite");
        for (int r = 0; r < 10; r++)
            for (int k = 0; k < 16; k++) MTG_REQUIRE(std::isfinite(bm.trate[r][k]), "mtg_set_single_bond: rates must be finite");
        MTG_REQUIRE(sb->patch_every >= 1, "mtg_set_single_bond: patch_every must be >= 1");
        MTG_REQUIRE(std::isfinite(sb->list_cut) && sb->list_cut > 0, "mtg_set_single_bond: list_cut must be positive");
        MTG_REQUIRE(std::isnan(sb->max_ang) || std::isfinite(sb->max_ang), "mtg_set_single_bond: max_ang must be finite or NAN");
        // patch numbering (GeneralPatch total_patches_per_type) and the FP64 constants of every replica
        std::vector<mtg::BindRep> br((size_t)nrep);
        std::vector<int> pslot(1, 0);
        int64_t poff = 0;
        for (int r = 0; r < nrep; r++) {
            const mtg_replica_desc &d = desc[r];
            const mtg_patch_model &m = d.model;
            mtg::BindRep &B = br[(size_t)r];
            std::memset(&B, 0, sizeof(B));
            int base = 0;
            for (int k = 0; k < m.n_types; k++) {
                B.pbase[k] = base;
                base += m.patches_per_type[k] * (m.count_per_type[k] - (k ? m.count_per_type[k - 1] : 0));
            }
            for (int k = m.n_types; k <= mtg::kMaxTypes; k++) B.pbase[k] = base;
            B.patch_off = (int)poff;
            B.npatch = base;
            B.periodic = d.periodic ? 1 : 0;
            B.seed_lo = (uint32_t)d.seed;
            B.seed_hi = (uint32_t)(d.seed >> 32);
            B.box = d.box;
            B.l2s = (d.box / 2.) * (d.box / 2.);
            int no = 0;
            for (int k = 0; k < m.n_types; k++) no += m.patches_per_type[k];
            for (int i = 0; i < no; i++)
                for (int c = 0; c < 3; c++) B.orient[i][c] = m.orient[i][c];
            double mc = 1.0, ma = 0.6;   // ComboPatch defaults (combopatch.h:15)
            const int npots = n_pots_of(m);
            for (int q = 0; q < npots; q++) {
                B.ctm[q] = std::cos(m.params[q][2]);
                B.disp[q] = 1.4 * m.params[q][1];
                mc = std::max(mc, B.disp[q]);
                ma = std::min(ma, B.ctm[q]);
            }
            B.mk2 = mc * mc;
            B.max_dis = mc + 1.;
            B.list_cut2 = sb->list_cut * sb->list_cut;
            B.max_ang = std::isnan(sb->max_ang) ? ma : sb->max_ang;
            for (int q = 0; q < npots; q++) {
                B.ctm_lo[q] = (float)(B.ctm[q] - 2e-5);
                B.ctm_hi[q] = (float)(B.ctm[q] + 2e-5);
                B.disp_f[q] = (float)B.disp[q];
            }
            const double memb2 = std::min(B.list_cut2, B.max_dis * B.max_dis);
            B.mk2_lo = (float)(B.mk2 * (1 - 1e-5));
            B.mk2_hi = (float)(B.mk2 * (1 + 1e-5));
            B.memb2_lo = (float)(memb2 * (1 - 1e-5));
            B.memb2_hi = (float)(memb2 * (1 + 1e-5));
            B.ang_lo = (float)(-0.4 - 4e-5);
            B.ang_hi = (float)(-0.4 + 4e-5);
            B.max_ang_f = (float)B.max_ang;
            MTG_REQUIRE(reps_obs[r].nc >= 1, "mtg_set_single_bond: no cell grid");
            poff += base;
            MTG_REQUIRE(poff < (int64_t)INT32_MAX, "mtg_set_single_bond: too many patches");
            pslot.push_back((int)poff);
        }
        mtg::BindModel hm;
        std::memset(&hm, 0, sizeof(hm));
        hm.rule = bm.species_rule;
        hm.div1 = bm.div1;
        hm.div2 = bm.div2;
        hm.np = bm.np >= 1 ? bm.np : 1;
        std::memcpy(hm.drate, bm.drate, sizeof(hm.drate));
        std::memcpy(hm.trate, bm.trate, sizeof(hm.trate));

        drop_graphs();
        free_bind();
        ptot = (int)poff;
        patch_every = sb->patch_every;
        patch_slot = pslot;
        const size_t np = (size_t)std::max(ptot, 1);
        scratch_threads = std::max(1, sms) * 8;
        scratch_threads = (scratch_threads + mtg::kLargeThreads - 1) / mtg::kLargeThreads * mtg::kLargeThreads;
        MTG_CUDA(cudaMalloc(&d_brep, sizeof(mtg::BindRep) * nrep));
        MTG_CUDA(cudaMalloc(&d_bmodel, sizeof(mtg::BindModel)));
        MTG_CUDA(cudaMalloc(&d_patch_slot, sizeof(int) * (nrep + 1)));
        MTG_CUDA(cudaMalloc(&d_bctr, sizeof(unsigned long long) * mtg::kBindCounters));
        const size_t nn = (size_t)std::max(ntot_, 1);
        // one snapshot set by global index, shared by both buffers
        MTG_CUDA(cudaMalloc(&buf[0].snap_a, sizeof(real) * 4 * nn));
        MTG_CUDA(cudaMalloc(&buf[0].snap_b, sizeof(real) * 4 * nn));
        MTG_CUDA(cudaMalloc(&buf[0].snap_c, sizeof(real) * 4 * nn));
        buf[1].snap_a = buf[0].snap_a;
        buf[1].snap_b = buf[0].snap_b;
        buf[1].snap_c = buf[0].snap_c;
        MTG_CUDA(cudaMalloc(&d_deg, sizeof(unsigned long long) * np));
        MTG_CUDA(cudaMalloc(&d_adj, sizeof(int2) * mtg::kAdjCap * np));
        MTG_CUDA(cudaMalloc(&d_boundto, sizeof(int) * np));
        MTG_CUDA(cudaMalloc(&d_isbound, np));
        MTG_CUDA(cudaMalloc(&d_large, sizeof(int) * np));
        // segment capacities: twice the even share of each list's bound (the warp-chosen segments fill
        // evenly), at least 1024 entries
        tcap = std::max<long long>(1024, 2 * ((long long)np + mtg::kSegs - 1) / mtg::kSegs);
        bcap = std::max<long long>(1024, 2 * ((long long)np / 2 + mtg::kSegs - 1) / mtg::kSegs);
        lcap = std::max<long long>(1024, 2 * (pair_cap + mtg::kSegs - 1) / mtg::kSegs);
        MTG_CUDA(cudaMalloc(&d_touched, sizeof(int) * (size_t)tcap * mtg::kSegs));
        if (use_pipe) {
            MTG_CUDA(cudaMalloc(&d_bind_pairs, sizeof(int2) * (size_t)lcap * mtg::kSegs));
            // patch pairs within a margin of a float threshold (margins a few 1e-5 wide: of the order of one
            // per thousand tested); room for one per 16 patches, and a full segment latches MTG_FLAG_BIND
            rcap = std::max<long long>(1024, ((long long)np / 16 + mtg::kSegs - 1) / mtg::kSegs);
            MTG_CUDA(cudaMalloc(&d_recheck, sizeof(int2) * (size_t)rcap * mtg::kSegs));
            MTG_CUDA(cudaMalloc(&d_bound, sizeof(int2) * (size_t)bcap * mtg::kSegs));
        }
        MTG_CUDA(cudaMalloc(&d_scratch, sizeof(int) * (size_t)mtg::kScratchInts * scratch_threads));
        MTG_CUDA(cudaMemcpy(d_brep, br.data(), sizeof(mtg::BindRep) * nrep, cudaMemcpyHostToDevice));
        MTG_CUDA(cudaMemcpy(d_bmodel, &hm, sizeof(hm), cudaMemcpyHostToDevice));
        bind_model_h = hm;
        MTG_CUDA(cudaMemcpy(d_patch_slot, pslot.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice));
        MTG_CUDA(cudaMemset(d_bctr, 0, sizeof(unsigned long long) * mtg::kBindCounters));
        MTG_CUDA(cudaMemset(d_deg, 0, sizeof(unsigned long long) * np));
        {   // BinaryBindStore starts zeroed (boundto 0 in replica-local numbering: the replica's first patch)
            std::vector<int> g0(np, 0);
            for (int r = 0; r < nrep; r++)
                for (int i = pslot[(size_t)r]; i < pslot[(size_t)r + 1]; i++) g0[(size_t)i] = pslot[(size_t)r];
            MTG_CUDA(cudaMemcpy(d_boundto, g0.data(), sizeof(int) * np, cudaMemcpyHostToDevice));
        }
        MTG_CUDA(cudaMemset(d_isbound, 0, np));
        ensure_slot_of();
        // the force pass keeps the WCA core and no patch term; its pair loop reaches max_check, where edges
        // can form, on the grid of the observable pass (cells >= max(force range, max_check))
        if (!single_bond) {
            reps_full = reps;
            ncells_full = ncells;
        }
        reps = reps_full;
        for (int r = 0; r < nrep; r++) {
            const double hs = 1.12246 * desc[r].hs_sigma * (1 + 1e-6);
            const double mk2 = br[(size_t)r].mk2 * (1 + 1e-5);
            reps[r].patch_r2 = (real)0;
            reps[r].rc2 = (real)std::max(hs * hs, mk2);
            reps[r].rc2_find = (real)find_range2(std::sqrt(std::max(hs * hs, mk2)), desc[r].box);
            reps[r].nc = reps_obs[r].nc;
            reps[r].nc_mul = reps_obs[r].nc_mul;
            reps[r].nc_sh = reps_obs[r].nc_sh;
            reps[r].cell_off = reps_obs[r].cell_off;
            reps[r].cell_scale = reps_obs[r].cell_scale;
        }
        ncells = ncells_obs;
        MTG_CUDA(cudaMemcpy(d_reps, reps.data(), sizeof(mtg::Replica<real>) * nrep, cudaMemcpyHostToDevice));
        reps_uniform = pair_uniform(reps);
        single_bond = true;
        forces_ready = false;
        cells_valid = bins_valid = false;
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    int64_t num_patches() const override { return single_bond ? ptot : 0; }
    int64_t patch_offset(int r) const override {
        return single_bond && r >= 0 && r <= nrep ? patch_slot[(size_t)r] : -1;
    }

    void set_bind_state(const int32_t *bt, const uint8_t *ib) override {
        MTG_REQUIRE(single_bond, "mtg_set_bind_state: the handle is not in single-bond mode");
        MTG_REQUIRE(bt && ib, "mtg_set_bind_state: boundto and isbound are required");
        std::vector<int> g((size_t)std::max(ptot, 1));
        std::vector<unsigned char> b((size_t)std::max(ptot, 1));
        for (int r = 0; r < nrep; r++) {
            const int o = patch_slot[(size_t)r], n = patch_slot[(size_t)r + 1] - o;
            for (int i = 0; i < n; i++) {
                const int v = bt[o + i];
                MTG_REQUIRE(v >= 0 && v < n, "mtg_set_bind_state: boundto[" + std::to_string(o + i) + "] = " +
                                                 std::to_string(v) + " is not a patch of its replica");
                g[(size_t)(o + i)] = o + v;
                b[(size_t)(o + i)] = ib[o + i] ? 1 : 0;
            }
        }
        MTG_CUDA(cudaMemcpyAsync(d_boundto, g.data(), sizeof(int) * (size_t)ptot, cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaMemcpyAsync(d_isbound, b.data(), (size_t)ptot, cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    void get_bind_state(int32_t *bt, uint8_t *ib) override {
        MTG_REQUIRE(single_bond, "mtg_get_bind_state: the handle is not in single-bond mode");
        std::vector<int> g((size_t)std::max(ptot, 1));
        std::vector<unsigned char> b((size_t)std::max(ptot, 1));
        MTG_CUDA(cudaMemcpyAsync(g.data(), d_boundto, sizeof(int) * (size_t)ptot, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaMemcpyAsync(b.data(), d_isbound, (size_t)ptot, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        for (int r = 0; r < nrep; r++) {
            const int o = patch_slot[(size_t)r], n = patch_slot[(size_t)r + 1] - o;
            for (int i = 0; i < n; i++) {
                if (bt) bt[o + i] = g[(size_t)(o + i)] - o;
                if (ib) ib[o + i] = b[(size_t)(o + i)];
            }
        }
    }

    // -log(1e-10 + calculate_score(wp1, wp2, before)) of every doublet row: BindingModelSingle returns
    // off_rate when the pair is bound to each other, else on_rate (BindingModelSingle.cpp:25-36; its table
    // holds them as [0] = [2] = off, [1] = [3] = on); BindingModelBinary the table's [3] / [0]
    // (BindingModelBinary.cpp:194-230); BindingModelTernary [before * 2 + 1] (BindingModelTernary.cpp:596-640)
    mtg::SetupScores setup_scores() const {
        mtg::SetupScores sc;
        const mtg::BindModel &m = bind_model_h;
        for (int row = 0; row < 6; row++)
            for (int before = 0; before < 2; before++) {
                const double *rt = m.drate[m.rule == 0 ? 0 : row];
                const double score = m.rule == 0 ? (before ? rt[2] : rt[1])
                                                 : (m.rule == 1 ? (before ? rt[3] : rt[0]) : rt[before * 2 + 1]);
                sc.scr4[row][before] = -std::log(1e-10 + score);
            }
        return sc;
    }

    // LangevinNVTR::setup_random_binding (LangevinRforceUtil.cpp:749-1010) with a seeded order (mtg_bind.cuh):
    // this update's edges at the current state (candidate list rebuilt), then rounds of mutual choices until
    // a round binds nothing
    void setup_random_binding(uint64_t seed) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_setup_random_binding: no state has been set"};
        MTG_REQUIRE(single_bond, "mtg_setup_random_binding: the handle is not in single-bond mode");
        if (!cells_valid) rebuild_cells(false);
        enqueue_bind_begin(cur, 1, 0);
        mtg::ForceArgs<real> a = force_args(cur, 0);
        a.bind_deg = d_deg;
        a.bind_adj = d_adj;
        a.bind_ctr = d_bctr;
        a.bind_touched = d_touched;
        a.bind_tcap = tcap;
        a.bind_listed = 0;
        mtg::force_kernel<real, mtg::kModeEdges><<<grid_for(ntot_, 128, occ_force, sms), 128, 0, st>>>(a);
        check_launch();
        counted(1);
        const size_t np = (size_t)std::max(ptot, 1);
        uint32_t *d_prio = nullptr;
        unsigned char *d_ok = nullptr;
        int *d_best = nullptr;
        unsigned long long *d_cnt = nullptr;
        auto release = [&]() {
            cudaFree(d_prio);
            cudaFree(d_ok);
            cudaFree(d_best);
            cudaFree(d_cnt);
        };
        try {
            MTG_CUDA(cudaMalloc(&d_prio, sizeof(uint32_t) * mtg::kAdjCap * np));
            MTG_CUDA(cudaMalloc(&d_ok, mtg::kAdjCap * np));
            MTG_CUDA(cudaMalloc(&d_best, sizeof(int) * np));
            MTG_CUDA(cudaMalloc(&d_cnt, sizeof(unsigned long long)));
            const mtg::BindState S = bind_state();
            const int g = grid_for(ptot, 256, occ_stream, sms);
            mtg::setup_edges_kernel<real><<<g, 256, 0, st>>>(a, S, setup_scores(), seed, d_prio, d_ok);
            check_launch();
            counted(1);
            bool done = false;
            for (int round = 0; round < 4096 && !done; round++) {   // every round binds at least one edge
                MTG_CUDA(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), st));
                mtg::setup_choose_kernel<<<g, 256, 0, st>>>(S, d_prio, d_ok, d_best);
                mtg::setup_commit_kernel<<<g, 256, 0, st>>>(S, d_best, d_cnt);
                check_launch();
                counted(2);
                unsigned long long bound = 0;
                MTG_CUDA(cudaMemcpyAsync(&bound, d_cnt, sizeof(bound), cudaMemcpyDeviceToHost, st));
                MTG_CUDA(cudaStreamSynchronize(st));
                done = bound == 0;
            }
            if (!done) throw Fail{MTG_ERR_TIMEOUT, "mtg_setup_random_binding: the matching did not finish in 4096 rounds"};
        } catch (...) {
            release();
            throw;
        }
        release();
        forces_ready = false;
    }

    void bind_update(double *F, double *T) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_bind_update: no state has been set"};
        MTG_REQUIRE(single_bond, "mtg_bind_update: the handle is not in single-bond mode");
        if (!cells_valid) rebuild_cells(false);
        tick_draw();
        enqueue_bind_begin(cur, 1, 0);
        size_t n = (size_t)ntot_;
        double *sF = d_stage, *sT = sF + 3 * n;
        mtg::ForceArgs<real> a = force_args(cur, 0);
        a.outF = sF;
        a.outT = sT;
        launch_force<mtg::kModeForces>(a, true);
        check_launch();
        if (F) MTG_CUDA(cudaMemcpyAsync(F, sF, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (T) MTG_CUDA(cudaMemcpyAsync(T, sT, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    // force pass in the given mode: the FP32 tile kernel where it applies, else the per-particle kernel.
    // In single-bond mode a bond-deciding pass (bind) records this update's edges in its pair loop and runs
    // the bond decisions before the forces of the bound pairs are summed (events: around the decisions).
    template <int MODE>
    void launch_force(const mtg::ForceArgs<real> &a0, bool bind = false, cudaEvent_t *bind_ev = nullptr) {
        mtg::ForceArgs<real> a = a0;
        bind = bind && single_bond;
        // the FP64 pipeline has no single-bond kernels: FP64 single-bond passes run per particle
        const bool piped = use_pipe && MODE != mtg::kModeObs && !a.outE &&
                           (std::is_same<real, float>::value || !single_bond);
        const bool listed = bind && piped;
        if (bind) {
            a.bind_deg = d_deg;
            a.bind_adj = d_adj;
            a.bind_ctr = d_bctr;
            a.bind_touched = d_touched;
            a.bind_tcap = tcap;
            a.bind_recheck = d_recheck;
            a.bind_rcap = rcap;
            a.bind_listed = listed ? 1 : 0;
        }
        auto decide = [&]() {
            if (bind_ev) MTG_CUDA(cudaEventRecord(bind_ev[0], st));
            enqueue_bind_decide(a, listed);
            if (bind_ev) MTG_CUDA(cudaEventRecord(bind_ev[1], st));
        };
        if (piped) {
            // with a skin the list is rebuilt only on rebuild steps (the gate); the force and epilogue
            // passes run every time
            const int *gate = skin > 0 ? d_skin : nullptr;
            auto mark = [&](int k) {
                if (prof_ev) MTG_CUDA(cudaEventRecord(prof_ev[k], st));
            };
            mark(0);
            mtg::pair_reset_kernel<<<1, 64, 0, st>>>(d_npairs, gate, bind ? nullptr : d_patch_ctr);
            // fused pair finding + WCA / pre-test (no list reuse): the pair kernel then only takes the pairs beyond
            // the warps' buffers.  A bond-deciding pass (FP32) fuses its own pair stage, which lists the bond
            // pass's candidate pairs.
            const bool fused = lc.fused_pairs && skin <= 0;
            {
                const int t = lc.pairfind_threads, gb = std::max(1, (ntot_ + t - 1) / t), rl = skin > 0 ? 1 : 0;
                auto find = [&](auto threads, auto stage) {
                    constexpr int T = decltype(threads)::value;
                    constexpr int SG = decltype(stage)::value;
                    if constexpr (SG == mtg::kPairBind)
                        mtg::pairfind_kernel<real, T, SG><<<gb, T, 0, st>>>(a, d_pairs, d_npairs, pair_cap, rl, gate,
                                                                            d_acc, d_bind_pairs, lcap, nullptr);
                    else
                        mtg::pairfind_kernel<real, T, SG><<<gb, T, 0, st>>>(a, d_pairs, d_npairs, pair_cap, rl, gate,
                                                                            d_acc, d_patch_list, patch_cap, d_patch_ctr);
                };
                auto with_stage = [&](auto threads) {
                    using S0 = std::integral_constant<int, 0>;
                    using SP = std::integral_constant<int, mtg::kPairSplit>;
                    if (!fused) {
                        find(threads, S0{});
                    } else if (bind) {
                        if constexpr (std::is_same<real, float>::value)
                            find(threads, std::integral_constant<int, mtg::kPairBind>{});
                        else
                            find(threads, S0{});   // (not reached: FP64 bond-deciding passes are not piped)
                    } else {
                        find(threads, SP{});
                    }
                };
                if (t == 128) with_stage(std::integral_constant<int, 128>{});
                else if (t == 512) with_stage(std::integral_constant<int, 512>{});
                else with_stage(std::integral_constant<int, 256>{});
            }
            mark(1);
            // after fused pair finding the pair-force kernel only takes the pairs beyond the warps' buffers
            // (normally none): one block per SM, so that its launch and exit cost little
            const int g_force = fused ? sms : sms * lc.pairforce_blocks_per_sm, g_patch = sms * lc.patch_blocks_per_sm;
            bool bind_pass = false;
            if constexpr (std::is_same<real, float>::value) {
                if (bind) {
                    bind_pass = true;
                    mtg::pairforce_kernel<float, mtg::kPairBind><<<g_force, mtg::kPipeThreads, 0, st>>>(
                        a, d_pairs, d_npairs, pair_cap, d_acc, d_bind_pairs, lcap);
                    mark(2);
                    mtg::bind_pairs_kernel<<<g_patch, mtg::kPipeThreads, 0, st>>>(a, d_bind_pairs, lcap);
                    mtg::bind_recheck_kernel<<<sms, mtg::kPipeThreads, 0, st>>>(a);
                    decide();
                    mtg::bound_pairs_kernel<<<sms * 4, mtg::kPipeThreads, 0, st>>>(a, d_bound, bcap, d_acc);
                }
            }
            if (!bind_pass) {
                mtg::pairforce_kernel<real, mtg::kPairSplit><<<g_force, mtg::kPipeThreads, 0, st>>>(
                    a, d_pairs, d_npairs, pair_cap, d_acc, d_patch_list, patch_cap, d_patch_ctr);
                mark(2);
                mtg::patch_pairs_kernel<real><<<g_patch, mtg::kPipeThreads, 0, st>>>(a, d_patch_list, patch_cap,
                                                                                   d_patch_ctr, d_acc);
            }
            mark(3);
            {
                const int t = lc.epilogue_threads, ge = std::max(1, (ntot_ + t - 1) / t);
                if (t == 128) mtg::pair_epilogue_kernel<real, MODE, 128><<<ge, 128, 0, st>>>(a, d_acc);
                else if (t == 512) mtg::pair_epilogue_kernel<real, MODE, 512><<<ge, 512, 0, st>>>(a, d_acc);
                else mtg::pair_epilogue_kernel<real, MODE, 256><<<ge, 256, 0, st>>>(a, d_acc);
            }
            mark(4);
            counted(bind_pass ? 7 : 5);  // (enqueue_bind_decide counts its own)
            return;
        }
        if constexpr (std::is_same<real, float>::value) {
            if (use_tiles && MODE != mtg::kModeObs && !a.outE && a.parts == 3) {
                const int g = std::max(1, std::min(ntiles, occ_tile * sms));  // persistent: one CTA per SM
                mtg::tile_force_kernel<MODE><<<g, mtg::kTileThreads, tile_smem, st>>>(a, d_tiles, ntiles);
                counted(1);
                return;
            }
        }
        const int gf = grid_for(ntot_, 128, occ_force, sms);
        if (bind) {   // the per-particle form: an edges-only pass, the decisions, then the force pass
            mtg::force_kernel<real, mtg::kModeEdges><<<gf, 128, 0, st>>>(a);
            counted(1);
            decide();
            a.bind_deg = nullptr;
        }
        mtg::force_kernel<real, MODE><<<gf, 128, 0, st>>>(a);
        counted(1);
    }

    // a skin-list step on buffer b (which stays the buffer in use): the decision, then either the
    // rebuild (binning, scan, scatter b -> b^1, copy back) or the in-place first half-step, then the force
    // pass in build or list mode -- one launch sequence, the unused branch's kernels return at once
    void enqueue_skin_step(int b, const double *ext_noise) {
        mtg::Tables<real> tb = tables();
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::skin_decide_kernel<<<1, 32, 0, st>>>(d_skin, d_draw);
        mtg::bin_kernel<real, true><<<g, 256, 0, st>>>(tb, buf[b], d_bin, d_count, d_flags, d_skin);
        int nblk = std::max(1, (ncells + mtg::kScanTile - 1) / mtg::kScanTile);
        mtg::scan_reduce_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, ncells, d_block, d_skin);
        mtg::scan_top_kernel<<<1, mtg::kScanThreads, 0, st>>>(d_block, nblk, d_start, ncells, d_draw, 0, d_skin);
        mtg::scan_down_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, ncells, d_block, d_start, d_skin);
        mtg::scatter_kernel<real, true><<<g, 256, 0, st>>>(tb, buf[b], buf[b ^ 1], d_bin, d_start, d_flags, d_skin);
        mtg::copy_back_kernel<real><<<g, 256, 0, st>>>(ntot_, buf[b ^ 1], buf[b], d_skin);
        mtg::integrate_kernel<real><<<g, 256, 0, st>>>(tb, buf[b], d_flags, d_skin);
        counted(8);
        mtg::ForceArgs<real> a = force_args(b, 1);
        a.ext_noise = ext_noise;
        launch_force<mtg::kModeStep>(a);
        check_launch();
    }

    void count_rebuild() {
        int h[4];
        MTG_CUDA(cudaMemcpyAsync(h, d_skin, sizeof(h), cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        h[3] += 1;
        MTG_CUDA(cudaMemcpyAsync(d_skin + 3, h + 3, sizeof(int), cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    void set_skin(int now, int next, int forced) {
        mtg::skin_set_kernel<<<1, 32, 0, st>>>(d_skin, now, next, forced);
        check_launch();
        nlaunch += 1;
    }

    int64_t rebuilds() override {
        if (skin <= 0) return 0;
        int h[4];
        MTG_CUDA(cudaMemcpyAsync(h, d_skin, sizeof(h), cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        return h[3];
    }

    // one step from buffer b: scan (+draw), scatter b -> b^1, force on b^1
    void enqueue_step(int b, const double *ext_noise) {
        if (skin > 0) {
            enqueue_skin_step(b, ext_noise);
            return;
        }
        mtg::Tables<real> tb = tables();
        if (single_bond) enqueue_bind_begin(b, 0, 1);
        scan(ncells, true);
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::scatter_kernel<real, true><<<g, 256, 0, st>>>(tb, buf[b], buf[b ^ 1], d_bin, d_start, d_flags, nullptr,
                                                           single_bond ? d_bctr + 4 : nullptr);
        counted(1);
        mtg::ForceArgs<real> a = force_args(b ^ 1, 1);
        a.ext_noise = ext_noise;
        launch_force<mtg::kModeStep>(a, true);
        check_launch();
    }

    void set_state(const double *x, const double *p, const double *Lb, const double *Q, const double *Ft,
                   const double *Tt) override {
        MTG_REQUIRE(x && p && Lb && Q, "mtg_set_state: x, p, Lb and Q are required");
        size_t n = (size_t)ntot_;
        double *sx = d_stage, *sp = sx + 3 * n, *sl = sp + 3 * n, *sq = sl + 3 * n, *sf = sq + 9 * n, *stt = sf + 3 * n;
        MTG_CUDA(cudaMemcpyAsync(sx, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaMemcpyAsync(sp, p, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaMemcpyAsync(sl, Lb, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaMemcpyAsync(sq, Q, sizeof(double) * 9 * n, cudaMemcpyHostToDevice, st));
        if (Ft) MTG_CUDA(cudaMemcpyAsync(sf, Ft, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        if (Tt) MTG_CUDA(cudaMemcpyAsync(stt, Tt, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::load_state_kernel<real><<<g, 256, 0, st>>>(ntot_, sx, sp, sl, sq, Ft ? sf : nullptr, Tt ? stt : nullptr,
                                                        buf[cur]);
        check_launch();
        nlaunch += 1;
        have_state = true;
        cells_valid = bins_valid = false;
        forces_ready = Ft && Tt;
    }

    mtg_status get_state(double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_get_state: no state has been set"};
        size_t n = (size_t)ntot_;
        double *sx = d_stage, *sp = sx + 3 * n, *sl = sp + 3 * n, *sq = sl + 3 * n, *sf = sq + 9 * n, *stt = sf + 3 * n;
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        // the slot of every global index: the maintained map when there is one (bonds, single-bond mode),
        // else a map built here into scratch kept for later calls
        const int *map = d_slot_of;
        if (!map) {
            if (!d_gather_map) MTG_CUDA(cudaMalloc(&d_gather_map, sizeof(int) * (size_t)std::max(ntot_, 1)));
            mtg::slot_map_kernel<<<g, 256, 0, st>>>(ntot_, buf[cur].ident, d_gather_map);
            check_launch();
            nlaunch += 1;
            map = d_gather_map;
        }
        mtg::gather_state_kernel<real><<<g, 256, 0, st>>>(ntot_, buf[cur], map, x ? sx : nullptr, p ? sp : nullptr,
                                                          Lb ? sl : nullptr, Q ? sq : nullptr, Ft ? sf : nullptr,
                                                          Tt ? stt : nullptr);
        check_launch();
        nlaunch += 1;
        if (x) MTG_CUDA(cudaMemcpyAsync(x, sx, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (p) MTG_CUDA(cudaMemcpyAsync(p, sp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (Lb) MTG_CUDA(cudaMemcpyAsync(Lb, sl, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (Q) MTG_CUDA(cudaMemcpyAsync(Q, sq, sizeof(double) * 9 * n, cudaMemcpyDeviceToHost, st));
        if (Ft) MTG_CUDA(cudaMemcpyAsync(Ft, sf, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (Tt) MTG_CUDA(cudaMemcpyAsync(Tt, stt, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        return (flags() & MTG_FLAG_NONFINITE) ? MTG_ERR_NONFINITE : MTG_OK;
    }

    void displacement(double *disp) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_get_displacement: no state has been set"};
        if (!track_disp) throw Fail{MTG_ERR_STATE, "mtg_get_displacement: handle created without displacement tracking"};
        size_t n = (size_t)ntot_;
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::store_state_kernel<real><<<g, 256, 0, st>>>(ntot_, buf[cur], nullptr, nullptr, nullptr, nullptr, nullptr,
                                                         nullptr, d_stage);
        check_launch();
        nlaunch += 1;
        MTG_CUDA(cudaMemcpyAsync(disp, d_stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    // the device draw counter <- (now, next)
    void set_device_draw(unsigned long long now, unsigned long long next) {
        mtg::draw_set_kernel<<<1, 32, 0, st>>>(d_draw, now, next);
        check_launch();
        counted(1);
    }

    void tick_draw() {
        // draw[0] <- draw[1]++ for a pass that does not run the scan
        set_device_draw(draw, draw + 1);
        draw += 1;
    }

    const double *upload_noise(const double *noise) {
        size_t n = (size_t)ntot_;
        if (!d_noise) MTG_CUDA(cudaMalloc(&d_noise, sizeof(double) * 6 * std::max<size_t>(n, 1)));
        MTG_CUDA(cudaMemcpyAsync(d_noise, noise, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, st));
        return d_noise;
    }

    void init_forces(const double *noise) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_init_forces: no state has been set"};
        rebuild_cells(false);
        tick_draw();
        if (skin > 0) {
            set_skin(1, 0, 0);  // this pass builds the lists (a rebuild)
            count_rebuild();
        }
        if (single_bond) {   // run_singlebond's first onlyone_nonlets call (Condensate.cpp:455-460)
            enqueue_bind_begin(cur, 1, 0);
        }
        mtg::ForceArgs<real> a = force_args(cur, 0);
        if (noise) a.ext_noise = upload_noise(noise);
        launch_force<mtg::kModeInit>(a, true);
        check_launch();
        cells_valid = true;
        bins_valid = true;
        forces_ready = true;
    }

    void build_graph(int b) {
        cudaGraph_t g;
        MTG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        {
            struct Capturing {
                bool &f;
                explicit Capturing(bool &x) : f(x) { f = true; }
                ~Capturing() { f = false; }
            } guard(capturing);  // cleared on every exit, an exception included
            enqueue_step(b, nullptr);
        }
        MTG_CUDA(cudaStreamEndCapture(st, &g));
        size_t nn = 0;
        MTG_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) MTG_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
        int k = 0;
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType t;
            MTG_CUDA(cudaGraphNodeGetType(nd, &t));
            if (t == cudaGraphNodeTypeKernel) k++;
        }
        graph_kernels[b] = k;
        MTG_CUDA(cudaGraphInstantiate(&graph[b], g, 0));
        MTG_CUDA(cudaGraphDestroy(g));
    }

    // MD::calculateforces(bond list, HarmonicPotential(k, r0)) added to every force pass from now on
    void set_bonds(const int32_t *bonds, int64_t nb, double k, double r0) override {
        MTG_REQUIRE(nb >= 0 && (nb == 0 || bonds), "mtg_set_bonds: nbonds must be >= 0 and bonds non-null");
        MTG_REQUIRE(std::isfinite(k) && std::isfinite(r0) && r0 >= 0, "mtg_set_bonds: k and r0 must be finite, r0 >= 0");
        MTG_REQUIRE(nb <= (int64_t)INT32_MAX / 2, "mtg_set_bonds: too many bonds");
        // every bond joins two different particles of one replica (host-order global indices)
        std::vector<int> deg((size_t)ntot_ + 1, 0);
        auto replica_of = [&](int i) {
            return (int)(std::upper_bound(rep_slot.begin(), rep_slot.end(), i) - rep_slot.begin()) - 1;
        };
        for (int64_t q = 0; q < nb; q++) {
            const int a = bonds[2 * q], b = bonds[2 * q + 1];
            MTG_REQUIRE(a >= 0 && a < ntot_ && b >= 0 && b < ntot_ && a != b,
                        "mtg_set_bonds: bond " + std::to_string(q) + " joins " + std::to_string(a) + " and " +
                            std::to_string(b) + " (the indices must differ and lie in [0, " + std::to_string(ntot_) + "))");
            MTG_REQUIRE(replica_of(a) == replica_of(b),
                        "mtg_set_bonds: bond " + std::to_string(q) + " joins particles of two replicas");
            deg[(size_t)a + 1]++;
            deg[(size_t)b + 1]++;
        }
        for (int i = 0; i < ntot_; i++) deg[(size_t)i + 1] += deg[i];
        std::vector<int> partner((size_t)std::max<int64_t>(1, 2 * nb)), fill(deg.begin(), deg.end() - 1);
        for (int64_t q = 0; q < nb; q++) {
            const int a = bonds[2 * q], b = bonds[2 * q + 1];
            partner[(size_t)fill[a]++] = b;
            partner[(size_t)fill[b]++] = a;
        }
        MTG_CUDA(cudaStreamSynchronize(st));
        cudaFree(d_bond_start); cudaFree(d_bond_partner);
        d_bond_start = d_bond_partner = nullptr;
        nbonds = 0;
        for (int b = 0; b < 2; b++) {
            if (graph[b]) cudaGraphExecDestroy(graph[b]);
            graph[b] = nullptr;  // captured with the previous force arguments
        }
        if (nb == 0) return;
        MTG_CUDA(cudaMalloc(&d_bond_start, sizeof(int) * ((size_t)ntot_ + 1)));
        MTG_CUDA(cudaMalloc(&d_bond_partner, sizeof(int) * partner.size()));
        MTG_CUDA(cudaMemcpy(d_bond_start, deg.data(), sizeof(int) * deg.size(), cudaMemcpyHostToDevice));
        MTG_CUDA(cudaMemcpy(d_bond_partner, partner.data(), sizeof(int) * partner.size(), cudaMemcpyHostToDevice));
        if (!d_slot_of) {
            MTG_CUDA(cudaMalloc(&d_slot_of, sizeof(int) * (size_t)ntot_));
            buf[0].slot_of = buf[1].slot_of = d_slot_of;
            if (have_state) {
                const int g = grid_for(ntot_, 256, occ_stream, sms);
                mtg::slot_map_kernel<<<g, 256, 0, st>>>(ntot_, buf[cur].ident, d_slot_of);
                check_launch();
                nlaunch += 1;
            }
        }
        nbonds = nb;
        bond_k = k;
        bond_r0 = r0;
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    void step(int nsteps, const double *noise) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_step: no state has been set"};
        MTG_REQUIRE(nsteps >= 0, "mtg_step: nsteps must be >= 0");
        if (!forces_ready) init_forces(nullptr);
        if (single_bond && !cells_valid) rebuild_cells(false);   // the candidate pass reads the force grid
        if (skin > 0) {
            if (!cells_valid) set_skin(-1, -1, 1);  // the buffer was re-sorted by another grid: rebuild first
        } else if (!bins_valid) {
            MTG_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int) * (ncells_alloc + 1), st));
            const int g = grid_for(ntot_, 256, occ_stream, sms);
            mtg::bin_kernel<real, true><<<g, 256, 0, st>>>(tables(), buf[cur], d_bin, d_count, d_flags);
            check_launch();
            nlaunch += 1;
            bins_valid = true;
        }
        // the device draw counter follows the host one
        set_device_draw(draw, draw);
        size_t n = (size_t)ntot_;
        if (noise) {
            for (int s = 0; s < nsteps; s++) {
                enqueue_step(cur, upload_noise(noise + (size_t)s * 6 * n));
                if (skin <= 0) cur ^= 1;  // a skin step leaves the state in the buffer it started in
                draw += 1;
            }
            MTG_CUDA(cudaStreamSynchronize(st));
        } else {
            for (int s = 0; s < nsteps; s++) replay_step();
        }
        cells_valid = true;
        bins_valid = true;
    }

    void step_profile(int nsteps, double *kernel_ms) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_step_profile: no state has been set"};
        MTG_REQUIRE(nsteps >= 1 && kernel_ms, "mtg_step_profile: nsteps >= 1 and an output are required");
        step(0, nullptr);  // initial forces / bins, as mtg_step would
        set_device_draw(draw, draw);
        cudaEvent_t ev[10], pev[5];
        for (auto &e : ev) MTG_CUDA(cudaEventCreate(&e));
        for (auto &e : pev) MTG_CUDA(cudaEventCreate(&e));
        struct Restore {
            cudaEvent_t *&p;
            ~Restore() { p = nullptr; }
        } restore{prof_ev};
        const bool piped = use_pipe && (std::is_same<real, float>::value || !single_bond);  // as launch_force
        if (piped) prof_ev = pev;
        // the pipeline's sub-kernel times of one force pass (pair reset + pairfind, pairforce, patch-pair or
        // edge/bound-pair kernels, epilogue); the decisions between them are slot 6
        auto pipe_times = [&](double *acc, float bind_ms) {
            if (!piped) return;
            for (int k = 0; k < 4; k++) {
                float ms = 0;
                MTG_CUDA(cudaEventElapsedTime(&ms, pev[k], pev[k + 1]));
                acc[7 + k] += k == 2 ? ms - bind_ms : ms;
            }
        };
        double acc[MTG_PROFILE_KERNELS] = {};
        mtg::Tables<real> tb = tables();
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        const int gf = grid_for(ntot_, 128, occ_force, sms);
        int nblk = std::max(1, (ncells + mtg::kScanTile - 1) / mtg::kScanTile);
        for (int s = 0; s < nsteps && skin > 0; s++) {
            const int b = cur;
            MTG_CUDA(cudaEventRecord(ev[0], st));
            mtg::skin_decide_kernel<<<1, 32, 0, st>>>(d_skin, d_draw);
            mtg::bin_kernel<real, true><<<g, 256, 0, st>>>(tb, buf[b], d_bin, d_count, d_flags, d_skin);
            mtg::scan_reduce_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, ncells, d_block, d_skin);
            MTG_CUDA(cudaEventRecord(ev[1], st));
            mtg::scan_top_kernel<<<1, mtg::kScanThreads, 0, st>>>(d_block, nblk, d_start, ncells, d_draw, 0, d_skin);
            MTG_CUDA(cudaEventRecord(ev[2], st));
            mtg::scan_down_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, ncells, d_block, d_start, d_skin);
            MTG_CUDA(cudaEventRecord(ev[3], st));
            mtg::scatter_kernel<real, true><<<g, 256, 0, st>>>(tb, buf[b], buf[b ^ 1], d_bin, d_start, d_flags, d_skin);
            mtg::copy_back_kernel<real><<<g, 256, 0, st>>>(ntot_, buf[b ^ 1], buf[b], d_skin);
            mtg::integrate_kernel<real><<<g, 256, 0, st>>>(tb, buf[b], d_flags, d_skin);
            MTG_CUDA(cudaEventRecord(ev[4], st));
            mtg::ForceArgs<real> a = force_args(b, 1);
            launch_force<mtg::kModeStep>(a);
            MTG_CUDA(cudaEventRecord(ev[5], st));
            check_launch();
            MTG_CUDA(cudaEventSynchronize(ev[5]));
            for (int k = 0; k < 5; k++) {
                float ms = 0;
                MTG_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
                acc[k] += ms;
            }
            pipe_times(acc, 0.f);
            nlaunch += 8;  // the explicit kernels above (launch_force counts its own)
            draw += 1;
        }
        for (int s = 0; s < nsteps && skin <= 0; s++) {
            const int b = cur;
            MTG_CUDA(cudaEventRecord(ev[6], st));
            if (single_bond) enqueue_bind_begin(b, 0, 1);
            MTG_CUDA(cudaEventRecord(ev[7], st));
            MTG_CUDA(cudaEventRecord(ev[8], st));
            MTG_CUDA(cudaEventRecord(ev[9], st));
            MTG_CUDA(cudaEventRecord(ev[0], st));
            mtg::scan_reduce_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, ncells, d_block);
            MTG_CUDA(cudaEventRecord(ev[1], st));
            mtg::scan_top_kernel<<<1, mtg::kScanThreads, 0, st>>>(d_block, nblk, d_start, ncells, d_draw, 1);
            MTG_CUDA(cudaEventRecord(ev[2], st));
            mtg::scan_down_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(d_count, ncells, d_block, d_start);
            MTG_CUDA(cudaEventRecord(ev[3], st));
            mtg::scatter_kernel<real, true><<<g, 256, 0, st>>>(tb, buf[b], buf[b ^ 1], d_bin, d_start, d_flags,
                                                               nullptr, single_bond ? d_bctr + 4 : nullptr);
            MTG_CUDA(cudaEventRecord(ev[4], st));
            mtg::ForceArgs<real> a = force_args(b ^ 1, 1);
            launch_force<mtg::kModeStep>(a, true, ev + 8);
            MTG_CUDA(cudaEventRecord(ev[5], st));
            check_launch();
            MTG_CUDA(cudaEventSynchronize(ev[5]));
            float ms = 0, bind_ms = 0;
            MTG_CUDA(cudaEventElapsedTime(&bind_ms, ev[8], ev[9]));
            for (int k = 0; k < 5; k++) {
                MTG_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
                acc[k] += k == 4 ? ms - bind_ms : ms;
            }
            MTG_CUDA(cudaEventElapsedTime(&ms, ev[6], ev[7]));
            acc[5] += ms;
            acc[6] += bind_ms;
            pipe_times(acc, bind_ms);
            cur ^= 1;
            nlaunch += 4;  // the scans and the scatter (launch_force and bind begin count their own)
            draw += 1;
        }
        for (auto &e : ev) cudaEventDestroy(e);
        for (auto &e : pev) cudaEventDestroy(e);
        for (int k = 0; k < MTG_PROFILE_KERNELS; k++) kernel_ms[k] = acc[k];
        cells_valid = true;
        bins_valid = true;
    }

    void forces(double *F, double *T, double *E) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_forces: no state has been set"};
        MTG_REQUIRE(F && T, "mtg_forces: F and T are required");
        // with a skin the lists are valid for the current positions as long as the sort they were built on is
        ensure_cells();
        size_t n = (size_t)ntot_;
        double *sF = d_stage, *sT = sF + 3 * n, *sE = sT + 3 * n;
        mtg::ForceArgs<real> a = force_args(cur, 0);
        a.outF = sF;
        a.outT = sT;
        a.outE = E ? sE : nullptr;
        launch_force<mtg::kModeForces>(a);
        check_launch();
        MTG_CUDA(cudaMemcpyAsync(F, sF, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaMemcpyAsync(T, sT, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (E) MTG_CUDA(cudaMemcpyAsync(E, sE, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    // ---------------------------------------------------------------- the step's phases one at a time

    // the cell list of the current positions (a phase that moved the particles invalidated it)
    void ensure_cells() {
        if (skin > 0) {
            if (!cells_valid) {
                rebuild_cells(false);
                set_skin(1, -1, -1);
                count_rebuild();
            } else {
                set_skin(0, -1, -1);
            }
        } else if (!cells_valid) {
            rebuild_cells(false);
        }
    }

    // parts 1: MD::calculateforces(pairs, HSPotential) (+ harmonic bonds) into F; parts 2: the patch forces and
    // lab torques of calculate_forces_and_torques3D (bound pairs only in single-bond mode) into F and T
    void phase_forces(int parts, double *F, double *T) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_phase_forces: no state has been set"};
        MTG_REQUIRE(parts == 1 || parts == 2, "mtg_phase_forces: parts must be 1 (central) or 2 (patch)");
        MTG_REQUIRE(F && (parts == 1 || T), "mtg_phase_forces: F (and T for the patch part) are required");
        ensure_cells();
        size_t n = (size_t)ntot_;
        double *sF = d_stage, *sT = sF + 3 * n;
        mtg::ForceArgs<real> a = force_args(cur, 0);
        a.outF = sF;
        a.outT = sT;
        a.parts = parts;
        launch_force<mtg::kModeForces>(a);
        check_launch();
        MTG_CUDA(cudaMemcpyAsync(F, sF, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        if (T) MTG_CUDA(cudaMemcpyAsync(T, sT, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    // create_forces_and_torques_sphere(F, T, R): F (lab) and T (lab) in, F~ (lab) and T~ (body) out, in place
    void phase_langevin(double *F, double *T, const double *noise) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_phase_langevin: no state has been set"};
        MTG_REQUIRE(F && T, "mtg_phase_langevin: F and T are required");
        size_t n = (size_t)ntot_;
        double *sF = d_stage, *sT = sF + 3 * n, *sN = sT + 3 * n, *oF = sN + 6 * n, *oT = oF + 3 * n;
        MTG_CUDA(cudaMemcpyAsync(sF, F, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaMemcpyAsync(sT, T, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        if (noise) MTG_CUDA(cudaMemcpyAsync(sN, noise, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, st));
        else tick_draw();
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::phase_langevin_kernel<real><<<g, 256, 0, st>>>(tables(), buf[cur], sF, sT, noise ? sN : nullptr, d_draw,
                                                           oF, oT, d_flags);
        check_launch();
        nlaunch += 1;
        MTG_CUDA(cudaMemcpyAsync(F, oF, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaMemcpyAsync(T, oT, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        forces_ready = true;
    }

    // advancemom_halfstep(F lab, T body)
    void phase_halfkick(const double *F, const double *T) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_phase_halfkick: no state has been set"};
        MTG_REQUIRE(F && T, "mtg_phase_halfkick: F and T are required");
        size_t n = (size_t)ntot_;
        double *sF = d_stage, *sT = sF + 3 * n;
        MTG_CUDA(cudaMemcpyAsync(sF, F, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        MTG_CUDA(cudaMemcpyAsync(sT, T, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::phase_halfkick_kernel<real><<<g, 256, 0, st>>>(tables(), buf[cur], sF, sT);
        check_launch();
        nlaunch += 1;
        MTG_CUDA(cudaStreamSynchronize(st));
        bins_valid = false;   // the next step's binning came from the old momenta
    }

    // LangevinNVT::advance_pos
    void phase_drift() override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_phase_advance_pos: no state has been set"};
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::phase_drift_kernel<real><<<g, 256, 0, st>>>(tables(), buf[cur], d_flags);
        check_launch();
        nlaunch += 1;
        MTG_CUDA(cudaStreamSynchronize(st));
        cells_valid = bins_valid = false;   // particles left their cells
    }

    // LangevinNVTR::rotate()
    void phase_rotate() override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_phase_rotate: no state has been set"};
        const int g = grid_for(ntot_, 256, occ_stream, sms);
        mtg::phase_rotate_kernel<real><<<g, 256, 0, st>>>(tables(), buf[cur]);
        check_launch();
        nlaunch += 1;
        MTG_CUDA(cudaStreamSynchronize(st));
    }

    // the per-replica sums of p^2 and L^2 at the current state, added to d_dst (6 x nrep doubles, zeroed)
    void enqueue_temperature_sums(double *d_dst) {
        const int chunk = 256 * mtg::kTempPerThread;
        mtg::temperature_kernel<real><<<std::max(1, (ntot_ + chunk - 1) / chunk), 256, 0, st>>>(tables(), buf[cur],
                                                                                              d_dst);
        check_launch();
        nlaunch += 1;
    }
    // the same sums into pinned host memory (asynchronous)
    void enqueue_temperature(double *h_dst) {
        MTG_CUDA(cudaMemsetAsync(d_obs, 0, sizeof(double) * 6 * nrep, st));
        enqueue_temperature_sums(d_obs);
        MTG_CUDA(cudaMemcpyAsync(h_dst, d_obs, sizeof(double) * 6 * nrep, cudaMemcpyDeviceToHost, st));
    }
    // sums -> <p_k^2/2m>, <L_k^2/2I> of each replica
    void normalise_temperature(const double *sums, double *out) const {
        for (int r = 0; r < nrep; r++) {
            double n = (double)desc[r].n;
            for (int k = 0; k < 3; k++) {
                out[6 * r + k] = sums[6 * r + k] / (2. * desc[r].mass) / n;
                out[6 * r + 3 + k] = sums[6 * r + 3 + k] / (2. * desc[r].inertia) / n;
            }
        }
    }
    void ensure_obs_ring(size_t doubles) {
        if (doubles <= h_obs_cap) return;
        if (h_obs) cudaFreeHost(h_obs);
        h_obs = nullptr;
        h_obs_cap = 0;
        MTG_CUDA(cudaMallocHost(&h_obs, sizeof(double) * doubles));  // pinned: asynchronous copies
        h_obs_cap = doubles;
    }

    uint32_t temperature(double *out) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_temperature: no state has been set"};
        ensure_obs_ring((size_t)6 * nrep);
        enqueue_temperature(h_obs);
        MTG_CUDA(cudaMemcpyAsync(h_flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));  // one round trip for the sums and the flags
        normalise_temperature(h_obs, out);
        return *h_flags;
    }

    // one more step of the captured step graph, after a step() call has set the device draw counter
    void replay_step() {
        if (!graph[cur]) build_graph(cur);
        MTG_CUDA(cudaGraphLaunch(graph[cur], st));
        nlaunch += graph_kernels[cur];
        if (skin <= 0) cur ^= 1;
        draw += 1;
    }

    // Every step's sums go to a device ring, zeroed once and copied back once per chunk of steps (at most
    // 32 MB of sums), so that a step adds only the reduction kernel to its graph; the caller sees the same
    // values, since the call returns after its last copy.
    uint32_t step_temperatures(int nsteps, double *out) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_step_temperatures: no state has been set"};
        const size_t per = (size_t)6 * nrep;
        ensure_obs_ring(per * (size_t)std::max(nsteps, 1));
        const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(nsteps, 1),
                                                                    (32u << 20) / (sizeof(double) * per)));
        if (nsteps > 0 && d_tring_cap < per * (size_t)chunk) {
            cudaFree(d_tring);
            d_tring = nullptr;
            d_tring_cap = 0;
            MTG_CUDA(cudaMalloc(&d_tring, sizeof(double) * per * (size_t)chunk));
            d_tring_cap = per * (size_t)chunk;
        }
        for (int s0 = 0; s0 < nsteps; s0 += chunk) {
            const int ns = std::min(chunk, nsteps - s0);
            MTG_CUDA(cudaMemsetAsync(d_tring, 0, sizeof(double) * per * (size_t)ns, st));
            for (int s = 0; s < ns; s++) {
                if (s0 + s == 0) step(1, nullptr);   // forces, bins and the device draw counter, then one step
                else replay_step();
                enqueue_temperature_sums(d_tring + per * (size_t)s);
            }
            MTG_CUDA(cudaMemcpyAsync(h_obs + per * (size_t)s0, d_tring, sizeof(double) * per * (size_t)ns,
                                     cudaMemcpyDeviceToHost, st));
        }
        if (nsteps > 0) {
            cells_valid = true;
            bins_valid = true;
        }
        MTG_CUDA(cudaMemcpyAsync(h_flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        for (int s = 0; s < nsteps; s++) normalise_temperature(h_obs + per * (size_t)s, out + per * (size_t)s);
        return *h_flags;
    }

    void observables(double *out) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_observables: no state has been set"};
        // the bond criterion reaches ComboPatch::max_check, beyond the force range: own cell grid
        rebuild_cells(true);
        MTG_CUDA(cudaMemsetAsync(d_obs, 0, sizeof(double) * 6 * nrep, st));
        mtg::ForceArgs<real> a = force_args(cur, 0);
        a.tb = tables(true);
        a.obs = d_obs;
        std::vector<double> h(6 * (size_t)nrep);
        launch_force<mtg::kModeObs>(a);
        check_launch();
        MTG_CUDA(cudaMemcpyAsync(h.data(), d_obs, sizeof(double) * 6 * nrep, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        for (int r = 0; r < nrep; r++)
            for (int k = 0; k < MTG_OBS_COUNT; k++) out[MTG_OBS_COUNT * r + k] = h[5 * (size_t)r + k];
        cells_valid = false;  // the buffer is now ordered by the observable grid
        bins_valid = false;
    }

    mtg_status pairs(int replica, double rc, int32_t *out, int64_t cap, int64_t *npairs) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_pairs: no state has been set"};
        MTG_REQUIRE(replica >= 0 && replica < nrep, "mtg_pairs: replica out of range");
        MTG_REQUIRE(rc > 0 && npairs, "mtg_pairs: rc must be positive and npairs non-null");
        const mtg_replica_desc &d = desc[replica];
        const int nc = analysis_cells(d.box, rc, d.n);
        const int ncell = nc * nc * nc;
        int n = d.n;
        int off = rep_slot[replica];
        // device scratch: bins, counts, starts, members, per-particle pair counts, offsets, pairs
        int2 *pbin = nullptr;
        int *pcount = nullptr, *pstart = nullptr, *pmem = nullptr, *pcnt = nullptr, *poff = nullptr, *pblock = nullptr;
        int32_t *pout = nullptr;
        mtg_status result = MTG_OK;
        auto cleanup = [&]() {
            cudaFree(pbin); cudaFree(pcount); cudaFree(pstart); cudaFree(pmem); cudaFree(pcnt); cudaFree(poff);
            cudaFree(pblock); cudaFree(pout);
        };
        try {
            size_t nn = (size_t)std::max(n, 1);
            MTG_CUDA(cudaMalloc(&pbin, sizeof(int2) * nn));
            MTG_CUDA(cudaMalloc(&pcount, sizeof(int) * (ncell + 1)));
            MTG_CUDA(cudaMalloc(&pstart, sizeof(int) * (ncell + 1)));
            MTG_CUDA(cudaMalloc(&pmem, sizeof(int) * nn));
            MTG_CUDA(cudaMalloc(&pcnt, sizeof(int) * nn));
            MTG_CUDA(cudaMalloc(&poff, sizeof(int) * (nn + 1)));
            int nblk = (ncell + mtg::kScanTile - 1) / mtg::kScanTile + 1;
            MTG_CUDA(cudaMalloc(&pblock, sizeof(int) * nblk));
            MTG_CUDA(cudaMemsetAsync(pcount, 0, sizeof(int) * (ncell + 1), st));
            mtg::PairGrid grid{off, n, nc, d.box, (double)nc / d.box, d.periodic ? 1 : 0, rc};
            const int g = grid_for(n, 256, occ_stream, sms);
            mtg::pair_bin_kernel<real><<<g, 256, 0, st>>>(grid, buf[cur], pbin, pcount);
            int nb = (ncell + mtg::kScanTile - 1) / mtg::kScanTile;
            if (nb < 1) nb = 1;
            mtg::scan_reduce_kernel<<<nb, mtg::kScanThreads, 0, st>>>(pcount, ncell, pblock);
            mtg::scan_top_kernel<<<1, mtg::kScanThreads, 0, st>>>(pblock, nb, pstart, ncell, d_draw, 0);
            mtg::scan_down_kernel<<<nb, mtg::kScanThreads, 0, st>>>(pcount, ncell, pblock, pstart);
            mtg::pair_fill_kernel<<<g, 256, 0, st>>>(grid, pbin, pstart, pmem);
            mtg::pair_count_kernel<real><<<g, 256, 0, st>>>(grid, buf[cur], pstart, pmem, pcnt);
            check_launch();
            std::vector<int> hc(n + 1, 0), ho(n + 1, 0);
            MTG_CUDA(cudaMemcpyAsync(hc.data(), pcnt, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
            MTG_CUDA(cudaStreamSynchronize(st));
            int64_t total = 0;
            for (int i = 0; i < n; i++) total += hc[i];
            *npairs = total;
            // the per-particle offsets and the write kernel index pairs with int
            if (out && total <= cap && total > (int64_t)INT32_MAX)   // (the handler below frees the scratch)
                throw Fail{MTG_ERR_CAPACITY, "mtg_pairs: " + std::to_string(total) +
                                                 " pairs exceed the 2^31 - 1 this call can write"};
            total = 0;
            for (int i = 0; i < n; i++) {
                ho[i] = (int)total;
                total += hc[i];
            }
            ho[n] = (int)total;
            if (total > cap || !out) {
                cleanup();
                return total > cap ? MTG_ERR_CAPACITY : MTG_OK;
            }
            MTG_CUDA(cudaMalloc(&pout, sizeof(int32_t) * 2 * std::max<int64_t>(total, 1)));
            MTG_CUDA(cudaMemcpyAsync(poff, ho.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
            mtg::pair_write_kernel<real><<<g, 256, 0, st>>>(grid, buf[cur], pstart, pmem, poff, pout);
            check_launch();
            std::vector<int32_t> hp(2 * (size_t)total);
            MTG_CUDA(cudaMemcpyAsync(hp.data(), pout, sizeof(int32_t) * 2 * total, cudaMemcpyDeviceToHost, st));
            MTG_CUDA(cudaStreamSynchronize(st));
            nlaunch += 7;
            // each particle's segment holds its partners j > i; sort them
            for (int i = 0; i < n; i++) {
                std::vector<int32_t> seg;
                for (int q = ho[i]; q < ho[i + 1]; q++) seg.push_back(hp[2 * (size_t)q + 1]);
                std::sort(seg.begin(), seg.end());
                for (int q = ho[i]; q < ho[i + 1]; q++) {
                    out[2 * (size_t)q] = i;
                    out[2 * (size_t)q + 1] = seg[q - ho[i]];
                }
            }
        } catch (...) {
            cleanup();
            throw;
        }
        cleanup();
        return result;
    }

    // one replica binned on a grid of side >= rc (the analysis passes); frees its device arrays
    struct ReplicaCells {
        mtg::PairGrid grid{};
        int ncell = 0;
        int2 *bin = nullptr;
        int *count = nullptr, *start = nullptr, *mem = nullptr, *block = nullptr;
        ~ReplicaCells() { cudaFree(bin); cudaFree(count); cudaFree(start); cudaFree(mem); cudaFree(block); }
    };

    void bin_replica(int replica, double rc, ReplicaCells &c) {
        const mtg_replica_desc &d = desc[replica];
        const int nc = analysis_cells(d.box, rc, d.n);
        c.ncell = nc * nc * nc;
        const int n = d.n;
        size_t nn = (size_t)std::max(n, 1);
        MTG_CUDA(cudaMalloc(&c.bin, sizeof(int2) * nn));
        MTG_CUDA(cudaMalloc(&c.count, sizeof(int) * (c.ncell + 1)));
        MTG_CUDA(cudaMalloc(&c.start, sizeof(int) * (c.ncell + 1)));
        MTG_CUDA(cudaMalloc(&c.mem, sizeof(int) * nn));
        const int nb = std::max(1, (c.ncell + mtg::kScanTile - 1) / mtg::kScanTile);
        MTG_CUDA(cudaMalloc(&c.block, sizeof(int) * (nb + 1)));
        MTG_CUDA(cudaMemsetAsync(c.count, 0, sizeof(int) * (c.ncell + 1), st));
        c.grid = mtg::PairGrid{rep_slot[replica], n, nc, d.box, (double)nc / d.box, d.periodic ? 1 : 0, rc};
        const int g = grid_for(n, 256, occ_stream, sms);
        mtg::pair_bin_kernel<real><<<g, 256, 0, st>>>(c.grid, buf[cur], c.bin, c.count);
        mtg::scan_reduce_kernel<<<nb, mtg::kScanThreads, 0, st>>>(c.count, c.ncell, c.block);
        mtg::scan_top_kernel<<<1, mtg::kScanThreads, 0, st>>>(c.block, nb, c.start, c.ncell, d_draw, 0);
        mtg::scan_down_kernel<<<nb, mtg::kScanThreads, 0, st>>>(c.count, c.ncell, c.block, c.start);
        mtg::pair_fill_kernel<<<g, 256, 0, st>>>(c.grid, c.bin, c.start, c.mem);
        check_launch();
        nlaunch += 5;
    }

    // calcg1 (Analysis/PairCorrelation.cpp:9-153) for one replica
    void gr(int replica, double rmax, double dr, int64_t *hist, int cap, int *nbins) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_gr: no state has been set"};
        MTG_REQUIRE(replica >= 0 && replica < nrep, "mtg_gr: replica out of range");
        MTG_REQUIRE(nbins && std::isfinite(rmax) && std::isfinite(dr) && rmax > 0 && dr > 0,
                    "mtg_gr: rmax and dr must be positive and nbins non-null");
        MTG_REQUIRE(rmax <= desc[replica].box, "mtg_gr: rmax must not exceed the box side (calcg1 needs a cell)");
        const double nbd = std::floor(rmax / dr);
        MTG_REQUIRE(nbd <= 1e8, "mtg_gr: more than 1e8 bins");
        const int nb = (int)nbd;
        *nbins = nb;
        if (!hist || nb == 0) return;
        MTG_REQUIRE(cap >= nb, "mtg_gr: hist holds fewer than floor(rmax / dr) bins");
        ReplicaCells c;
        bin_replica(replica, rmax, c);
        unsigned long long *dh = nullptr;
        MTG_CUDA(cudaMalloc(&dh, sizeof(unsigned long long) * nb));
        std::unique_ptr<void, void (*)(void *)> guard(dh, [](void *q) { cudaFree(q); });
        MTG_CUDA(cudaMemsetAsync(dh, 0, sizeof(unsigned long long) * nb, st));
        const int smem_bins = 4096;  // 32 KB of block histogram
        const int g = grid_for(desc[replica].n, 256, 1, sms);
        mtg::pair_hist_kernel<real><<<g, 256, nb <= smem_bins ? sizeof(unsigned long long) * nb : 0, st>>>(
            c.grid, buf[cur], c.start, c.mem, dr, nb, smem_bins, dh);
        check_launch();
        nlaunch += 1;
        std::vector<unsigned long long> h((size_t)nb);
        MTG_CUDA(cudaMemcpyAsync(h.data(), dh, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        for (int b = 0; b < nb; b++) hist[b] = (int64_t)h[(size_t)b];
    }

    // distance_graph (Analysis/AnalyzeGrowth.cpp:136-171) for one replica: smallest local index of each
    // particle's connected component, pairs closer than cut
    void clusters(int replica, double cut, int32_t *labels) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_clusters: no state has been set"};
        MTG_REQUIRE(replica >= 0 && replica < nrep, "mtg_clusters: replica out of range");
        MTG_REQUIRE(labels && std::isfinite(cut) && cut > 0, "mtg_clusters: cut must be positive and labels non-null");
        const int n = desc[replica].n;
        ReplicaCells c;
        bin_replica(replica, cut, c);
        int *parent = nullptr;
        int32_t *dl = nullptr;
        MTG_CUDA(cudaMalloc(&parent, sizeof(int) * (size_t)n));
        std::unique_ptr<void, void (*)(void *)> g1(parent, [](void *q) { cudaFree(q); });
        MTG_CUDA(cudaMalloc(&dl, sizeof(int32_t) * (size_t)n));
        std::unique_ptr<void, void (*)(void *)> g2(dl, [](void *q) { cudaFree(q); });
        const int g = grid_for(n, 256, occ_stream, sms);
        const int limit = wait_limit > 0 ? (int)std::min<int64_t>(wait_limit, (int64_t)n + 1) : n + 1;
        mtg::uf_init_kernel<<<g, 256, 0, st>>>(n, parent);
        mtg::uf_hook_kernel<real><<<g, 256, 0, st>>>(c.grid, buf[cur], c.start, c.mem, parent, d_flags, limit);
        mtg::uf_label_kernel<<<g, 256, 0, st>>>(n, parent, dl, d_flags, limit);
        check_launch();
        nlaunch += 3;
        MTG_CUDA(cudaMemcpyAsync(labels, dl, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        if (flags() & MTG_FLAG_TIMEOUT) throw Fail{MTG_ERR_TIMEOUT, "mtg_clusters: a union-find walk exceeded its bound"};
    }

    void set_wait_limit(int64_t v) override { wait_limit = v; }

    static bool valid_threads(int t) { return t == 128 || t == 256 || t == 512; }
    void get_launch_config(mtg_launch_config *out) const override { *out = lc; }
    void set_launch_config(const mtg_launch_config *c) override {
        MTG_REQUIRE(valid_threads(c->pairfind_threads) && valid_threads(c->epilogue_threads),
                    "mtg_set_launch_config: pairfind_threads and epilogue_threads must be 128, 256 or 512");
        MTG_REQUIRE(c->pairforce_blocks_per_sm >= 1 && c->pairforce_blocks_per_sm <= 64 &&
                        c->patch_blocks_per_sm >= 1 && c->patch_blocks_per_sm <= 64,
                    "mtg_set_launch_config: blocks per SM must lie in [1, 64]");
        MTG_REQUIRE(c->fused_pairs == 0 || c->fused_pairs == 1, "mtg_set_launch_config: fused_pairs must be 0 or 1");
        MTG_CUDA(cudaStreamSynchronize(st));
        lc = *c;
        drop_graphs();   // the step graphs captured the old shapes
    }

    // ms per step of `n` graph-replayed steps (two untimed steps first capture the graphs of both buffer parities)
    double time_steps(int n) {
        step(2, nullptr);
        cudaEvent_t e0, e1;
        MTG_CUDA(cudaEventCreate(&e0));
        MTG_CUDA(cudaEventCreate(&e1));
        MTG_CUDA(cudaEventRecord(e0, st));
        step(n, nullptr);
        MTG_CUDA(cudaEventRecord(e1, st));
        MTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        MTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return (double)ms / n;
    }

    // Coordinate descent over the pipeline's launch shapes, two sweeps, each candidate timed on `trial` steps
    // of the live state (the steps advance the simulation like any others); the fastest shape stays set.
    void autotune(int trial, mtg_launch_config *best, double *best_ms) override {
        if (!have_state) throw Fail{MTG_ERR_STATE, "mtg_autotune: no state has been set"};
        MTG_REQUIRE(trial >= 1, "mtg_autotune: steps_per_trial must be >= 1");
        if (!use_pipe) {   // only the pair pipeline has tunable shapes
            *best = lc;
            *best_ms = time_steps(trial);
            return;
        }
        static const int threads[] = {128, 256, 512};
        static const int onoff[] = {0, 1};
        static const int force_bps[] = {4, 8, 12, 16, 24, 32};
        static const int patch_bps[] = {2, 4, 8, 16, 24};
        mtg_launch_config cur = lc;
        double cur_ms = time_steps(trial);
        using Field = int mtg_launch_config::*;
        auto try_field = [&](Field f, const int *vals, int nv) {
            const int first = cur.*f;
            for (int i = 0; i < nv; i++) {
                if (vals[i] == first) continue;
                mtg_launch_config c = cur;
                c.*f = vals[i];
                set_launch_config(&c);
                const double ms = time_steps(trial);
                if (ms < cur_ms) {
                    cur_ms = ms;
                    cur.*f = vals[i];
                }
            }
            set_launch_config(&cur);
        };
        for (int sweep = 0; sweep < 2; sweep++) {
            try_field(&mtg_launch_config::pairforce_blocks_per_sm, force_bps, 6);
            try_field(&mtg_launch_config::patch_blocks_per_sm, patch_bps, 5);
            try_field(&mtg_launch_config::pairfind_threads, threads, 3);
            try_field(&mtg_launch_config::epilogue_threads, threads, 3);
            try_field(&mtg_launch_config::fused_pairs, onoff, 2);
        }
        set_launch_config(&cur);
        *best = cur;
        *best_ms = time_steps(trial);   // the chosen shape, timed once more
    }
    void set_draw(uint64_t d) override { draw = d; }
    uint64_t get_draw() const override { return draw; }

    uint32_t flags() override {
        MTG_CUDA(cudaMemcpyAsync(h_flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        MTG_CUDA(cudaStreamSynchronize(st));
        return *h_flags;
    }
    void clear_flags() override {
        MTG_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(unsigned), st));
        MTG_CUDA(cudaStreamSynchronize(st));
    }
};


}  // namespace mtg_impl
