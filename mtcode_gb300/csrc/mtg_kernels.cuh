// mtg_kernels.cuh -- sm_103a kernels of one rotational-Langevin step (all replicas in every launch).
//
// Step pipeline (slot order = cell-sorted order of the previous step):
//   [bin]      next position of every particle -> global cell id + rank inside the cell
//              (atomic histogram, warp-aggregated with __match_any_sync).  Fused into the force
//              epilogue of the previous step; launched on its own only after a state upload.
//   [scan]     exclusive scan of the cell histogram (warp-shuffle block scans, 3 phases)
//   [scatter]  half-kick, drift + wrap, free-rotor rotation, written straight to the particle's new
//              slot: the counting sort and the first half of the integrator are one pass
//   [force]    one thread per particle: WCA core + KF2 patch force/torque over the 27 neighbour
//              cells (9 contiguous row ranges of the sorted positions), then friction + Philox noise,
//              the second half-kick, and the binning of the next step
#pragma once

#include <cooperative_groups.h>

#include "mtg_device.cuh"

namespace mtg {
namespace {  // internal linkage: every translation unit keeps its own kernels

// kModeEdges: single-bond mode, the pass that only records this update's bond candidates (edges)
enum ForceMode : int { kModeStep = 0, kModeInit = 1, kModeForces = 2, kModeObs = 3, kModeEdges = 4 };

template <class real>
struct Buffers {
    real *pos, *rota, *rotb;  // 4 reals per slot each: (x, y, z, Q8), (Q0..Q3), (Q4..Q7)
    real *motion;
    int *ident;
    double *dx, *dy, *dz;  // unwrapped displacement (nullable)
    int *slot_of;          // global index -> slot of the buffer in use (shared by both buffers; nullable,
                           // kept only when bonds are set)
    real *xref;            // skin lists: position of each slot at the last list build (4 reals), shared
    int *home_cell;        // skin lists: cell of each slot at the last list build, shared
    real *snap_a, *snap_b, *snap_c;  // single-bond mode: position and rotation at the last candidate-list
                                     // build, laid out like pos / rota / rotb but indexed by the particle's
                                     // global index (ident), so a re-sort leaves it in place; one set shared
                                     // by both buffers
};

// Skin-list state (int[4], device): [0] this step rebuilds, [1] a particle will have moved more than half
// the skin by the next step, [2] rebuild requested by the host, [3] rebuilds so far
constexpr int kListCap = 32;  // candidates kept per particle; a longer list marks the particle overflowed

// a kernel on a skin-list step runs when the step's rebuild flag equals `want` (always without a gate)
__device__ __forceinline__ bool gated_off(const int *gate, int want) { return gate && *gate != want; }

template <class real>
struct Tables {
    const Replica<real> *reps;
    const int *rep_slot;   // n_rep + 1 slot offsets (== particle offsets)
    const Model<real> *models;
    int nrep;
    int ntot;
    int ncells;
    int uniform;   // every replica has the pair constants of replica 0 and one particle type: pair kernels
                   // read replica 0 instead of searching the slot's replica
    const unsigned short *slot_rep;   // replica of every slot (slot ranges are fixed), or null: binary search
};

// the device's noise-draw counter (draw used by the next pass, next draw), set from the host by value: a
// kernel parameter, so the call neither waits for the stream nor needs a host buffer that outlives it
__global__ void draw_set_kernel(unsigned long long *draw, unsigned long long now, unsigned long long next) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        draw[0] = now;
        draw[1] = next;
    }
}

__device__ __forceinline__ int find_replica(const int *rep_slot, int nrep, int s) {
    int lo = 0, hi = nrep;  // rep_slot[lo] <= s < rep_slot[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (__ldg(rep_slot + mid) <= s) lo = mid;
        else hi = mid;
    }
    return lo;
}

// the replica of slot s: one 2-byte load where the per-slot table exists (fewer than 65,536 replicas)
template <class real>
__device__ __forceinline__ int replica_of(const Tables<real> &tb, int s) {
    return tb.slot_rep ? (int)__ldg(tb.slot_rep + s) : find_replica(tb.rep_slot, tb.nrep, s);
}

// cell id of a position inside replica R (cube::assign_box with cells of the force grid)
template <class real>
__device__ __forceinline__ int cell_of(const Replica<real> &R, real x, real y, real z) {
    int cx = axis_cell<real>(x, R.cell_scale, R.nc);
    int cy = axis_cell<real>(y, R.cell_scale, R.nc);
    int cz = axis_cell<real>(z, R.cell_scale, R.nc);
    return R.cell_off + cx + R.nc * (cy + R.nc * cz);
}

// next position: p_h = p + (dt/2) F~ ; x' = x + (dt/m) p_h ; wrap (advancemom_halfstep, advance_pos)
template <class real>
__device__ __forceinline__ void drift_position(const Replica<real> &R, real x[3], real p[3], const real F[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        p[k] = add_rn(p[k], mul_rn(R.half_dt, F[k]));
        x[k] = add_rn(x[k], mul_rn(R.c1, p[k]));
        wrap_coord<real>(x[k], p[k], R.box, R.periodic);
    }
}

// warp-aggregated atomic increment of count[key]; returns this lane's rank
__device__ __forceinline__ int aggregated_rank(int *count, int key) {
    unsigned active = __activemask();
    unsigned peers = __match_any_sync(active, key);
    int leader = __ffs(peers) - 1;
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader) base = atomicAdd(count + key, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

// ------------------------------------------------------------------ bin (standalone)
template <class real, bool MOVE>
__global__ void __launch_bounds__(256) bin_kernel(Tables<real> tb, Buffers<real> in, int2 *bin, int *count,
                                                  unsigned *flags, const int *gate = nullptr) {
    if (gated_off(gate, 1)) return;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < tb.ntot; s += gridDim.x * blockDim.x) {
        const int r = replica_of(tb, s);
        const Replica<real> R = tb.reps[r];
        real x[3];
        load_pos(in.pos + 4 * (size_t)s, x[0], x[1], x[2]);
        if (MOVE) {
            Row<real> m;
            m.load(in.motion + (size_t)s * kRow);
            real p[3] = {m.v[0], m.v[1], m.v[2]}, F[3] = {m.v[6], m.v[7], m.v[8]};
            drift_position<real>(R, x, p, F);
        }
        if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) {
            atomicOr(flags, 1u);
            x[0] = x[1] = x[2] = real(0);
        }
        int key = cell_of<real>(R, x[0], x[1], x[2]);
        int rank = aggregated_rank(count, key);
        bin[s] = make_int2(key, rank);
    }
}

// ------------------------------------------------------------------ scan of the cell histogram
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;  // per thread -> 4096 cells per block
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_sums, int &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
        int winc = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, winc, o);
            if (lane >= o) winc += t;
        }
        warp_sums[lane] = winc - w;
        if (lane == 31) warp_sums[32] = winc;
    }
    __syncthreads();
    int excl = inc - v + warp_sums[warp];
    total = warp_sums[32];
    __syncthreads();
    return excl;
}

// A thread's kScanItems cells start at a multiple of 32 bytes of a cudaMalloc'd array: whole groups move as
// two 16-byte words, the ragged end of the array element by element.
static_assert(kScanItems == 8, "the scans move a thread's cells as two int4");
__device__ __forceinline__ void scan_load8(const int *p, int base, int n, int v[8]) {
    if (base + 8 <= n) {
        const int4 x = *reinterpret_cast<const int4 *>(p + base), y = *reinterpret_cast<const int4 *>(p + base + 4);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
        v[4] = y.x; v[5] = y.y; v[6] = y.z; v[7] = y.w;
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = base + k < n ? p[base + k] : 0;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const int *count, int n, int *block_sums,
                                                                   const int *gate = nullptr) {
    if (gated_off(gate, 1)) return;
    __shared__ int ws[33];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    scan_load8(count, base, n, v);
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) s += v[k];
    int total;
    block_exclusive_scan(s, ws, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// single block: exclusive scan of the block sums; also advances the noise draw counter
__global__ void __launch_bounds__(kScanThreads) scan_top_kernel(int *block_sums, int nblocks, int *start, int n,
                                                                unsigned long long *draw, int consume_draw,
                                                                const int *gate = nullptr) {
    if (gated_off(gate, 1)) return;
    __shared__ int ws[33];
    int carry = 0;
    for (int b0 = 0; b0 < nblocks; b0 += kScanThreads) {
        int i = b0 + threadIdx.x;
        int v = i < nblocks ? block_sums[i] : 0;
        int total;
        int e = block_exclusive_scan(v, ws, total);
        if (i < nblocks) block_sums[i] = e + carry;
        carry += total;
    }
    if (threadIdx.x == 0) {
        start[n] = carry;
        if (consume_draw) {
            draw[0] = draw[1];  // draw used by this step
            draw[1] = draw[1] + 1ull;
        }
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_down_kernel(int *count, int n, const int *block_sums,
                                                                 int *start, const int *gate = nullptr) {
    if (gated_off(gate, 1)) return;
    __shared__ int ws[33];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    scan_load8(count, base, n, v);
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) s += v[k];
    int total;
    int e = block_exclusive_scan(s, ws, total) + block_sums[blockIdx.x];
    int o[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        o[k] = e;
        e += v[k];
    }
    if (base + 8 <= n) {  // the counts are cleared for the next histogram
        *reinterpret_cast<int4 *>(start + base) = make_int4(o[0], o[1], o[2], o[3]);
        *reinterpret_cast<int4 *>(start + base + 4) = make_int4(o[4], o[5], o[6], o[7]);
        *reinterpret_cast<int4 *>(count + base) = make_int4(0, 0, 0, 0);
        *reinterpret_cast<int4 *>(count + base + 4) = make_int4(0, 0, 0, 0);
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            if (base + k < n) {
                start[base + k] = o[k];
                count[base + k] = 0;
            }
        }
    }
}

// ------------------------------------------------------------------ scatter (+ first half of the step)

// LangevinNVTR::genfullmat (LangevinR.cpp:392-461) built as the product of its five Cayley
// rotations: x(dt/2) y(dt/2) z(dt) y(dt/2) x(dt/2) of the free rotor, omega = L/I.
template <class real>
__device__ __forceinline__ void free_rotor(real dt, real inertia, const real L[3], real R[9]) {
    real tx = dt * L[0] / inertia, ty = dt * L[1] / inertia, tz = dt * L[2] / inertia;
    real hx = tx * real(0.25), hy = ty * real(0.25), hz = tz * real(0.5);
    real dx_ = real(1) / (real(1) + hx * hx), dy_ = real(1) / (real(1) + hy * hy), dz_ = real(1) / (real(1) + hz * hz);
    // sines enter with a minus sign: the rotations turn L forward by +omega dt
    real cx = (real(1) - hx * hx) * dx_, sx = real(-2) * hx * dx_;
    real cy = (real(1) - hy * hy) * dy_, sy = real(-2) * hy * dy_;
    real cz = (real(1) - hz * hz) * dz_, sz = real(-2) * hz * dz_;
    // M = Ax * Ay * Az * Ay * Ax with Ax = [[1,0,0],[0,c,s],[0,-s,c]], Ay = [[c,0,-s],[0,1,0],[s,0,c]],
    // Az = [[c,s,0],[-s,c,0],[0,0,1]] (s as above); checked against genfullmat's closed form
    real M[9] = {1, 0, 0, 0, cx, sx, 0, -sx, cx};
    auto mul_y = [&](real c, real s) {
        for (int r = 0; r < 3; r++) {
            real a = M[3 * r], b = M[3 * r + 2];
            M[3 * r] = a * c + b * s;
            M[3 * r + 2] = -a * s + b * c;
        }
    };
    auto mul_z = [&](real c, real s) {
        for (int r = 0; r < 3; r++) {
            real a = M[3 * r], b = M[3 * r + 1];
            M[3 * r] = a * c - b * s;
            M[3 * r + 1] = a * s + b * c;
        }
    };
    auto mul_x = [&](real c, real s) {
        for (int r = 0; r < 3; r++) {
            real a = M[3 * r + 1], b = M[3 * r + 2];
            M[3 * r + 1] = a * c - b * s;
            M[3 * r + 2] = a * s + b * c;
        }
    };
    mul_y(cy, sy);
    mul_z(cz, sz);
    mul_y(cy, sy);
    mul_x(cx, sx);
#pragma unroll
    for (int k = 0; k < 9; k++) R[k] = M[k];
}

// First half of the step for one particle (advancemom_halfstep, advance_pos, rotate: LangevinR.cpp:327-347,
// Langevin.cpp:205-222, LangevinR.cpp:594-695): half-kick with the carried F~/T~, drift + wrap/reflect,
// free-rotor rotation.  step receives the unwrapped drift (c1 * p_half) for the displacement sums.
template <class real>
__device__ __forceinline__ void advance_particle(const Replica<real> &R, Payload<real> &P, Row<real> &M, real step[3],
                                                 unsigned *flags) {
    real x[3] = {P.v[0], P.v[1], P.v[2]}, p[3] = {M.v[0], M.v[1], M.v[2]};
    real F[3] = {M.v[6], M.v[7], M.v[8]};
    real L[3] = {M.v[3], M.v[4], M.v[5]}, T[3] = {M.v[9], M.v[10], M.v[11]};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        real ph = add_rn(p[k], mul_rn(R.half_dt, F[k]));
        step[k] = mul_rn(R.c1, ph);
    }
    drift_position<real>(R, x, p, F);  // identical arithmetic to the binning pass
    if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) atomicOr(flags, 1u);
#pragma unroll
    for (int k = 0; k < 3; k++) L[k] = L[k] + R.half_dt * T[k];
    real Rm[9];
    free_rotor<real>(R.dt, R.inertia, L, Rm);
    real Ln[3];
#pragma unroll
    for (int a = 0; a < 3; a++) Ln[a] = L[0] * Rm[3 * a] + L[1] * Rm[3 * a + 1] + L[2] * Rm[3 * a + 2];
    // Q <- R^T Q (LangevinR.cpp:611-683)
    real Q[9] = {P.v[3], P.v[4], P.v[5], P.v[6], P.v[7], P.v[8], P.v[9], P.v[10], P.v[11]};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
            P.v[3 + 3 * a + b] = Q[b] * Rm[a] + Q[3 + b] * Rm[3 + a] + Q[6 + b] * Rm[6 + a];
    P.v[0] = x[0]; P.v[1] = x[1]; P.v[2] = x[2];
    M.v[0] = p[0]; M.v[1] = p[1]; M.v[2] = p[2];
    M.v[3] = Ln[0]; M.v[4] = Ln[1]; M.v[5] = Ln[2];
}

template <class real, bool MOVE>
__global__ void __launch_bounds__(256) scatter_kernel(Tables<real> tb, Buffers<real> in, Buffers<real> out,
                                                      const int2 *bin, const int *start, unsigned *flags,
                                                      const int *gate = nullptr,
                                                      const unsigned long long *snap_due = nullptr) {
    if (gated_off(gate, 1)) return;
    // every particle must have been binned exactly once; otherwise nothing is moved (latched error)
    if (__ldg(start + tb.ncells) != tb.ntot) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(flags, 16u);
        return;
    }
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < tb.ntot; s += gridDim.x * blockDim.x) {
        const int2 kb = bin[s];
        const int d = __ldg(start + kb.x) + kb.y;
        if (kb.x < 0 || kb.x >= tb.ncells || d < 0 || d >= tb.ntot) {
            atomicOr(flags, 16u);
            continue;
        }
        Payload<real> P;
        Row<real> M;
        P.load(in.pos, in.rota, in.rotb, s);
        M.load(in.motion + (size_t)s * kRow);
        const int id = in.ident[s];
        if (out.snap_a) {
            // single-bond mode: the candidate list is built from the positions at the start of the step
            // (calculate_patch_list before advancemom_halfstep, Condensate.cpp:464-475); otherwise the
            // particle carries its snapshot along
            if (snap_due && *snap_due) P.store(out.snap_a, out.snap_b, out.snap_c, id);
        }
        if (MOVE) {
            const int r = replica_of(tb, s);
            const Replica<real> R = tb.reps[r];
            real step[3];
            advance_particle<real>(R, P, M, step, flags);
            if (in.dx) {
                out.dx[d] = in.dx[s] + (double)step[0];
                out.dy[d] = in.dy[s] + (double)step[1];
                out.dz[d] = in.dz[s] + (double)step[2];
            }
        } else if (in.dx) {
            out.dx[d] = in.dx[s];
            out.dy[d] = in.dy[s];
            out.dz[d] = in.dz[s];
        }
        P.store(out.pos, out.rota, out.rotb, d);
        M.store(out.motion + (size_t)d * kRow);
        out.ident[d] = id;
        if (out.slot_of) out.slot_of[id] = d;
        if (out.xref) {
            out.xref[4 * (size_t)d] = P.v[0];
            out.xref[4 * (size_t)d + 1] = P.v[1];
            out.xref[4 * (size_t)d + 2] = P.v[2];
        }
        if (out.home_cell) out.home_cell[d] = kb.x;
    }
}

// ------------------------------------------------------------------ skin-list steps

// decides whether this step rebuilds the lists, and takes the step's noise draw (draw[0] <- draw[1]++)
__global__ void skin_decide_kernel(int *skin, unsigned long long *draw) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const int rebuild = (skin[1] | skin[2]) ? 1 : 0;
        skin[0] = rebuild;
        skin[1] = 0;
        skin[2] = 0;
        skin[3] += rebuild;
        draw[0] = draw[1];
        draw[1] = draw[1] + 1ull;
    }
}

__global__ void skin_set_kernel(int *skin, int now, int next, int forced) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (now >= 0) skin[0] = now;
        if (next >= 0) skin[1] = next;
        if (forced >= 0) skin[2] = forced;
    }
}

// the first half of the step in place (no re-sort) on steps that keep their lists
template <class real>
__global__ void __launch_bounds__(256) integrate_kernel(Tables<real> tb, Buffers<real> b, unsigned *flags,
                                                        const int *gate) {
    if (gated_off(gate, 0)) return;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < tb.ntot; s += gridDim.x * blockDim.x) {
        Payload<real> P;
        Row<real> M;
        P.load(b.pos, b.rota, b.rotb, s);
        M.load(b.motion + (size_t)s * kRow);
        const int r = replica_of(tb, s);
        const Replica<real> R = tb.reps[r];
        real step[3];
        advance_particle<real>(R, P, M, step, flags);
        if (b.dx) {
            b.dx[s] += (double)step[0];
            b.dy[s] += (double)step[1];
            b.dz[s] += (double)step[2];
        }
        P.store(b.pos, b.rota, b.rotb, s);
        M.store(b.motion + (size_t)s * kRow);
    }
}

// after a rebuild's scatter into the spare buffer, the sorted state goes back to the buffer in use
template <class real>
__global__ void __launch_bounds__(256) copy_back_kernel(int ntot, Buffers<real> from, Buffers<real> to,
                                                        const int *gate) {
    if (gated_off(gate, 1)) return;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ntot; s += gridDim.x * blockDim.x) {
        Payload<real> P;
        Row<real> M;
        P.load(from.pos, from.rota, from.rotb, s);
        M.load(from.motion + (size_t)s * kRow);
        P.store(to.pos, to.rota, to.rotb, s);
        M.store(to.motion + (size_t)s * kRow);
        to.ident[s] = from.ident[s];
        if (from.dx) {
            to.dx[s] = from.dx[s];
            to.dy[s] = from.dy[s];
            to.dz[s] = from.dz[s];
        }
    }
}

// ------------------------------------------------------------------ force + Langevin epilogue

// ------------------------------------------------------------------ patch numbering
template <class real>
__device__ __forceinline__ int patch_of(const BindRep &B, const Model<real> &M, int li, int t, int c) {
    return B.patch_off + B.pbase[t] + (li - (t ? M.ncum[t - 1] : 0)) * M.np[t] + c;
}

// replica of global patch wp (binary search over the replicas' first patches)
__device__ __forceinline__ int patch_replica(const BindRep *reps, int nrep, int wp) {
    int lo = 0, hi = nrep;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (reps[mid].patch_off <= wp) lo = mid;
        else hi = mid;
    }
    return lo;
}

// GeneralPatch::which_particle: local particle, type and patch number of local patch lp
template <class real>
__device__ __forceinline__ void patch_owner(const BindRep &B, const Model<real> &M, int lp, int &li, int &t, int &c) {
    t = 0;
#pragma unroll
    for (int k = 1; k < kMaxTypes; k++)
        if (k < M.n_types && lp >= B.pbase[k]) t = k;
    const int rel = lp - B.pbase[t], np = M.np[t] > 0 ? M.np[t] : 1;
    li = (t ? M.ncum[t - 1] : 0) + rel / np;
    c = rel % np;
}


template <class real>
struct ForceArgs {
    Tables<real> tb;
    Buffers<real> buf;      // current (cell-sorted) buffers; motion is updated in place
    const int *start;       // cell starts of the current order
    int2 *bin;              // next-step bins (modes step / init)
    int *count;             // next-step histogram (modes step / init)
    unsigned *flags;
    const unsigned long long *draw;  // draw[0] = draw index of this pass
    const double *ext_noise;         // ntot x 6 by global index, or null (Philox)
    double *outF, *outT, *outE;      // mode forces: by global index
    double *obs;                     // mode obs: n_rep x 5
    int do_kick;                     // second half-kick (step) or not (init)
    int parts;                       // terms summed: bit 0 central (WCA core + harmonic bonds), bit 1 patch
                                     // (Kern-Frenkel force + torque, bound-pair forces); 3 for every pass
                                     // but the per-phase force calls
    // fixed bonds, by global index (CSR: partners of i are bond_partner[bond_start[i] .. bond_start[i+1]));
    // null when the system has none.  HarmonicPotential(bond_k, bond_r0).
    const int *bond_start, *bond_partner;
    real bond_k, bond_r0;
    // skin lists (null without): rebuild flag of this step, the next step's flag, candidate lists
    // (list[t * ntot + slot], kListCap per slot) and their lengths by slot
    const int *skin;
    int *skin_next;
    unsigned *list;
    int *list_n;
    // single-bond-per-patch mode (null otherwise): patch numbering per replica, bond state by global patch;
    // on a pass that decides bonds also this update's adjacency (stamped counters, kAdjCap partners per
    // patch) and the update counters (stamp = bind_ctr[2])
    const BindRep *bind_reps;
    const unsigned char *bind_on;
    const int *bind_to;
    unsigned long long *bind_deg;
    int2 *bind_adj;
    unsigned long long *bind_ctr;    // [2] stamp; segment counters of the update's lists (kSegTouched, ...)
    int *bind_touched;               // patches with an edge this update, kSegs segments of bind_tcap
    long long bind_tcap;
    int2 *bind_recheck;              // patch pairs for the FP64 tests (float edge pass), kSegs segments of bind_rcap
    long long bind_rcap;
    int bind_listed;                 // bound-pair forces summed by a pair kernel, not by the epilogue
};

// ------------------------------------------------------------------ single-bond mode: bond candidates
// The edges of LangevinNVTR::calculate_forces_and_torques3D_onlyone_nonlets (LangevinRforce.cpp:2900-3090):
// a patch pair (p1 < p2) is an edge when it is on the candidate list of the last list build
// (calculate_patch_list, LangevinR.cpp:1702-1852) and now |x1 - x2|^2 < max_check^2, both cones hold
// (c_i, c_j > cos thetam) and |x1 - x2| < disp2, the bind-state dependent range.  The list itself is not
// stored: every particle carries its position and rotation of the list build (the snapshot), and a patch
// pair that passes the current test is checked against the list's condition on the snapshot.  Every test is
// the reference's FP64 expression in its operation order; float evaluations decide only outside a margin.
constexpr int kAdjCap = 8;            // candidate partners of one patch in one update
constexpr unsigned kFlagBind = 0x20u; // a capacity of this mode was exceeded (MTG_FLAG_BIND), with one of:
constexpr unsigned kBindWhyAdj = 1u << 16;      // a patch had more than kAdjCap candidate partners
constexpr unsigned kBindWhyCluster = 1u << 17;  // a patch cluster exceeded the large-cluster capacity
constexpr unsigned kBindWhyList = 1u << 18;     // a segment of a pass's list was full
constexpr unsigned kBindWhyRef = 1u << 19;      // a cluster reached one of the reference's error() paths
constexpr unsigned kBindWhySpin = 1u << 20;     // an atomic retry loop reached its bound

// cube::distance_vector (geometry.h:277-294): un = x_a - x_b (minimum image), returns |un|^2
__device__ __forceinline__ double exact_dist_vec(const BindRep &B, const double xa[3], const double xb[3], double un[3]) {
    double temp = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double as = __dsub_rn(xa[k], xb[k]);
        if (B.periodic && __dmul_rn(as, as) > B.l2s) as = as >= 0.0 ? __dsub_rn(as, B.box) : __dadd_rn(as, B.box);
        temp = __dadd_rn(temp, __dmul_rn(as, as));
        un[k] = as;
    }
    return temp;
}

// Q^T n_b (LangevinRforce.cpp:2980-2985) then -(n . u) or (n . u)
__device__ __forceinline__ double exact_cos(const double nb[3], const double q[9], const double u[3], bool negate) {
    double n[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        n[k] = __dadd_rn(__dadd_rn(__dmul_rn(nb[0], q[k]), __dmul_rn(nb[1], q[3 + k])), __dmul_rn(nb[2], q[6 + k]));
    const double d = __dadd_rn(__dadd_rn(__dmul_rn(n[0], u[0]), __dmul_rn(n[1], u[1])), __dmul_rn(n[2], u[2]));
    return negate ? -d : d;
}

// position and rotation of slot s of a (pos, rota, rotb)-shaped triple as doubles (exact conversions)
template <class real>
__device__ __forceinline__ void load_state_d(const real *pa, const real *pb, const real *pc, int s, double x[3],
                                             double q[9]) {
    Payload<real> P;
    P.load(pa, pb, pc, s);
#pragma unroll
    for (int k = 0; k < 3; k++) x[k] = (double)P.v[k];
#pragma unroll
    for (int k = 0; k < 9; k++) q[k] = (double)P.v[3 + k];
}

// value against a bracketed threshold: +1 certainly above, -1 certainly below, 0 inside the margin
template <class T>
__device__ __forceinline__ int side_of(T v, float lo, float hi) {
    return v > (T)hi ? 1 : (v < (T)lo ? -1 : 0);
}

// the reference's bind-state dependent range (LangevinRforce.cpp:3010-3030): class 0 disp (neither or both
// bound to each other), 1 0.5 disp (both bound elsewhere), 2 0.7 disp (exactly one bound)
__device__ __forceinline__ int range_class(bool b1, bool b2, int boundto1, int boundto2, int w1, int w2) {
    const bool cond1 = boundto1 == w2 && boundto2 == w1;
    return (b1 && b2) ? (cond1 ? 0 : 1) : (b1 != b2 ? 2 : 0);
}
__device__ __forceinline__ double disp2_of(double disp, int cls) {
    return cls == 1 ? __dmul_rn(0.5, disp) : (cls == 2 ? __dmul_rn(0.7, disp) : disp);
}

// FP64 edge test of the current state; with score != null also the edge's score (LangevinRforce.cpp:3040-3060)
template <class real>
__device__ __noinline__ bool exact_edge(const BindRep &B, const real *pos, const real *rota, const real *rotb, int s1,
                                        int s2, int o1, int o2, int potn, double disp2, double *score) {
    double xa[3], qa[9], xb[3], qb[9], un[3];
    load_state_d<real>(pos, rota, rotb, s1, xa, qa);
    load_state_d<real>(pos, rota, rotb, s2, xb, qb);
    double dis = exact_dist_vec(B, xa, xb, un);
    if (!(dis < B.mk2)) return false;
    dis = __dsqrt_rn(dis);
    un[0] = __ddiv_rn(un[0], dis); un[1] = __ddiv_rn(un[1], dis); un[2] = __ddiv_rn(un[2], dis);
    const double ai = exact_cos(B.orient[o1], qa, un, true), aj = exact_cos(B.orient[o2], qb, un, false);
    const double ctm = B.ctm[potn];
    if (!(ai > ctm && aj > ctm && dis < disp2)) return false;
    if (score) {
        const double scr1 = __dsub_rn(1.0, __dsub_rn(ai, ctm));
        const double scr2 = __dsub_rn(1.0, __dsub_rn(aj, ctm));
        const double scr3 = __dmul_rn(2.0, __ddiv_rn(dis, disp2));
        *score = __dadd_rn(__dadd_rn(scr1, scr2), scr3);
    }
    return true;
}

// FP64 candidate-list condition on the snapshot (s1, s2: the particles' global indices): distance < the list
// cut and < max_check + 1, and (c_i - max_ang) + (c_j - max_ang) > -0.4 (LangevinR.cpp:1722-1800)
template <class real>
__device__ __noinline__ bool exact_member(const BindRep &B, const real *sa, const real *sb, const real *sc, int s1,
                                          int s2, int o1, int o2) {
    double xa[3], qa[9], xb[3], qb[9], un[3];
    load_state_d<real>(sa, sb, sc, s1, xa, qa);
    load_state_d<real>(sa, sb, sc, s2, xb, qb);
    const double d2 = exact_dist_vec(B, xa, xb, un);
    if (!(d2 < B.list_cut2)) return false;
    const double dis = __dsqrt_rn(d2);
    if (!(dis < B.max_dis)) return false;
    un[0] = __ddiv_rn(un[0], dis); un[1] = __ddiv_rn(un[1], dis); un[2] = __ddiv_rn(un[2], dis);
    const double ai = exact_cos(B.orient[o1], qa, un, true), aj = exact_cos(B.orient[o2], qb, un, false);
    return __dadd_rn(__dsub_rn(ai, B.max_ang), __dsub_rn(aj, B.max_ang)) > -0.4;
}

// the candidate-list condition in float on snapshot rows A and C (the particles of patch rows o1, o2): 1 member,
// -1 not, 0 within a margin of a threshold (the FP64 test, exact_member, decides)
template <class real>
__device__ __forceinline__ int candidate_side(const BindRep &B, const Replica<real> &R, const Model<real> &M,
                                              const Payload<real> &A, const Payload<real> &C, int o1, int o2) {
    const real dx = min_image_sep<real>(A.v[0], C.v[0], R.box, R.box_lo, R.l2s, R.periodic);
    const real dy = min_image_sep<real>(A.v[1], C.v[1], R.box, R.box_lo, R.l2s, R.periodic);
    const real dz = min_image_sep<real>(A.v[2], C.v[2], R.box, R.box_lo, R.l2s, R.periodic);
    const real r2 = dx * dx + dy * dy + dz * dz;
    const int t = side_of<real>(r2, B.memb2_lo, B.memb2_hi);
    if (t != -1) return t > 0 ? -1 : 0;
    const real rr = sqrt(r2), u[3] = {dx / rr, dy / rr, dz / rr};
    const real *v1 = M.orient[o1], *v2 = M.orient[o2];
    real ci = 0, cj = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        ci -= (v1[0] * A.v[3 + k] + v1[1] * A.v[6 + k] + v1[2] * A.v[9 + k]) * u[k];
        cj += (v2[0] * C.v[3 + k] + v2[1] * C.v[6 + k] + v2[2] * C.v[9 + k]) * u[k];
    }
    return side_of<real>((ci - (real)B.max_ang_f) + (cj - (real)B.max_ang_f), B.ang_lo, B.ang_hi);
}

template <class real>
__device__ __forceinline__ bool candidate(const BindRep &B, const Replica<real> &R, const Model<real> &M,
                                          const real *sa, const real *sb, const real *sc, int s1, int s2, int o1,
                                          int o2) {
    if (std::is_same<real, double>::value) return exact_member<real>(B, sa, sb, sc, s1, s2, o1, o2);
    Payload<real> A, C;
    A.load(sa, sb, sc, s1);
    C.load(sa, sb, sc, s2);
    const int w = candidate_side<real>(B, R, M, A, C, o1, o2);
    return w == 0 ? exact_member<real>(B, sa, sb, sc, s1, s2, o1, o2) : w > 0;
}

// slot of this update's adjacency for patch p (stamped counter: a stale stamp counts as zero edges).  A max of
// (stamp << 32) followed by an add would take the slot without the load, but the two atomics on one address
// measured far slower than the load and the compare-and-swap.
__device__ __forceinline__ int adj_take(unsigned long long *deg, int p, unsigned stamp, unsigned *flags) {
    unsigned long long old = deg[p];
    for (int it = 0; it < (1 << 20); it++) {
        const unsigned cnt = (unsigned)(old >> 32) == stamp ? (unsigned)old : 0u;
        const unsigned long long nw = ((unsigned long long)stamp << 32) | (unsigned long long)(cnt + 1u);
        const unsigned long long prev = atomicCAS(deg + p, old, nw);
        if (prev == old) return (int)cnt;
        old = prev;
    }
    atomicOr(flags, kFlagBind | kBindWhySpin);
    return kAdjCap;
}

// Lists built during a pass (pairs for the edge pass, touched patches, bound pairs) are split into kSegs
// segments, each with its own counter, chosen by warp: appends from different warps rarely meet on one
// address.  Segment k holds entries [k * cap, k * cap + count[k]).
constexpr int kSegs = 64;
constexpr int kSegPairs = 8;                   // bind_ctr offsets of the segment counters
constexpr int kSegTouched = kSegPairs + kSegs;
constexpr int kSegBound = kSegTouched + kSegs;
constexpr int kSegRecheck = kSegBound + kSegs;
constexpr int kBindCounters = kSegRecheck + kSegs;

// A kernel that reads a segmented list first lays its segments end to end: seg_prefix (every thread of the
// block, before any early exit) leaves the exclusive prefix of the segment lengths in shared memory, and
// seg_slot maps an index below sh[kSegs] to its entry.
__device__ __forceinline__ void seg_prefix(const unsigned long long *counts, long long cap, long long *sh) {
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int k = 0; k < kSegs; k++) {
            sh[k] = t;
            const long long c = (long long)counts[k];
            t += c < cap ? c : cap;
        }
        sh[kSegs] = t;
    }
    __syncthreads();
}
__device__ __forceinline__ size_t seg_slot(const long long *sh, long long cap, long long i) {
    int lo = 0, hi = kSegs;   // sh[lo] <= i < sh[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (sh[mid] <= i) lo = mid;
        else hi = mid;
    }
    return (size_t)lo * (size_t)cap + (size_t)(i - sh[lo]);
}

template <class T>
__device__ __forceinline__ void seg_append(T *list, unsigned long long *counts, long long cap, const T &e,
                                           unsigned *flags, unsigned full_flag = kFlagBind | kBindWhyList) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    const int k = (int)((blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) & (kSegs - 1));
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counts + k, (unsigned long long)g.size());
    base = g.shfl(base, 0) + g.thread_rank();
    if ((long long)base < cap) list[(size_t)k * (size_t)cap + base] = e;
    else atomicOr(flags, full_flag);
}

template <class real>
__device__ __forceinline__ void add_edge_t(const ForceArgs<real> &a, int w1, int w2, int cls, unsigned stamp) {
    const int k1 = adj_take(a.bind_deg, w1, stamp, a.flags), k2 = adj_take(a.bind_deg, w2, stamp, a.flags);
    if (k1 < kAdjCap) a.bind_adj[(size_t)w1 * kAdjCap + k1] = make_int2(w2, cls);
    else atomicOr(a.flags, kFlagBind | kBindWhyAdj);
    if (k2 < kAdjCap) a.bind_adj[(size_t)w2 * kAdjCap + k2] = make_int2(w1, cls);
    else atomicOr(a.flags, kFlagBind | kBindWhyAdj);
    if (k1 == 0) seg_append<int>(a.bind_touched, a.bind_ctr + kSegTouched, a.bind_tcap, w1, a.flags);
    if (k2 == 0) seg_append<int>(a.bind_touched, a.bind_ctr + kSegTouched, a.bind_tcap, w2, a.flags);
}

// One patch pair (patch ka of particle s1, kb of s2; s1 the lower particle index) with cosines c1, c2 and
// distance rr from the caller's float geometry (t0: the max_check test's side): the edge test, the
// candidate-list condition, and the edge into both patches' adjacency.
template <class real>
__device__ __forceinline__ void bind_patch_edge(const ForceArgs<real> &a, const BindRep &B, const Replica<real> &R,
                                                const Model<real> &M, int s1, int s2, int li1, int li2, int ty1,
                                                int ty2, int ka, int kb, real c1, real c2, real rr, int t0,
                                                unsigned stamp) {
    const int q = M.pstart[ty1][ty2] + ka * M.np[ty2] + kb;
    const int e1 = side_of<real>(c1, B.ctm_lo[q], B.ctm_hi[q]), e2 = side_of<real>(c2, B.ctm_lo[q], B.ctm_hi[q]);
    if (e1 < 0 || e2 < 0) return;
    const int wp1 = patch_of<real>(B, M, li1, ty1, ka), wp2 = patch_of<real>(B, M, li2, ty2, kb);
    const int cls = range_class(a.bind_on[wp1] != 0, a.bind_on[wp2] != 0, a.bind_to[wp1], a.bind_to[wp2], wp1, wp2);
    const float dfl = cls == 1 ? 0.5f * B.disp_f[q] : (cls == 2 ? 0.7f * B.disp_f[q] : B.disp_f[q]);
    const int e3 = side_of<real>(rr, dfl * (1.f - 1e-5f), dfl * (1.f + 1e-5f));
    if (e3 > 0) return;
    const int o1 = M.ooff[ty1] + ka, o2 = M.ooff[ty2] + kb;
    const bool sure = !std::is_same<real, double>::value && t0 < 0 && e1 > 0 && e2 > 0 && e3 < 0;
    if (!sure && !exact_edge<real>(B, a.buf.pos, a.buf.rota, a.buf.rotb, s1, s2, o1, o2, q, disp2_of(B.disp[q], cls),
                                   nullptr))
        return;
    if (!candidate<real>(B, R, M, a.buf.snap_a, a.buf.snap_b, a.buf.snap_c, li1 + R.off, li2 + R.off, o1, o2))
        return;
    add_edge_t<real>(a, wp1, wp2, cls, stamp);
}

// bind_patch_edge in float only, for the listed edge pass (bind_pairs_kernel): the same decision where every
// float test is clear of its margin; a patch pair with a float test within a margin goes to the recheck list
// (wp1 of particle s1, wp2 of s2) for bind_recheck_kernel, which repeats it with the FP64 tests.  With no FP64
// code and no call the pass keeps its values in registers.  Both patches' bond states and both snapshot rows
// are read before any of them is used, so a patch pair waits on memory once for all of them (reading the
// adjacency counters there too, for compare-and-swaps issued together, measured a little slower).
__device__ __forceinline__ void bind_patch_edge_f(const ForceArgs<float> &a, const BindRep &B, const Replica<float> &R,
                                                  const Model<float> &M, int li1, int li2, int ty1, int ty2, int ka,
                                                  int kb, float c1, float c2, float rr, int t0, unsigned stamp) {
    const int q = M.pstart[ty1][ty2] + ka * M.np[ty2] + kb;
    const int e1 = side_of<float>(c1, B.ctm_lo[q], B.ctm_hi[q]), e2 = side_of<float>(c2, B.ctm_lo[q], B.ctm_hi[q]);
    if (e1 < 0 || e2 < 0) return;
    const int wp1 = patch_of<float>(B, M, li1, ty1, ka), wp2 = patch_of<float>(B, M, li2, ty2, kb);
    const bool b1 = a.bind_on[wp1] != 0, b2 = a.bind_on[wp2] != 0;
    const int bt1 = a.bind_to[wp1], bt2 = a.bind_to[wp2];
    Payload<float> A, C;
    A.load(a.buf.snap_a, a.buf.snap_b, a.buf.snap_c, li1 + R.off);
    C.load(a.buf.snap_a, a.buf.snap_b, a.buf.snap_c, li2 + R.off);
    const int cls = range_class(b1, b2, bt1, bt2, wp1, wp2);
    const float dfl = cls == 1 ? 0.5f * B.disp_f[q] : (cls == 2 ? 0.7f * B.disp_f[q] : B.disp_f[q]);
    const int e3 = side_of<float>(rr, dfl * (1.f - 1e-5f), dfl * (1.f + 1e-5f));
    if (e3 > 0) return;
    const int w = (t0 < 0 && e1 > 0 && e2 > 0 && e3 < 0)
                      ? candidate_side<float>(B, R, M, A, C, M.ooff[ty1] + ka, M.ooff[ty2] + kb) : 0;
    if (w < 0) return;
    if (w == 0) seg_append<int2>(a.bind_recheck, a.bind_ctr + kSegRecheck, a.bind_rcap, make_int2(wp1, wp2), a.flags);
    else add_edge_t<float>(a, wp1, wp2, cls, stamp);
}

// Every edge of the particle pair (s1, s2), s1 the lower particle index, d = x1 - x2 (minimum image) and
// r2 = |d|^2 as the caller's pair loop computed them.  Called once per pair on a bond-deciding pass.
template <class real>
__device__ __forceinline__ void bind_pair_edges(const ForceArgs<real> &a, const Replica<real> &R, const Model<real> &M,
                                             int r, int s1, int s2, int li1, int li2, const real d[3], real r2) {
    const BindRep &B = a.bind_reps[r];
    const int t0 = side_of<real>(r2, B.mk2_lo, B.mk2_hi);
    if (t0 > 0) return;
    const int ty1 = type_of<real>(M, li1), ty2 = type_of<real>(M, li2), na = M.np[ty1], nb = M.np[ty2];
    if (na == 0 || nb == 0) return;
    const real rr = sqrt(r2), u[3] = {d[0] / rr, d[1] / rr, d[2] / rr};
    Payload<real> P1;
    P1.load(a.buf.pos, a.buf.rota, a.buf.rotb, s1);
    real w1[3];
#pragma unroll
    for (int k = 0; k < 3; k++) w1[k] = P1.v[3 + 3 * k] * u[0] + P1.v[4 + 3 * k] * u[1] + P1.v[5 + 3 * k] * u[2];
    // particle 1's cones first: most pairs have no patch of it near any cone
    const real pre = (real)M.mincos[ty1][ty2] - (real)4e-5;
    const int o1 = M.ooff[ty1], o2 = M.ooff[ty2];
    real c1[kMaxOrient];
    bool any = false;
    for (int ka = 0; ka < na; ka++) {
        const real *v = M.orient[o1 + ka];
        c1[ka] = -(v[0] * w1[0] + v[1] * w1[1] + v[2] * w1[2]);
        any |= c1[ka] > pre;
    }
    if (!any) return;
    Payload<real> P2;
    P2.load(a.buf.pos, a.buf.rota, a.buf.rotb, s2);
    real w2[3];
#pragma unroll
    for (int k = 0; k < 3; k++) w2[k] = P2.v[3 + 3 * k] * u[0] + P2.v[4 + 3 * k] * u[1] + P2.v[5 + 3 * k] * u[2];
    const unsigned stamp = (unsigned)a.bind_ctr[2];
    for (int ka = 0; ka < na; ka++) {
        if (!(c1[ka] > pre)) continue;
        for (int kb = 0; kb < nb; kb++) {
            const real *v = M.orient[o2 + kb];
            bind_patch_edge<real>(a, B, R, M, s1, s2, li1, li2, ty1, ty2, ka, kb, c1[ka], v[0] * w2[0] + v[1] * w2[1] + v[2] * w2[2],
                                  rr, t0, stamp);
        }
    }
}

// skin lists: flags the next step for a rebuild when slot s's next position (xn) is more than half the
// skin away from where it was at the last build (minimum image)
template <class real>
__device__ __forceinline__ void skin_check(const ForceArgs<real> &a, const Replica<real> &R, int s, const real xn[3]) {
    real xr, yr, zr;
    load_pos(a.buf.xref + 4 * (size_t)s, xr, yr, zr);
    const real dx = min_image_sep<real>(xn[0], xr, R.box, R.box_lo, R.l2s, R.periodic);
    const real dy = min_image_sep<real>(xn[1], yr, R.box, R.box_lo, R.l2s, R.periodic);
    const real dz = min_image_sep<real>(xn[2], zr, R.box, R.box_lo, R.l2s, R.periodic);
    if (!(dx * dx + dy * dy + dz * dz <= R.half_skin2)) *a.skin_next = 1;
}

// Harmonic bonds of particle idi at (xi, yi, zi): HarmonicPotential::force (potential.h:274-276),
// f = -k (r - r0), along the minimum-image separation, as MD::calculateforces applies it to a bond list
// (MD.cpp:1684-1764).  Each bond is evaluated from both of its ends: x_j - x_i is exactly -(x_i - x_j),
// so the two forces are equal and opposite bit for bit and nothing is scattered.  Adds the force on idi
// to f, half of each bond's energy 0.5 k (r - r0)^2 to e.
template <class real>
__device__ __forceinline__ void bond_forces(const ForceArgs<real> &a, const Replica<real> &R, int idi, real xi, real yi,
                                            real zi, real f[3], real &e, bool &big) {
    const int b0 = __ldg(a.bond_start + idi), b1 = __ldg(a.bond_start + idi + 1);
    for (int b = b0; b < b1; b++) {
        const int j = __ldg(a.buf.slot_of + __ldg(a.bond_partner + b));
        real xj, yj, zj;
        load_pos(a.buf.pos + 4 * (size_t)j, xj, yj, zj);
        const real dx = min_image_sep<real>(xi, xj, R.box, R.box_lo, R.l2s, R.periodic);
        const real dy = min_image_sep<real>(yi, yj, R.box, R.box_lo, R.l2s, R.periodic);
        const real dz = min_image_sep<real>(zi, zj, R.box, R.box_lo, R.l2s, R.periodic);
        const real r = sqrt(dx * dx + dy * dy + dz * dz);
        const real f1 = -a.bond_k * (r - a.bond_r0);
        big |= fabs(f1) > real(1e4);
        f[0] += f1 * dx / r;
        f[1] += f1 * dy / r;
        f[2] += f1 * dz / r;
        e += real(0.25) * a.bond_k * (r - a.bond_r0) * (r - a.bond_r0);
    }
}

// ------------------------------------------------------------------ bound-pair forces (force epilogue)
// KernFrenkelOnePatch2::force_and_torque of every bound patch of particle idi (LangevinRforce.cpp:3940-4030):
// each pair is evaluated in its canonical order (lower particle index first) from both of its ends, so the
// two ends see equal and opposite forces bit for bit.  Adds the force and the lab torque on idi, and half of
// each pair's energy.
template <class real>
__device__ __forceinline__ void bound_patch_forces(const ForceArgs<real> &a, const Replica<real> &R,
                                                   const Model<real> &M, int r, int idi, const real Pi[12], real f[3],
                                                   real t[3], real &e) {
    const BindRep &B = a.bind_reps[r];
    const int li = idi - R.off, ti = type_of<real>(M, li), na = M.np[ti];
    for (int ka = 0; ka < na; ka++) {
        const int wp = patch_of<real>(B, M, li, ti, ka);
        if (!a.bind_on[wp]) continue;
        const int wq = a.bind_to[wp];
        int lj, tj, kb;
        patch_owner<real>(B, M, wq - B.patch_off, lj, tj, kb);
        const int sj = a.buf.slot_of[R.off + lj];
        Payload<real> Pj;
        Pj.load(a.buf.pos, a.buf.rota, a.buf.rotb, sj);
        const bool i_first = li < lj;
        const real *P1 = i_first ? Pi : Pj.v, *P2 = i_first ? Pj.v : Pi;
        const int t1 = i_first ? ti : tj, t2 = i_first ? tj : ti, c1 = i_first ? ka : kb, c2 = i_first ? kb : ka;
        const real dx = min_image_sep<real>(P1[0], P2[0], R.box, R.box_lo, R.l2s, R.periodic);
        const real dy = min_image_sep<real>(P1[1], P2[1], R.box, R.box_lo, R.l2s, R.periodic);
        const real dz = min_image_sep<real>(P1[2], P2[2], R.box, R.box_lo, R.l2s, R.periodic);
        const real rr = sqrt(dx * dx + dy * dy + dz * dz);
        const int q = M.pstart[t1][t2] + c1 * M.np[t2] + c2;
        if (rr > M.rmax[q]) continue;   // interaction_distance (potentialtheta.h:522)
        const real u[3] = {dx / rr, dy / rr, dz / rr};
        const real *b1 = M.orient[M.ooff[t1] + c1], *b2 = M.orient[M.ooff[t2] + c2];
        real n1[3], n2[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            n1[k] = b1[0] * P1[3 + k] + b1[1] * P1[6 + k] + b1[2] * P1[9 + k];
            n2[k] = b2[0] * P2[3 + k] + b2[1] * P2[6 + k] + b2[2] * P2[9 + k];
        }
        const real ci = -(n1[0] * u[0] + n1[1] * u[1] + n1[2] * u[2]);
        const real cj = n2[0] * u[0] + n2[1] * u[1] + n2[2] * u[2];
        if (!(ci > M.costm[q] && cj > M.costm[q])) continue;
        real fa[3] = {0, 0, 0}, ta[3] = {0, 0, 0}, tb[3] = {0, 0, 0}, ee = 0;
        kf2_pair<real>(M.att[q], M.dis[q], M.inv_dis[q], M.kfac[q], u, rr, n1, n2, ci, cj, fa, ta, tb, ee);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            f[k] += i_first ? fa[k] : -fa[k];
            t[k] += i_first ? ta[k] : tb[k];
        }
        e += real(0.5) * ee;
    }
}

// One particle by one thread: the straightforward form of the force loop.  Used by the FP64 path,
// the observable pass, replicas with fewer than three cells per side, and the FP32 tile kernel's
// fallback for crowded tiles.
template <class real, int MODE>
__device__ __noinline__ void simple_particle(const ForceArgs<real> &a, int s) {
    const Tables<real> &tb = a.tb;
    {
        const int r = replica_of(tb, s);
        const Replica<real> &R = tb.reps[r];
        const Model<real> &Mo = tb.models[R.model];
        Payload<real> P;
        P.load(a.buf.pos, a.buf.rota, a.buf.rotb, s);
        const real xi = P.v[0], yi = P.v[1], zi = P.v[2];
        const real *Qi = P.v + 3;
        const int idi = a.buf.ident[s];
        const int li = idi - R.off;
        const int ti = type_of<real>(Mo, li);
        const bool single_type = Mo.n_types == 1;

        Acc3<real> F, T;
        F.zero();
        T.zero();
        real ewca = real(0), epatch = real(0), vir = real(0);
        int bonds = 0, npairs = 0;
        bool big = false;

        const int nc = R.nc;
        int cx, cy, cz;
        if (a.skin && MODE != kModeObs) {
            // skin lists: the cell the slot was sorted into at the last build; particles have moved less
            // than half the skin since, so its stencil still holds every partner within the force range
            int key = a.buf.home_cell[s] - R.cell_off;
            if (key < 0 || key >= nc * nc * nc) {  // never after a rebuild on this grid; keep in range anyway
                atomicOr(a.flags, 16u);
                key = 0;
            }
            cx = key % nc;
            cy = (key / nc) % nc;
            cz = key / (nc * nc);
        } else {
            cx = axis_cell<real>(xi, R.cell_scale, nc);
            cy = axis_cell<real>(yi, R.cell_scale, nc);
            cz = axis_cell<real>(zi, R.cell_scale, nc);
        }
        // stencil offsets per axis, de-duplicated for grids of 1 or 2 cells (geometry.h:523-608)
        const int lo = nc >= 3 ? -1 : 0, hi = nc >= 2 ? 1 : 0;
        const real range2 = MODE == kModeObs ? (R.rc2 > R.bond_r * R.bond_r ? R.rc2 : R.bond_r * R.bond_r) : R.rc2;

        for (int dz = lo; dz <= hi; dz++) {
            // fewer than three cells per side: every cell of the side is a neighbour, walls or not
            int zz = nc < 3 ? dz : cz + dz;
            if (zz < 0 || zz >= nc) {
                if (!R.periodic) continue;
                zz = zz < 0 ? zz + nc : zz - nc;
            }
            for (int dy = lo; dy <= hi; dy++) {
                int yy = nc < 3 ? dy : cy + dy;
                if (yy < 0 || yy >= nc) {
                    if (!R.periodic) continue;
                    yy = yy < 0 ? yy + nc : yy - nc;
                }
                const int row = R.cell_off + nc * (yy + nc * zz);
                // x-range [cx+lo, cx+hi] as at most two contiguous slot segments
                int seg_a0, seg_a1, seg_b0 = 0, seg_b1 = 0;
                if (nc < 3) {
                    seg_a0 = __ldg(a.start + row);
                    seg_a1 = __ldg(a.start + row + nc);
                } else {
                    int x0 = cx - 1, x1 = cx + 1;
                    if (x0 < 0) {
                        seg_a0 = __ldg(a.start + row);
                        seg_a1 = __ldg(a.start + row + x1 + 1);
                        if (R.periodic) {
                            seg_b0 = __ldg(a.start + row + nc - 1);
                            seg_b1 = __ldg(a.start + row + nc);
                        }
                    } else if (x1 >= nc) {
                        seg_a0 = __ldg(a.start + row + x0);
                        seg_a1 = __ldg(a.start + row + nc);
                        if (R.periodic) {
                            seg_b0 = __ldg(a.start + row);
                            seg_b1 = __ldg(a.start + row + 1);
                        }
                    } else {
                        seg_a0 = __ldg(a.start + row + x0);
                        seg_a1 = __ldg(a.start + row + x1 + 1);
                    }
                }
                for (int seg = 0; seg < 2; seg++) {
                    const int j0 = seg ? seg_b0 : seg_a0, j1 = seg ? seg_b1 : seg_a1;
                    for (int j = j0; j < j1; j++) {
                        if (j == s) continue;
                        real xj, yj, zj;
                        load_pos(a.buf.pos + 4 * (size_t)j, xj, yj, zj);
                        real dx = min_image_sep<real>(xi, xj, R.box, R.box_lo, R.l2s, R.periodic);
                        real dy2 = min_image_sep<real>(yi, yj, R.box, R.box_lo, R.l2s, R.periodic);
                        real dz2 = min_image_sep<real>(zi, zj, R.box, R.box_lo, R.l2s, R.periodic);
                        real r2 = dx * dx + dy2 * dy2 + dz2 * dz2;
                        if (!(r2 < range2)) continue;
                        if (MODE == kModeEdges) {   // single-bond mode: this update's edges, each pair once
                            const int idj = __ldg(a.buf.ident + j);
                            if (idi < idj) {
                                const real dd[3] = {dx, dy2, dz2};
                                bind_pair_edges<real>(a, R, Mo, r, s, j, li, idj - R.off, dd, r2);
                            }
                            continue;
                        }
                        const real rr = sqrt(r2);
                        if (r2 < R.rc2) npairs++;
                        // WCA core: same vector for both orientations of the pair
                        real fi[3] = {0, 0, 0};
                        if (rr < R.hs_limit && (a.parts & 1)) {
                            real s_ = hs_force_over_r<real>(R, r2);
                            big |= fabs(s_ * rr) > real(1e4);
                            fi[0] = s_ * dx; fi[1] = s_ * dy2; fi[2] = s_ * dz2;
                            ewca += real(0.5) * wca_energy<real>(R, r2);
                        }
                        real ti_[3] = {0, 0, 0};
                        if ((a.parts & 2) && (r2 < R.patch_r2 || MODE == kModeObs)) {
                            const int idj = __ldg(a.buf.ident + j);
                            const int tj = single_type ? 0 : type_of<real>(Mo, idj - R.off);
                            if (Mo.np[ti] > 0 && Mo.np[tj] > 0) {
                                Payload<real> Pj;
                                Pj.load(a.buf.pos, a.buf.rota, a.buf.rotb, j);
                                const bool i_first = idi < idj;  // canonical order of the reference (p1 < p2)
                                real u[3];
                                const real inv = real(1) / rr;
                                const real sg = i_first ? real(1) : real(-1);
                                u[0] = sg * dx * inv; u[1] = sg * dy2 * inv; u[2] = sg * dz2 * inv;
                                real f[3] = {0, 0, 0}, tqa[3] = {0, 0, 0}, tqb[3] = {0, 0, 0}, e = 0;
                                int nb = 0;
                                const bool force_ok = r2 < R.max_dist2;
                                if (force_ok || MODE == kModeObs) {
                                    if (i_first)
                                        patch_pair<real>(Mo, ti, tj, Qi, Pj.v + 3, u, rr, R.bond_r, f, tqa, tqb, e, nb);
                                    else
                                        patch_pair<real>(Mo, tj, ti, Pj.v + 3, Qi, u, rr, R.bond_r, f, tqa, tqb, e, nb);
                                }
                                if (!force_ok) { f[0] = f[1] = f[2] = 0; tqa[0] = tqa[1] = tqa[2] = 0; tqb[0] = tqb[1] = tqb[2] = 0; e = 0; }
                                bonds += nb;
                                epatch += real(0.5) * e;
#pragma unroll
                                for (int k = 0; k < 3; k++) {
                                    fi[k] += sg * f[k];
                                    ti_[k] = i_first ? tqa[k] : tqb[k];
                                }
                            }
                        }
                        F.add(fi[0], fi[1], fi[2]);
                        T.add(ti_[0], ti_[1], ti_[2]);
                        vir += real(0.5) * (dx * fi[0] + dy2 * fi[1] + dz2 * fi[2]);
                    }
                }
            }
        }
        if (MODE == kModeEdges) return;
        real ebond = real(0);
        if (a.bond_start && MODE != kModeObs && (a.parts & 1)) {
            real fb[3] = {real(0), real(0), real(0)};
            bond_forces<real>(a, R, idi, xi, yi, zi, fb, ebond, big);
            F.add(fb[0], fb[1], fb[2]);
        }
        if (a.bind_on && MODE != kModeObs && (a.parts & 2)) {
            real fb[3] = {real(0), real(0), real(0)}, tb[3] = {real(0), real(0), real(0)};
            bound_patch_forces<real>(a, R, Mo, r, idi, P.v, fb, tb, epatch);
            F.add(fb[0], fb[1], fb[2]);
            T.add(tb[0], tb[1], tb[2]);
        }
        if (big) atomicOr(a.flags, 2u);

        if (MODE == kModeForces) {
            a.outF[3 * (size_t)idi + 0] = F.get(0);
            a.outF[3 * (size_t)idi + 1] = F.get(1);
            a.outF[3 * (size_t)idi + 2] = F.get(2);
            a.outT[3 * (size_t)idi + 0] = T.get(0);
            a.outT[3 * (size_t)idi + 1] = T.get(1);
            a.outT[3 * (size_t)idi + 2] = T.get(2);
            if (a.outE) a.outE[idi] = (double)ewca + (double)epatch + (double)ebond;
            return;
        }
        if (MODE == kModeObs) {
            // warp-shuffle reduction when the whole warp is in one replica, else per-lane atomics
            double v[5] = {0, 0, 0, 0, 0};
            v[2] = (double)vir;
            v[4] = 0.5 * (double)npairs;
            v[3] = 0.5 * (double)bonds;
            v[0] = (double)epatch;
            v[1] = (double)ewca;
            double *o = a.obs + 5 * (size_t)r;
#pragma unroll
            for (int k = 0; k < 5; k++) atomicAdd(o + k, v[k]);
            return;
        }

        // ---- create_forces_and_torques_sphere (LangevinR.cpp:474-578) + advancemom_halfstep
        Row<real> Mv;
        Mv.load(a.buf.motion + (size_t)s * kRow);
        real p[3] = {Mv.v[0], Mv.v[1], Mv.v[2]}, L[3] = {Mv.v[3], Mv.v[4], Mv.v[5]};
        real xi6[6];
        if (a.ext_noise) {
#pragma unroll
            for (int k = 0; k < 6; k++) xi6[k] = (real)a.ext_noise[6 * (size_t)idi + k];
        } else {
            philox_noise6<real>((uint32_t)li, (uint32_t)r, a.draw[0], R.seed_lo, R.seed_hi, xi6);
        }
        real pb[3], fb[3];
#pragma unroll
        for (int k = 0; k < 3; k++) pb[k] = Qi[3 * k] * p[0] + Qi[3 * k + 1] * p[1] + Qi[3 * k + 2] * p[2];
#pragma unroll
        for (int k = 0; k < 3; k++) fb[k] = R.fric_t * pb[k] + R.Rt * xi6[k];
        real Ft[3], Tt[3], Fl[3] = {F.get(0), F.get(1), F.get(2)}, Tl[3] = {T.get(0), T.get(1), T.get(2)};
#pragma unroll
        for (int k = 0; k < 3; k++) {
            Ft[k] = Fl[k] + fb[0] * Qi[k] + fb[1] * Qi[3 + k] + fb[2] * Qi[6 + k];
            Tt[k] = R.fric_r * L[k] + R.Rr * xi6[3 + k] + Tl[0] * Qi[3 * k] + Tl[1] * Qi[3 * k + 1] + Tl[2] * Qi[3 * k + 2];
        }
        if (a.do_kick) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                p[k] = add_rn(p[k], mul_rn(R.half_dt, Ft[k]));
                L[k] = L[k] + R.half_dt * Tt[k];
            }
        }
        if (!(isfinite(Ft[0]) && isfinite(Ft[1]) && isfinite(Ft[2]) && isfinite(Tt[0]) && isfinite(Tt[1]) &&
              isfinite(Tt[2]) && isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2])))
            atomicOr(a.flags, 1u);
        Mv.v[0] = p[0]; Mv.v[1] = p[1]; Mv.v[2] = p[2];
        Mv.v[3] = L[0]; Mv.v[4] = L[1]; Mv.v[5] = L[2];
        Mv.v[6] = Ft[0]; Mv.v[7] = Ft[1]; Mv.v[8] = Ft[2];
        Mv.v[9] = Tt[0]; Mv.v[10] = Tt[1]; Mv.v[11] = Tt[2];
        Mv.store(a.buf.motion + (size_t)s * kRow);

        // ---- bin the next step's position (same arithmetic as the scatter pass), or with skin lists
        // check how far it will be from where the lists were built
        real xn[3] = {xi, yi, zi}, pn[3] = {p[0], p[1], p[2]};
        drift_position<real>(R, xn, pn, Ft);
        if (!(isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]))) {
            atomicOr(a.flags, 1u);
            xn[0] = xn[1] = xn[2] = real(0);
        }
        if (a.skin) {
            skin_check<real>(a, R, s, xn);
        } else {
            const int key = cell_of<real>(R, xn[0], xn[1], xn[2]);
            const int rank = aggregated_rank(a.count, key);
            a.bin[s] = make_int2(key, rank);
        }
    }
}

template <class real, int MODE>
__global__ void __launch_bounds__(128) force_kernel(ForceArgs<real> a) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < a.tb.ntot; s += gridDim.x * blockDim.x)
        simple_particle<real, MODE>(a, s);
}

// ------------------------------------------------------------------ state in / out, reductions

// host-order doubles (ntot rows) -> rows in slot order == global index order
template <class real>
__global__ void load_state_kernel(int ntot, const double *x, const double *p, const double *Lb, const double *Q,
                                  const double *Ft, const double *Tt, Buffers<real> out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntot; i += gridDim.x * blockDim.x) {
        Payload<real> P;
        Row<real> M;
        P.v[0] = (real)x[3 * (size_t)i]; P.v[1] = (real)x[3 * (size_t)i + 1]; P.v[2] = (real)x[3 * (size_t)i + 2];
        for (int k = 0; k < 9; k++) P.v[3 + k] = (real)Q[9 * (size_t)i + k];
        for (int k = 0; k < 3; k++) {
            M.v[k] = (real)p[3 * (size_t)i + k];
            M.v[3 + k] = (real)Lb[3 * (size_t)i + k];
            M.v[6 + k] = Ft ? (real)Ft[3 * (size_t)i + k] : real(0);
            M.v[9 + k] = Tt ? (real)Tt[3 * (size_t)i + k] : real(0);
        }
        P.store(out.pos, out.rota, out.rotb, i);
        M.store(out.motion + (size_t)i * kRow);
        out.ident[i] = i;
        if (out.slot_of) out.slot_of[i] = i;
        if (out.dx) { out.dx[i] = 0; out.dy[i] = 0; out.dz[i] = 0; }
    }
}

// id -> slot map of a buffer (when bonds are set on a system that already holds a state)
__global__ void slot_map_kernel(int ntot, const int *ident, int *slot_of) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ntot; s += gridDim.x * blockDim.x) slot_of[ident[s]] = s;
}

// slot order -> host order doubles by global index i, from the slot map (slot_of[i]): the rows are gathered
// and the doubles written in order, so every warp writes contiguous bytes (the slot-order form scatters its
// 24-byte rows across the whole array)
template <class real>
__global__ void gather_state_kernel(int ntot, Buffers<real> in, const int *slot_of, double *x, double *p, double *Lb,
                                    double *Q, double *Ft, double *Tt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntot; i += gridDim.x * blockDim.x) {
        const size_t s = (size_t)__ldg(slot_of + i), ii = (size_t)i;
        Payload<real> P;
        Row<real> M;
        P.load(in.pos, in.rota, in.rotb, s);
        M.load(in.motion + s * kRow);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (x) x[3 * ii + k] = (double)P.v[k];
            if (p) p[3 * ii + k] = (double)M.v[k];
            if (Lb) Lb[3 * ii + k] = (double)M.v[3 + k];
            if (Ft) Ft[3 * ii + k] = (double)M.v[6 + k];
            if (Tt) Tt[3 * ii + k] = (double)M.v[9 + k];
        }
        if (Q)
#pragma unroll
            for (int k = 0; k < 9; k++) Q[9 * ii + k] = (double)P.v[3 + k];
    }
}

// slot order -> host order doubles; which: bit0 x, bit1 p, bit2 Lb, bit3 Q, bit4 Ft, bit5 Tt, bit6 disp
template <class real>
__global__ void store_state_kernel(int ntot, Buffers<real> in, double *x, double *p, double *Lb, double *Q, double *Ft,
                                   double *Tt, double *disp) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ntot; s += gridDim.x * blockDim.x) {
        Payload<real> P;
        Row<real> M;
        P.load(in.pos, in.rota, in.rotb, s);
        M.load(in.motion + (size_t)s * kRow);
        const size_t i = (size_t)in.ident[s];
        for (int k = 0; k < 3; k++) {
            if (x) x[3 * i + k] = (double)P.v[k];
            if (p) p[3 * i + k] = (double)M.v[k];
            if (Lb) Lb[3 * i + k] = (double)M.v[3 + k];
            if (Ft) Ft[3 * i + k] = (double)M.v[6 + k];
            if (Tt) Tt[3 * i + k] = (double)M.v[9 + k];
        }
        if (Q)
            for (int k = 0; k < 9; k++) Q[9 * i + k] = (double)P.v[3 + k];
        if (disp && in.dx) {
            disp[3 * i] = in.dx[s];
            disp[3 * i + 1] = in.dy[s];
            disp[3 * i + 2] = in.dz[s];
        }
    }
}

// LangevinNVTR::measured_temperature sums (LangevinR.cpp:170-193): per replica sum p_k^2, sum L_k^2
// p and L of a motion row (its first six values)
__device__ __forceinline__ void load_pl(const float *row, float v[6]) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(row));
    const float2 b = __ldg(reinterpret_cast<const float2 *>(row + 4));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
}
__device__ __forceinline__ void load_pl(const double *row, double v[6]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(row) + k);
        v[2 * k] = a.x;
        v[2 * k + 1] = a.y;
    }
}

// Sum of squares of a thread's values.  FP32 rows: each square is split exactly into two floats (product
// and its rounding error, by FMA) and added with TwoSum, so the float pair (hi, lo) carries about 48 bits
// and the result matches a double-precision sum of the squares to ~1e-14 relative without FP64 arithmetic
// per particle.  FP64 rows: plain double arithmetic.
template <class real> struct SqSum;
template <> struct SqSum<float> {
    float hi[6], lo[6];
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int k = 0; k < 6; k++) hi[k] = lo[k] = 0.f;
    }
    __device__ __forceinline__ void add(const float v[6]) {
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const float p = __fmul_rn(v[k], v[k]), pe = __fmaf_rn(v[k], v[k], -p);   // p + pe = v^2 exactly
            const float s = __fadd_rn(hi[k], p), bb = __fsub_rn(s, hi[k]);
            const float e = __fadd_rn(__fsub_rn(hi[k], __fsub_rn(s, bb)), __fsub_rn(p, bb));  // hi + p = s + e
            hi[k] = s;
            lo[k] = __fadd_rn(lo[k], __fadd_rn(e, pe));
        }
    }
    __device__ __forceinline__ double get(int k) const { return (double)hi[k] + (double)lo[k]; }
    // the sums of all 32 lanes into lane 0, as float pairs (TwoSum of the high parts, low parts added): the
    // warp's reduction stays off the FP64 pipe, which on this part runs at a small fraction of the FP32 rate
    __device__ __forceinline__ void warp_reduce() {
#pragma unroll
        for (int k = 0; k < 6; k++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_down_sync(0xffffffffu, hi[k], o), ol = __shfl_down_sync(0xffffffffu, lo[k], o);
                const float s = __fadd_rn(hi[k], oh), bb = __fsub_rn(s, hi[k]);
                const float e = __fadd_rn(__fsub_rn(hi[k], __fsub_rn(s, bb)), __fsub_rn(oh, bb));
                hi[k] = s;
                lo[k] = __fadd_rn(lo[k], __fadd_rn(ol, e));
            }
        }
    }
};
template <> struct SqSum<double> {
    double v_[6];
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int k = 0; k < 6; k++) v_[k] = 0.0;
    }
    __device__ __forceinline__ void add(const double v[6]) {
#pragma unroll
        for (int k = 0; k < 6; k++) v_[k] += v[k] * v[k];
    }
    __device__ __forceinline__ double get(int k) const { return v_[k]; }
    __device__ __forceinline__ void warp_reduce() {
#pragma unroll
        for (int k = 0; k < 6; k++)
            for (int o = 16; o > 0; o >>= 1) v_[k] += __shfl_down_sync(0xffffffffu, v_[k], o);
    }
};

constexpr int kTempPerThread = 8;   // slots per thread: a block of 256 threads sums 2048 slots

template <class real>
__global__ void __launch_bounds__(256) temperature_kernel(Tables<real> tb, Buffers<real> in, double *out) {
    // block b sums 2048 consecutive slots, the last ones first (the step's epilogue wrote them last, so more
    // of them are still in L2: 5 us a step less): replicas are contiguous slot ranges, so a thread's slots
    // almost always belong to one replica.  A thread loads all its rows first (independent loads in flight
    // together), then walks the replica boundaries in slot order, adds its slots of a replica up, and the warp
    // reduces before the atomics.  (Four slots a thread, 48 registers instead of 76, measured no faster.)
    const int base = (gridDim.x - 1 - blockIdx.x) * (kTempPerThread * blockDim.x) + threadIdx.x;
    real v[kTempPerThread][6];
#pragma unroll
    for (int i = 0; i < kTempPerThread; i++) {
        const int s = base + i * blockDim.x;
        if (s < tb.ntot) {
            load_pl(in.motion + (size_t)s * kRow, v[i]);
        } else {
#pragma unroll
            for (int k = 0; k < 6; k++) v[i][k] = real(0);
        }
    }
    SqSum<real> acc;
    acc.clear();
    int cur = -1, next_start = 0;
#pragma unroll
    for (int i = 0; i < kTempPerThread; i++) {
        const int s = base + i * blockDim.x;
        if (s >= tb.ntot) break;
        if (s >= next_start) {  // a replica boundary (slots ascend)
            if (cur >= 0)
                for (int k = 0; k < 6; k++) atomicAdd(out + 6 * (size_t)cur + k, acc.get(k));
            cur = replica_of(tb, s);
            next_start = __ldg(tb.rep_slot + cur + 1);
            acc.clear();
        }
        acc.add(v[i]);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, cur);
    if (peers == 0xffffffffu) {
        acc.warp_reduce();
        if ((threadIdx.x & 31) == 0 && cur >= 0)
            for (int k = 0; k < 6; k++) atomicAdd(out + 6 * (size_t)cur + k, acc.get(k));
    } else if (cur >= 0) {
        for (int k = 0; k < 6; k++) atomicAdd(out + 6 * (size_t)cur + k, acc.get(k));
    }
}


// ------------------------------------------------------------------ the step's phases one at a time
// The reference's loop body calls advancemom_halfstep, advance_pos, rotate, the force routines and
// create_forces_and_torques_sphere separately (Condensate.cpp:335-378).  These kernels run one phase on the
// handle's state (every slot) with the caller's forces, torques and noise given by global index, in the same
// arithmetic as the fused step, so a driver can swap its loop body method by method.

// LangevinNVTR::advancemom_halfstep(F, T) (LangevinR.cpp:327-347): p += dt/2 F (lab), L_body += dt/2 T (body)
template <class real>
__global__ void phase_halfkick_kernel(Tables<real> tb, Buffers<real> b, const double *F, const double *T) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < tb.ntot; s += gridDim.x * blockDim.x) {
        const Replica<real> &R = tb.reps[replica_of(tb, s)];
        const size_t id = (size_t)b.ident[s];
        Row<real> M;
        M.load(b.motion + (size_t)s * kRow);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            M.v[k] = add_rn(M.v[k], mul_rn(R.half_dt, (real)F[3 * id + k]));
            M.v[3 + k] = M.v[3 + k] + R.half_dt * (real)T[3 * id + k];
        }
        M.store(b.motion + (size_t)s * kRow);
    }
}

// LangevinNVT::advance_pos (Langevin.cpp:205-222): x += dt/m p, then cube::correct_position_and_momentum
// (wrap, or reflect and negate p at a wall, geometry.h:403-446); the FP64 displacement follows the drift
template <class real>
__global__ void phase_drift_kernel(Tables<real> tb, Buffers<real> b, unsigned *flags) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < tb.ntot; s += gridDim.x * blockDim.x) {
        const Replica<real> &R = tb.reps[replica_of(tb, s)];
        Row<real> M;
        M.load(b.motion + (size_t)s * kRow);
        real x[4];
        load4(b.pos + 4 * (size_t)s, x);
        real step[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            step[k] = mul_rn(R.c1, M.v[k]);
            x[k] = add_rn(x[k], step[k]);
            wrap_coord<real>(x[k], M.v[k], R.box, R.periodic);
        }
        if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) atomicOr(flags, 1u);
        store4(b.pos + 4 * (size_t)s, x[0], x[1], x[2], x[3]);
        M.store(b.motion + (size_t)s * kRow);
        if (b.dx) {
            b.dx[s] += (double)step[0];
            b.dy[s] += (double)step[1];
            b.dz[s] += (double)step[2];
        }
    }
}

// LangevinNVTR::rotate() (LangevinR.cpp:594-695): the free-rotor propagator of genfullmat, L <- R L, Q <- R^T Q
template <class real>
__global__ void phase_rotate_kernel(Tables<real> tb, Buffers<real> b) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < tb.ntot; s += gridDim.x * blockDim.x) {
        const Replica<real> &R = tb.reps[replica_of(tb, s)];
        Payload<real> P;
        Row<real> M;
        P.load(b.pos, b.rota, b.rotb, s);
        M.load(b.motion + (size_t)s * kRow);
        const real L[3] = {M.v[3], M.v[4], M.v[5]};
        real Rm[9];
        free_rotor<real>(R.dt, R.inertia, L, Rm);
#pragma unroll
        for (int a = 0; a < 3; a++) M.v[3 + a] = L[0] * Rm[3 * a] + L[1] * Rm[3 * a + 1] + L[2] * Rm[3 * a + 2];
        real Q[9];
#pragma unroll
        for (int k = 0; k < 9; k++) Q[k] = P.v[3 + k];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) P.v[3 + 3 * a + c] = Q[c] * Rm[a] + Q[3 + c] * Rm[3 + a] + Q[6 + c] * Rm[6 + a];
        P.store(b.pos, b.rota, b.rotb, s);
        M.store(b.motion + (size_t)s * kRow);
    }
}

// LangevinNVTR::create_forces_and_torques_sphere(F, T, R) (LangevinR.cpp:474-592): friction and noise added to
// the caller's lab-frame F and T; out: F~ (lab) and T~ (body) by global index, also kept as the carried F~/T~
// of the state.  noise: the caller's R (ntot x 6 by global index), or null for the handle's Philox draw.
template <class real>
__global__ void phase_langevin_kernel(Tables<real> tb, Buffers<real> b, const double *F, const double *T,
                                      const double *noise, const unsigned long long *draw, double *outF,
                                      double *outT, unsigned *flags) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < tb.ntot; s += gridDim.x * blockDim.x) {
        const int r = replica_of(tb, s);
        const Replica<real> &R = tb.reps[r];
        const int id = b.ident[s];
        Payload<real> P;
        Row<real> M;
        P.load(b.pos, b.rota, b.rotb, s);
        M.load(b.motion + (size_t)s * kRow);
        const real *Qi = P.v + 3;
        real xi6[6];
        if (noise) {
#pragma unroll
            for (int k = 0; k < 6; k++) xi6[k] = (real)noise[6 * (size_t)id + k];
        } else {
            philox_noise6<real>((uint32_t)(id - R.off), (uint32_t)r, draw[0], R.seed_lo, R.seed_hi, xi6);
        }
        real Fl[3], Tl[3], pb[3], fb[3], Ft[3], Tt[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            Fl[k] = (real)F[3 * (size_t)id + k];
            Tl[k] = (real)T[3 * (size_t)id + k];
        }
#pragma unroll
        for (int k = 0; k < 3; k++) pb[k] = Qi[3 * k] * M.v[0] + Qi[3 * k + 1] * M.v[1] + Qi[3 * k + 2] * M.v[2];
#pragma unroll
        for (int k = 0; k < 3; k++) fb[k] = R.fric_t * pb[k] + R.Rt * xi6[k];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            Ft[k] = Fl[k] + fb[0] * Qi[k] + fb[1] * Qi[3 + k] + fb[2] * Qi[6 + k];
            Tt[k] = R.fric_r * M.v[3 + k] + R.Rr * xi6[3 + k] + Tl[0] * Qi[3 * k] + Tl[1] * Qi[3 * k + 1] +
                    Tl[2] * Qi[3 * k + 2];
        }
        if (!(isfinite(Ft[0]) && isfinite(Ft[1]) && isfinite(Ft[2]) && isfinite(Tt[0]) && isfinite(Tt[1]) &&
              isfinite(Tt[2])))
            atomicOr(flags, 1u);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            M.v[6 + k] = Ft[k];
            M.v[9 + k] = Tt[k];
            outF[3 * (size_t)id + k] = (double)Ft[k];
            outT[3 * (size_t)id + k] = (double)Tt[k];
        }
        M.store(b.motion + (size_t)s * kRow);
    }
}

}  // namespace
}  // namespace mtg
