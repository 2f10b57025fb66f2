// mtg_pipe.cuh -- the force pass as a pair pipeline: high-occupancy kernels, no shared-memory tiles.
// FP32 (the batched path) and FP64 (the plain single-system path) share the kernels; they differ in the
// per-particle sums (FP32: 64-bit fixed point, order-independent; FP64: double atomics) and in the
// single-bond kernels, which are FP32 only.
//
//   pairfind   one thread per particle (slot s): every candidate t > s of the 27 cells around s's cell
//              within the range (the force range, or with a neighbour skin the list range) is one
//              unordered pair (s, t), appended through a per-block buffer to a list in HBM
//   pairforce  one thread per pair: WCA core (HSPotential, MD::calculateforces) and the Kern-Frenkel
//              patch potentials (calculate_forces_and_torques3D) of the pair in the reference's canonical
//              order (lower particle index first), added to BOTH particles as 64-bit fixed-point sums
//              (integer atomics commute: the sums do not depend on the order of the pairs)
//   epilogue   one thread per particle: read and clear the sums, bonds, friction + Philox noise,
//              half-kick, next-step binning (or the skin displacement check)
//
// With a neighbour skin the pair list is built only on rebuild steps (slots do not move in between) and
// the force kernel drops the pairs beyond the force range each step.
#pragma once

#include "mtg_tile.cuh"

namespace mtg {
namespace {  // internal linkage

constexpr int kPipeThreads = 256;      // block size of the grid-stride pair kernels; pairfind and the epilogue
                                       // take theirs from the launch configuration (128, 256 or 512)
constexpr int kPairsPerThread = 8;     // pairs a pairfind block buffers in shared memory, per thread
constexpr int kPairsPerParticle = 16;  // capacity of the pair list (unordered pairs per particle)

// |d|^2 with explicit roundings (no contraction).  Pair finding tests a cheaper separation against a range widened
// by its rounding (rc2_find), so it finds a superset of the pairs; the pair kernels decide each pair with the
// exact separation (min_image_sep) and drop the rest, so every path takes the same pair set.
template <class real>
__device__ __forceinline__ real sep_r2(real dx, real dy, real dz) {
    return add_rn(add_rn(mul_rn(dx, dx), mul_rn(dy, dy)), mul_rn(dz, dz));
}

__device__ __forceinline__ float sqrt_r(float v) { return sqrtf(v); }
__device__ __forceinline__ double sqrt_r(double v) { return sqrt(v); }

// the per-slot force/torque sums of the pair kernels: FP32 in 64-bit fixed point (integer atomics commute,
// so the sums do not depend on the order of the pairs), FP64 in doubles (hardware double atomics; the
// order changes the last bits only)
template <class real> struct PairAcc { using type = long long; };
template <> struct PairAcc<double> { using type = double; };

// orientation rows of a slot for the FP64 pipeline (the FP32 form sits beside the tile kernel)
__device__ __forceinline__ void load_q(const ForceArgs<double> &a, int slot, double q8, double Q[9]) {
    double b[4], c[4];
    load4(a.buf.rota + 4 * (size_t)slot, b);
    load4(a.buf.rotb + 4 * (size_t)slot, c);
    Q[0] = b[0]; Q[1] = b[1]; Q[2] = b[2]; Q[3] = b[3];
    Q[4] = c[0]; Q[5] = c[1]; Q[6] = c[2]; Q[7] = c[3]; Q[8] = q8;
}

// The squared separation pair finding tests: fused multiply-adds, rounded differently from sep_r2 by at most a
// few units in the last place, which the relative widening of the finding range (1e-6) covers.
__device__ __forceinline__ float find_r2(float dx, float dy, float dz) { return fmaf(dx, dx, fmaf(dy, dy, dz * dz)); }
__device__ __forceinline__ double find_r2(double dx, double dy, double dz) { return fma(dx, dx, fma(dy, dy, dz * dz)); }

// Pair finding keeps each warp's pairs in its own part of the block's shared-memory buffer.
constexpr int kWarpPairs = kPairsPerThread * 32;

// Appends the pairs (s, c0 + b) for every bit b of each lane's mask to the warp's part of the buffer: per round
// one ballot, and every lane with a bit left writes its lowest at the warp's count plus the number of lower
// lanes writing in that round.  `cnt` (the same in every lane) counts the warp's pairs; entries past the part
// go straight to the list, where the pair-force kernel takes them.  Called by all 32 lanes.
__device__ __forceinline__ void warp_append(int2 *part, int &cnt, int s, int c0, unsigned mask, int2 *pairs,
                                            unsigned long long *npairs, long long cap, unsigned *flags) {
    const unsigned lower = (1u << (threadIdx.x & 31)) - 1u;
    for (;;) {
        const unsigned bal = __ballot_sync(0xffffffffu, mask != 0u);
        if (bal == 0u) break;
        if (mask) {
            const int b = __ffs(mask) - 1;
            mask &= mask - 1u;
            const int q = cnt + __popc(bal & lower);
            const int2 p = make_int2(s, c0 + b);
            if (q < kWarpPairs) {
                part[q] = p;
            } else {
                const unsigned long long w = atomicAdd(npairs, 1ull);
                if ((long long)w < cap) pairs[w] = p;
                else atomicOr(flags, 8u);
            }
        }
        cnt += __popc(bal);
    }
}

// The candidates [t0, t1) of one lane, tested against the lane's position minus the segment's image shift
// (qx, qy, qz), in chunks of at most 32 slots whose hits are marked in a bit mask and appended by the warp
// together (the chunk loop is warp-uniform; the candidate loop is not unrolled: the lanes' trip counts differ,
// and an unrolled body keeps the short lanes idle for longer).
template <class real>
__device__ __forceinline__ void scan_segment(const real *pos, int t0, int t1, real qx, real qy, real qz, real range2,
                                             int2 *part, int &cnt, int s, int2 *pairs, unsigned long long *npairs,
                                             long long cap, unsigned *flags) {
    for (int c0 = t0; __any_sync(0xffffffffu, c0 < t1); c0 += 32) {
        unsigned mask = 0u;
        const int ce = t1 < c0 + 32 ? t1 : c0 + 32;
#pragma unroll 1
        for (int t = c0; t < ce; t++) {
            real pj[3];
            load_pos(pos + 4 * (size_t)t, pj[0], pj[1], pj[2]);
            if (find_r2(qx - pj[0], qy - pj[1], qz - pj[2]) < range2) mask |= 1u << (t - c0);
        }
        warp_append(part, cnt, s, c0, mask, pairs, npairs, cap, flags);
    }
}

// the pair list's length (on list-building steps) and the patch list's segment counters (every pass)
__global__ void pair_reset_kernel(unsigned long long *npairs, const int *gate, unsigned long long *patch_counts) {
    if (patch_counts && blockIdx.x == 0)
        for (int k = threadIdx.x; k < kSegs; k += blockDim.x) patch_counts[k] = 0ull;
    if (gated_off(gate, 1)) return;
    if (threadIdx.x == 0 && blockIdx.x == 0) *npairs = 0ull;
}

// Pairs a pair kernel lists go through a per-block staging buffer in shared memory (a shared-memory
// atomic per appending warp) and reach their segmented list with one global atomic per block at the end
// (segment blockIdx mod kSegs); entries past the buffer go straight to the list.
constexpr int kBlockListCap = 1024;

__device__ __forceinline__ void block_list_put(int2 *sbuf, int *sn, int2 e, int2 *list, unsigned long long *counts,
                                               long long cap, unsigned *flags, unsigned full_flag) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    int q = 0;
    if (g.thread_rank() == 0) q = atomicAdd(sn, (int)g.size());
    q = g.shfl(q, 0) + (int)g.thread_rank();
    if (q < kBlockListCap) sbuf[q] = e;
    else seg_append<int2>(list, counts, cap, e, flags, full_flag);
}

// all threads of the block
__device__ __forceinline__ void block_list_flush(const int2 *sbuf, const int *sn, unsigned long long *sbase,
                                                 int2 *list, unsigned long long *counts, long long cap,
                                                 unsigned *flags, unsigned full_flag) {
    __syncthreads();
    const int n = *sn < kBlockListCap ? *sn : kBlockListCap;
    const int k = (int)(blockIdx.x & (kSegs - 1));
    if (threadIdx.x == 0) *sbase = n ? atomicAdd(counts + k, (unsigned long long)n) : 0ull;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const unsigned long long w = *sbase + (unsigned long long)i;
        if ((long long)w < cap) list[(size_t)k * (size_t)cap + w] = sbuf[i];
        else atomicOr(flags, full_flag);
    }
}

__device__ __forceinline__ void fixed_add(long long *acc, float v) {
    if (v != 0.f) atomicAdd(reinterpret_cast<unsigned long long *>(acc), (unsigned long long)to_fixed(v));
}
__device__ __forceinline__ void fixed_add(double *acc, double v) {
    if (v != 0.0) atomicAdd(acc, v);
}
// a term already in the sum's representation (FP32: fixed point; FP64: double)
__device__ __forceinline__ void acc_add_raw(long long *acc, long long v) {
    if (v != 0) atomicAdd(reinterpret_cast<unsigned long long *>(acc), (unsigned long long)v);
}
__device__ __forceinline__ void acc_add_raw(double *acc, double v) {
    if (v != 0.0) atomicAdd(acc, v);
}

// Forces and torques of the listed pairs into acc (6 fixed-point sums per slot: F lab, T lab).
// KIND kPairSplit: WCA core here; pairs where both particles have a patch near a cone go to `list` for
//   patch_pairs_kernel, which evaluates their patch terms with every lane busy (the rest of the pairs
//   never reach the patch code, so this kernel runs without the divergent, register-heavy branch).
// KIND kPairBind (single-bond mode, a bond-deciding pass): WCA core here; pairs where both particles have
//   a patch near a cone go, in canonical order (lower particle index first), to `list` for
//   bind_pairs_kernel.
enum PairKind : int { kPairBind = 1, kPairSplit = 2 };

// whether a patch of type ty has sign (n . w) above mc: up to four patches unrolled, their loads issued together
template <class real>
__device__ __forceinline__ bool cone_any(const Model<real> &M, int ty, const real w[3], real mc, real sign) {
    const int np = M.np[ty], o = M.ooff[ty];
    bool any = false;
    if (np <= 4) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k < np) {
                const real *v = M.orient[o + k];
                any |= sign * (v[0] * w[0] + v[1] * w[1] + v[2] * w[2]) > mc;
            }
        }
        return any;
    }
    for (int k = 0; k < np; k++) {
        const real *v = M.orient[o + k];
        any |= sign * (v[0] * w[0] + v[1] * w[1] + v[2] * w[2]) > mc;
    }
    return any;
}

// One listed pair (sa, sb): the WCA core into acc (both particles), and -- KIND kPairSplit -- the pair onto
// `list` when both particles have a patch near a cone, or -- KIND kPairBind -- onto `list` in canonical order
// when both do (single-bond mode).  List entries are staged in the block's lbuf (block_list_put).
// rhint >= 0: sa's replica, known to the caller.
// The WCA core of the pair (sa, sb) into both particles' sums: FP32 as exact-ish float-float components summed
// in fixed point, FP64 in double.
template <class real>
__device__ __forceinline__ void wca_core(const ForceArgs<real> &a, const Replica<real> &R, int sa, int sb,
                                         const real d[3], real r2, typename PairAcc<real>::type *acc, bool &big) {
    typename PairAcc<real>::type fa[3] = {0, 0, 0};
    if constexpr (sizeof(real) == 4) {
        float hi[3], lo[3];
        hs_force_ff(R, d, hi, lo);
        big |= hi[0] * hi[0] + hi[1] * hi[1] + hi[2] * hi[2] > 1e8f;   // |f| > 1e4
#pragma unroll
        for (int k = 0; k < 3; k++) fa[k] = to_fixed(hi[k]) + to_fixed(lo[k]);
    } else {
        const real s_ = hs_force_over_r<real>(R, r2);
        big |= fabs(s_ * sqrt_r(r2)) > real(1e4);
        fa[0] = s_ * d[0];
        fa[1] = s_ * d[1];
        fa[2] = s_ * d[2];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        acc_add_raw(acc + 6 * (size_t)sa + k, fa[k]);
        acc_add_raw(acc + 6 * (size_t)sb + k, -fa[k]);
    }
}

// the separation of the pair (sa, sb) in replica R: d = x_a - x_b (minimum image), returns |d|^2
template <class real>
__device__ __forceinline__ real pair_sep(const ForceArgs<real> &a, const Replica<real> &R, int sa, int sb, real d[3],
                                         real xa[4], real xb[4]) {
    load4(a.buf.pos + 4 * (size_t)sa, xa);
    load4(a.buf.pos + 4 * (size_t)sb, xb);
    d[0] = min_image_sep<real>(xa[0], xb[0], R.box, R.box_lo, R.l2s, R.periodic);
    d[1] = min_image_sep<real>(xa[1], xb[1], R.box, R.box_lo, R.l2s, R.periodic);
    d[2] = min_image_sep<real>(xa[2], xb[2], R.box, R.box_lo, R.l2s, R.periodic);
    return sep_r2<real>(d[0], d[1], d[2]);
}

// wca: null evaluates the WCA core here; else *wca tells whether the pair needs it, for the caller to
// evaluate later (wca_core)
template <class real, int KIND>
__device__ __forceinline__ void pair_core(const ForceArgs<real> &a, int sa, int sb, typename PairAcc<real>::type *acc,
                                          int2 *lbuf, int *lnb, int2 *list, long long list_cap,
                                          unsigned long long *lcounts, unsigned lflag, bool &big, int rhint = -1,
                                          bool *wca = nullptr) {
    constexpr bool BIND = KIND == kPairBind;
    const int r = rhint >= 0 ? rhint : (a.tb.uniform ? 0 : replica_of(a.tb, sa));
    const Replica<real> &R = a.tb.reps[r];
    real xa[4], xb[4], d[3];
    const real r2 = pair_sep<real>(a, R, sa, sb, d, xa, xb);
    if (!(r2 < R.rc2)) return;  // skin lists hold pairs up to the list range
    const real rr = sqrt_r(r2);
    // the WCA core (patch terms come from the pair lists' kernels)
    const bool core = rr < R.hs_limit && (a.parts & 1);
    if (wca) *wca = core;
    else if (core) wca_core<real>(a, R, sa, sb, d, r2, acc, big);
    if (BIND) {
        // along d = x_a - x_b: a's cosines are -(n_a . d) / r and b's (n_b . d) / r in either canonical order
        const Model<real> &M = a.tb.models[R.model];
        const int ida = __ldg(a.buf.ident + sa), idb = __ldg(a.buf.ident + sb);
        const bool single = M.n_types == 1;
        const int tya = single ? 0 : type_of<real>(M, ida - R.off), tyb = single ? 0 : type_of<real>(M, idb - R.off);
        if (M.np[tya] > 0 && M.np[tyb] > 0) {
            const real inv = real(1) / sqrt_r(r2), pre = M.mincos[tya][tyb] - real(4e-5);
            real Q[9], w[3];
            load_q(a, sa, xa[3], Q);
#pragma unroll
            for (int k = 0; k < 3; k++) w[k] = (Q[3 * k] * d[0] + Q[3 * k + 1] * d[1] + Q[3 * k + 2] * d[2]) * inv;
            if (cone_any<real>(M, tya, w, pre, real(-1))) {
                load_q(a, sb, xb[3], Q);
#pragma unroll
                for (int k = 0; k < 3; k++) w[k] = (Q[3 * k] * d[0] + Q[3 * k + 1] * d[1] + Q[3 * k + 2] * d[2]) * inv;
                if (cone_any<real>(M, tyb, w, pre, real(1)))
                    block_list_put(lbuf, lnb, ida < idb ? make_int2(sa, sb) : make_int2(sb, sa), list, lcounts,
                                   list_cap, a.flags, lflag);
            }
        }
    }
    if (KIND == kPairSplit && (a.parts & 2) && r2 < R.patch_r2) {
        // the one-sided tests of both particles along d = x_a - x_b (with the 1e-5 margin of the full
        // kernel's own early test): a's cosines -(n . Qa d) / r, b's (n . Qb d) / r
        const Model<real> &M = a.tb.models[R.model];
        const int ida = __ldg(a.buf.ident + sa);
        const int tya = M.n_types == 1 ? 0 : type_of<real>(M, ida - R.off);
        if (M.np[tya] > 0) {
            const real inv = real(1) / sqrt_r(r2);
            real Q[9], w[3];
            load_q(a, sa, xa[3], Q);
#pragma unroll
            for (int k = 0; k < 3; k++) w[k] = (Q[3 * k] * d[0] + Q[3 * k + 1] * d[1] + Q[3 * k + 2] * d[2]) * inv;
            const bool any = cone_any<real>(M, tya, w, M.mincos_any[tya] - real(1e-5), real(-1));
            if (any) {
                const int idb = __ldg(a.buf.ident + sb);
                const int tyb = M.n_types == 1 ? 0 : type_of<real>(M, idb - R.off);
                if (M.np[tyb] > 0) {
                    load_q(a, sb, xb[3], Q);
#pragma unroll
                    for (int k = 0; k < 3; k++)
                        w[k] = (Q[3 * k] * d[0] + Q[3 * k + 1] * d[1] + Q[3 * k + 2] * d[2]) * inv;
                    const bool anyb = cone_any<real>(M, tyb, w, M.mincos_any[tyb] - real(1e-5), real(1));
                    if (anyb) block_list_put(lbuf, lnb, make_int2(sa, sb), list, lcounts, list_cap, a.flags, lflag);
                }
            }
        }
    }
}

template <class real, int KIND>
__global__ void __launch_bounds__(kPipeThreads, 4) pairforce_kernel(ForceArgs<real> a, const int2 *pairs,
                                                                 const unsigned long long *npairs, long long cap,
                                                                 typename PairAcc<real>::type *acc,
                                                                 int2 *list = nullptr, long long list_cap = 0,
                                                                 unsigned long long *list_counts = nullptr) {
    constexpr bool BIND = KIND == kPairBind;
    __shared__ int2 lbuf[kBlockListCap];
    __shared__ int lnb;
    __shared__ unsigned long long lbase;
    if (threadIdx.x == 0) lnb = 0;
    __syncthreads();
    unsigned long long *const lcounts = BIND ? a.bind_ctr + kSegPairs : list_counts;
    const unsigned lflag = BIND ? (kFlagBind | kBindWhyList) : 8u;
    const long long n = (long long)*npairs < cap ? (long long)*npairs : cap;
    const long long stride = (long long)gridDim.x * blockDim.x;
    bool big = false;
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int2 next = q < n ? __ldcs(pairs + q) : make_int2(0, 0);
    for (; q < n; q += stride) {
        const int2 pr = next;  // the next iteration's entry is loaded one iteration ahead
        if (q + stride < n) next = __ldcs(pairs + q + stride);
        pair_core<real, KIND>(a, pr.x, pr.y, acc, lbuf, &lnb, list, list_cap, lcounts, lflag, big);
    }
    if (big) atomicOr(a.flags, 2u);
    block_list_flush(lbuf, &lnb, &lbase, list, lcounts, list_cap, a.flags, lflag);
}

// the Kern-Frenkel terms of one listed pair (sa, sb) into both particles' sums: the full kernel's patch branch
template <class real>
__device__ __forceinline__ void patch_terms(const ForceArgs<real> &a, int sa, int sb, typename PairAcc<real>::type *acc) {
    const int r = a.tb.uniform ? 0 : replica_of(a.tb, sa);
    const Replica<real> &R = a.tb.reps[r];
    const Model<real> &M = a.tb.models[R.model];
    real xa[4], xb[4];
    load4(a.buf.pos + 4 * (size_t)sa, xa);
    load4(a.buf.pos + 4 * (size_t)sb, xb);
    const real d[3] = {min_image_sep<real>(xa[0], xb[0], R.box, R.box_lo, R.l2s, R.periodic),
                       min_image_sep<real>(xa[1], xb[1], R.box, R.box_lo, R.l2s, R.periodic),
                       min_image_sep<real>(xa[2], xb[2], R.box, R.box_lo, R.l2s, R.periodic)};
    const real rr = sqrt_r(sep_r2<real>(d[0], d[1], d[2]));
    const int ida = __ldg(a.buf.ident + sa), idb = __ldg(a.buf.ident + sb);
    const bool single = M.n_types == 1;
    const int tya = single ? 0 : type_of<real>(M, ida - R.off), tyb = single ? 0 : type_of<real>(M, idb - R.off);
    real Qa[9], Qb[9];
    load_q(a, sa, xa[3], Qa);
    load_q(a, sb, xb[3], Qb);
    const bool a_first = ida < idb;  // canonical order of the reference (p1 < p2)
    const real sg = a_first ? real(1) : real(-1), inv = real(1) / rr;
    const real u[3] = {sg * d[0] * inv, sg * d[1] * inv, sg * d[2] * inv};
    real f[3] = {real(0), real(0), real(0)}, t1[3] = {real(0), real(0), real(0)},
         t2[3] = {real(0), real(0), real(0)}, e = real(0);
    int nbond = 0;
    // the canonical first particle's rows and type by selects, not by a branch around two copies of the patch
    // code (each copy ran with the half of the lanes whose pairs had that order)
    real Q1[9], Q2[9];
#pragma unroll
    for (int k = 0; k < 9; k++) {
        Q1[k] = a_first ? Qa[k] : Qb[k];
        Q2[k] = a_first ? Qb[k] : Qa[k];
    }
    patch_pair<real>(M, a_first ? tya : tyb, a_first ? tyb : tya, Q1, Q2, u, rr, R.bond_r, f, t1, t2, e, nbond);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        fixed_add(acc + 6 * (size_t)sa + k, sg * f[k]);
        fixed_add(acc + 6 * (size_t)sb + k, -sg * f[k]);
        fixed_add(acc + 6 * (size_t)sa + 3 + k, a_first ? t1[k] : t2[k]);
        fixed_add(acc + 6 * (size_t)sb + 3 + k, a_first ? t2[k] : t1[k]);
    }
}

// range_list: use the replica's list range (skin lists) instead of its force range.
// Each lane scans its particle's candidate segments (scan_segment): chunks of at most 32 slots whose hits are
// marked in a bit mask and appended by the warp together to its own part of the block buffer (warp_append), so
// the candidate loop carries no appends and no shared-memory atomics.  Warps whose lanes all sit in grids of
// three or more cells per side take the five rows of the forward half-stencil unrolled (row offsets and image
// shifts known at compile time, the shifts taken out of the candidate loop); warps with a lane in a smaller grid
// take the general row loop.
//
// STAGE kPairSplit or kPairBind (no list reuse: every step rebuilds): the pairs do not go to the list at all
// (FUSED).  After its scan each
// warp takes its own buffered pairs, one per lane, through pair_core (WCA core, cone pre-test, patch list)
// while their positions are still in L1; only pairs beyond a warp's part reach the HBM list, for
// pairforce_kernel.
// FP32 register budgets: the fused form at 48 (five 256-thread blocks per SM; its natural 64 allow four,
// measured 8% slower), the search alone at 40 (six blocks).  FP64 keeps its natural count (no spills).
template <class real, int THREADS, int STAGE, bool FUSED = STAGE != 0>
__global__ void __launch_bounds__(THREADS, sizeof(real) == 4 ? (FUSED ? 1280 : 1536) / THREADS : 1)
    pairfind_kernel(ForceArgs<real> a, int2 *pairs,
                                                           unsigned long long *npairs, long long cap,
                                                           int range_list, const int *gate,
                                                           typename PairAcc<real>::type *acc = nullptr,
                                                           int2 *list = nullptr, long long list_cap = 0,
                                                           unsigned long long *list_counts = nullptr) {
    if (gated_off(gate, 1)) return;
    constexpr int kLBuf = FUSED ? kBlockListCap : 1;
    __shared__ int2 buf[kWarpPairs * (THREADS / 32)];
    __shared__ int2 lbuf[kLBuf];
    __shared__ int lnb;
    __shared__ unsigned long long lbase;
    if constexpr (FUSED) {
        if (threadIdx.x == 0) lnb = 0;
        __syncthreads();
    }
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int2 *const part = buf + kWarpPairs * (threadIdx.x >> 5);
    int cnt = 0;   // the warp's pairs (the same in every lane)
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = s < a.tb.ntot;
    int r = 0;
    if (valid) r = replica_of(a.tb, s);
    const Replica<real> &R = a.tb.reps[r];
    const real range2 = range_list ? R.rc2_list_find : R.rc2_find;   // a superset: the pair kernels re-test
    const int nc = R.nc;
    int key = valid ? a.buf.home_cell[s] - R.cell_off : 0;
    if (key < 0 || key >= nc * nc * nc) {
        atomicOr(a.flags, 16u);
        key = 0;
    }
    const int q1 = div_nc(R, key), cz = div_nc(R, q1);
    const int cx = key - q1 * nc, cy = q1 - cz * nc;
    real pi[3] = {real(0), real(0), real(0)};
    if (valid) load_pos(a.buf.pos + 4 * (size_t)s, pi[0], pi[1], pi[2]);
    const real L = R.box;
    const int periodic = R.periodic;
    // Each unordered pair once.  With three or more cells per side: the forward half of the stencil
    // (rows (dy, dz) = (0, 0) [cells x, x + 1], (1, 0), (-1..1, 1) [cells x - 1 .. x + 1]) -- an offset
    // and its negative are distinct cells, so exactly one of the two particles' scans holds the
    // other -- and in the own cell only the later slots.  Smaller grids: every cell, later slots.
    // pairfind runs right after a sort, so every particle lies in its cell: a neighbour cell reached across a
    // periodic face holds coordinates one box length away (image shift).
    const bool small = nc < 3;
    if (!__any_sync(full, valid && small)) {
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const int dy = k == 0 ? 0 : (k == 1 ? 1 : k - 3), dz = k <= 1 ? 0 : 1;
            int zz = cz + dz, yy = cy + dy;
            real shz = real(0), shy = real(0), shb = real(0);
            bool skip = !valid;
            if (dz > 0 && zz >= nc) {
                skip |= !periodic;
                shz = L;
                zz -= nc;
            }
            if (dy < 0 && yy < 0) {
                skip |= !periodic;
                shy = -L;
                yy += nc;
            } else if (dy > 0 && yy >= nc) {
                skip |= !periodic;
                shy = L;
                yy -= nc;
            }
            // the x cells of the row as at most two contiguous slot segments: [a0, a1) unshifted and one
            // wrapped cell [b0, b1) (image shift shb)
            int a0 = 0, a1 = 0, b0 = 0, b1 = 0;
            if (!skip) {
                const int row = R.cell_off + nc * (yy + nc * zz);
                const int x0 = k == 0 ? cx : cx - 1, x1 = cx + 1;  // the own row starts at the own cell
                a0 = __ldg(a.start + row + (x0 < 0 ? 0 : x0));
                a1 = __ldg(a.start + row + (x1 >= nc ? nc : x1 + 1));
                if (periodic) {
                    if (x0 < 0) {
                        b0 = __ldg(a.start + row + nc - 1);
                        b1 = __ldg(a.start + row + nc);
                        shb = -L;
                    } else if (x1 >= nc) {
                        b0 = __ldg(a.start + row);
                        b1 = __ldg(a.start + row + 1);
                        shb = L;
                    }
                }
                // only the own cell filters by slot; the wrapped cell of the own row is a forward neighbour
                // whose slots may lie below s
                if (k == 0 && a0 <= s) a0 = s + 1;
            }
            const real qy = pi[1] - shy, qz = pi[2] - shz;
            scan_segment<real>(a.buf.pos, a0, a1, pi[0], qy, qz, range2, part, cnt, s, pairs, npairs, cap, a.flags);
            scan_segment<real>(a.buf.pos, b0, b1, pi[0] - shb, qy, qz, range2, part, cnt, s, pairs, npairs, cap,
                               a.flags);
        }
    } else {
        const int nrows = !valid ? 0 : (small ? 9 : 5);
        const int nrows_warp = __any_sync(full, nrows == 9) ? 9 : 5;
        for (int rr = 0; rr < nrows_warp; rr++) {  // warp-uniform; rows past a lane's nrows are empty
            int a0 = 0, a1 = 0, b0 = 0, b1 = 0;
            real shz = real(0), shy = real(0), shb = real(0);
            if (rr < nrows) {
                int dy, dz;
                if (small) {
                    dy = rr % 3;
                    dz = rr / 3;
                } else {
                    dy = rr == 0 ? 0 : (rr == 1 ? 1 : rr - 3);
                    dz = rr <= 1 ? 0 : 1;
                }
                int zz = small ? dz : cz + dz, yy = small ? dy : cy + dy;
                bool skip = small && (dy >= nc || dz >= nc);
                if (zz >= nc) {
                    skip |= !periodic;
                    shz = L;
                    zz -= nc;
                }
                if (yy < 0 || yy >= nc) {
                    skip |= !periodic;
                    shy = yy < 0 ? -L : L;
                    yy = yy < 0 ? yy + nc : yy - nc;
                }
                if (!skip) {
                    const int row = R.cell_off + nc * (yy + nc * zz);
                    if (small) {
                        a0 = __ldg(a.start + row);
                        a1 = __ldg(a.start + row + nc);
                    } else {
                        const int x0 = rr == 0 ? cx : cx - 1, x1 = cx + 1;
                        a0 = __ldg(a.start + row + (x0 < 0 ? 0 : x0));
                        a1 = __ldg(a.start + row + (x1 >= nc ? nc : x1 + 1));
                        if (periodic) {
                            if (x0 < 0) {
                                b0 = __ldg(a.start + row + nc - 1);
                                b1 = __ldg(a.start + row + nc);
                                shb = -L;
                            } else if (x1 >= nc) {
                                b0 = __ldg(a.start + row);
                                b1 = __ldg(a.start + row + 1);
                                shb = L;
                            }
                        }
                    }
                    if ((small || rr == 0) && a0 <= s) a0 = s + 1;
                }
            }
            for (int seg = 0; seg < 2; seg++) {
                const int t0 = seg ? b0 : a0, t1 = seg ? b1 : a1;
                for (int c0 = t0; __any_sync(full, c0 < t1); c0 += 32) {
                    unsigned mask = 0u;
                    const int ce = t1 < c0 + 32 ? t1 : c0 + 32;
#pragma unroll 1
                    for (int t = c0; t < ce; t++) {
                        real pj[3];
                        load_pos(a.buf.pos + 4 * (size_t)t, pj[0], pj[1], pj[2]);
                        real dx, dy2, dz2;
                        if (small) {   // tiny grids: no cell geometry to lean on
                            dx = min_image_sep<real>(pi[0], pj[0], R.box, R.box_lo, R.l2s, periodic);
                            dy2 = min_image_sep<real>(pi[1], pj[1], R.box, R.box_lo, R.l2s, periodic);
                            dz2 = min_image_sep<real>(pi[2], pj[2], R.box, R.box_lo, R.l2s, periodic);
                        } else {
                            dx = (pi[0] - (seg ? shb : real(0))) - pj[0];
                            dy2 = (pi[1] - shy) - pj[1];
                            dz2 = (pi[2] - shz) - pj[2];
                        }
                        if (find_r2(dx, dy2, dz2) < range2) mask |= 1u << (t - c0);
                    }
                    warp_append(part, cnt, s, c0, mask, pairs, npairs, cap, a.flags);
                }
            }
        }
    }
    __syncwarp();
    const int n = cnt < kWarpPairs ? cnt : kWarpPairs;
    if constexpr (FUSED) {
        // the warp's pairs (s, t) have s among its own slots: when those lie in one replica, so do all of them
        const int r0 = __shfl_sync(full, r, 0);
        const int rhint = __all_sync(full, !valid || r == r0) && __shfl_sync(full, valid, 0) ? r0 : -1;
        // kPairBind (single-bond mode, a bond-deciding pass): the listed pairs go to the bond pass's segments
        unsigned long long *const lcounts = STAGE == kPairBind ? a.bind_ctr + kSegPairs : list_counts;
        const unsigned lflag = STAGE == kPairBind ? (kFlagBind | kBindWhyList) : 8u;
        bool big = false;
        constexpr int K = STAGE == kPairBind ? kPairBind : kPairSplit;
        if constexpr (sizeof(real) == 4 && K == kPairBind) {
            // FP32 bond-deciding passes (pairs out to max_check): the pairs inside the WCA range (about one in
            // eight) are taken out first and their float-float core evaluated afterwards with every lane on one,
            // instead of by the few lanes of each round that have one while the rest wait: 2.04 -> 2.02 ms a
            // step.  (In the force pass, whose pairs reach only the force range, it measured 0.5% slower.)  They
            // are compacted into the front of the warp's own part: a round's entries are in registers before
            // the __syncwarp, and the writes stay below the round's end.
            int nw = 0;
            for (int base = 0; base < n; base += 32) {
                const int i = base + lane;
                int2 pr = make_int2(0, 0);
                bool w = false;
                if (i < n) {
                    pr = part[i];
                    pair_core<real, K>(a, pr.x, pr.y, acc, lbuf, &lnb, list, list_cap, lcounts, lflag, big, rhint,
                                       &w);
                }
                const unsigned m = __ballot_sync(full, w);
                __syncwarp();
                if (w) part[nw + __popc(m & ((1u << lane) - 1u))] = pr;
                nw += __popc(m);
                __syncwarp();
            }
            for (int j = lane; j < nw; j += 32) {
                const int2 pr = part[j];
                const int r1 = rhint >= 0 ? rhint : (a.tb.uniform ? 0 : replica_of(a.tb, pr.x));
                const Replica<real> &R = a.tb.reps[r1];
                real xa[4], xb[4], d[3];
                const real r2 = pair_sep<real>(a, R, pr.x, pr.y, d, xa, xb);
                wca_core<real>(a, R, pr.x, pr.y, d, r2, acc, big);
            }
        } else {
            for (int i = lane; i < n; i += 32)
                pair_core<real, K>(a, part[i].x, part[i].y, acc, lbuf, &lnb, list, list_cap, lcounts, lflag, big, rhint);
        }
        if (big) atomicOr(a.flags, 2u);
        block_list_flush(lbuf, &lnb, &lbase, list, lcounts, list_cap, a.flags, lflag);
        return;
    }
    // one list reservation per block (a single counter serves the whole grid): the warps' counts, then each
    // warp copies its part after the parts of the warps before it
    __shared__ int wcount[THREADS / 32];
    if (lane == 0) wcount[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < THREADS / 32; w++) tot += wcount[w];
        lbase = tot ? atomicAdd(npairs, (unsigned long long)tot) : 0ull;
    }
    int before = 0;
    for (int w = 0; w < (int)(threadIdx.x >> 5); w++) before += wcount[w];
    __syncthreads();
    const unsigned long long base = lbase + (unsigned long long)before;
    for (int i = lane; i < n; i += 32) {
        if ((long long)(base + i) < cap) pairs[base + i] = part[i];
        else atomicOr(a.flags, 8u);
    }
}

// the Kern-Frenkel terms of the pairs pairforce_kernel<kPairSplit> listed, one pair per thread, into the
// fixed-point sums of both particles (the same evaluation as the full kernel's patch branch); capped at 64
// registers (four blocks per SM), measured a little faster than its natural 80
template <class real>
__global__ void __launch_bounds__(kPipeThreads, 4) patch_pairs_kernel(ForceArgs<real> a, const int2 *list_all,
                                                                    long long cap, const unsigned long long *counts,
                                                                    typename PairAcc<real>::type *acc) {
    __shared__ long long segs[kSegs + 1];
    seg_prefix(counts, cap, segs);
    const long long n = segs[kSegs];
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int2 pr = list_all[seg_slot(segs, cap, q)];
        patch_terms<real>(a, pr.x, pr.y, acc);
    }
}

// single-bond mode, a bond-deciding pass: this update's edges of the pairs pairforce_kernel<kPairBind> listed
// (canonical order, both particles with a patch near a cone), one pair per thread, in float
// (bind_patch_edge_f; bind_recheck_kernel takes the patch pairs within a margin): every listed pair has passed
// the cone pre-test, so the lanes of a warp run the patch-pair loop together and overlap the bond-state,
// snapshot and adjacency accesses of their pairs.  Four blocks per SM (64 registers): the kernel waits on
// dependent loads and atomics, and more resident warps hide more of that.
__global__ void __launch_bounds__(kPipeThreads, 4) bind_pairs_kernel(ForceArgs<float> a, const int2 *list_all,
                                                                   long long cap) {
    __shared__ long long segs[kSegs + 1];
    seg_prefix(a.bind_ctr + kSegPairs, cap, segs);
    const long long n = segs[kSegs];
    const unsigned stamp = (unsigned)a.bind_ctr[2];
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int2 pr = list_all[seg_slot(segs, cap, q)];
        const int s1 = pr.x, s2 = pr.y;
        const int r = replica_of(a.tb, s1);
        const Replica<float> &R = a.tb.reps[r];
        const BindRep &B = a.bind_reps[r];
        const Model<float> &M = a.tb.models[R.model];
        // both particles' rows and indices are read before any is used: the pair waits on memory once
        float x1[4], x2[4], Q1[9], Q2[9];
        load4(a.buf.pos + 4 * (size_t)s1, x1);
        load4(a.buf.pos + 4 * (size_t)s2, x2);
        load_q(a, s1, 0.f, Q1);
        load_q(a, s2, 0.f, Q2);
        const int id1 = __ldg(a.buf.ident + s1), id2 = __ldg(a.buf.ident + s2);
        Q1[8] = x1[3];
        Q2[8] = x2[3];
        const float d[3] = {min_image_sep<float>(x1[0], x2[0], R.box, R.box_lo, R.l2s, R.periodic),
                            min_image_sep<float>(x1[1], x2[1], R.box, R.box_lo, R.l2s, R.periodic),
                            min_image_sep<float>(x1[2], x2[2], R.box, R.box_lo, R.l2s, R.periodic)};
        const float r2 = sep_r2(d[0], d[1], d[2]);
        const int t0 = side_of<float>(r2, B.mk2_lo, B.mk2_hi);
        if (t0 > 0) continue;
        const int li1 = id1 - R.off, li2 = id2 - R.off;
        const int ty1 = type_of<float>(M, li1), ty2 = type_of<float>(M, li2);
        const float rr = sqrtf(r2), u[3] = {d[0] / rr, d[1] / rr, d[2] / rr};
        float w1[3], w2[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            w1[k] = Q1[3 * k] * u[0] + Q1[3 * k + 1] * u[1] + Q1[3 * k + 2] * u[2];
            w2[k] = Q2[3 * k] * u[0] + Q2[3 * k + 1] * u[1] + Q2[3 * k + 2] * u[2];
        }
        const float pre = M.mincos[ty1][ty2] - 4e-5f;
        // the patches of each particle near a cone, as masks; the combinations are then taken in mask order,
        // so that every lane of a warp handles its first combination in the same round (usually the only one)
        // and the warp waits on the edge's memory accesses once, not once per combination some lane has
        const int na = M.np[ty1], nb = M.np[ty2];
        unsigned m1 = 0u, m2 = 0u;
        for (int k = 0; k < na; k++) {
            const float *v = M.orient[M.ooff[ty1] + k];
            if (-(v[0] * w1[0] + v[1] * w1[1] + v[2] * w1[2]) > pre) m1 |= 1u << k;
        }
        for (int k = 0; k < nb; k++) {
            const float *v = M.orient[M.ooff[ty2] + k];
            if (v[0] * w2[0] + v[1] * w2[1] + v[2] * w2[2] > pre) m2 |= 1u << k;
        }
        if (!m2) m1 = 0u;
        for (; m1; m1 &= m1 - 1u) {
            const int ka = __ffs(m1) - 1;
            const float *va = M.orient[M.ooff[ty1] + ka];
            const float c1 = -(va[0] * w1[0] + va[1] * w1[1] + va[2] * w1[2]);
            for (unsigned mb = m2; mb; mb &= mb - 1u) {
                const int kb = __ffs(mb) - 1;
                const float *vb = M.orient[M.ooff[ty2] + kb];
                const float c2 = vb[0] * w2[0] + vb[1] * w2[1] + vb[2] * w2[2];
                bind_patch_edge_f(a, B, R, M, li1, li2, ty1, ty2, ka, kb, c1, c2, rr, t0, stamp);
            }
        }
    }
}

// single-bond mode, after bind_pairs_kernel: the patch pairs whose float tests fell within a margin, one per
// thread, through bind_patch_edge (the FP64 edge and candidate tests where the float ones are not clear).  The
// margins are a few 1e-5 wide, so the list is short: of the order of one patch pair per thousand tested.
__global__ void __launch_bounds__(kPipeThreads) bind_recheck_kernel(ForceArgs<float> a) {
    __shared__ long long segs[kSegs + 1];
    seg_prefix(a.bind_ctr + kSegRecheck, a.bind_rcap, segs);
    const long long n = segs[kSegs];
    const unsigned stamp = (unsigned)a.bind_ctr[2];
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int2 e = a.bind_recheck[seg_slot(segs, a.bind_rcap, q)];
        const int r = patch_replica(a.bind_reps, a.tb.nrep, e.x);
        const Replica<float> &R = a.tb.reps[r];
        const BindRep &B = a.bind_reps[r];
        const Model<float> &M = a.tb.models[R.model];
        int li1, ty1, ka, li2, ty2, kb;
        patch_owner<float>(B, M, e.x - B.patch_off, li1, ty1, ka);
        patch_owner<float>(B, M, e.y - B.patch_off, li2, ty2, kb);
        const int s1 = a.buf.slot_of[R.off + li1], s2 = a.buf.slot_of[R.off + li2];
        float x1[4], x2[4], Q[9], w1[3], w2[3];
        load4(a.buf.pos + 4 * (size_t)s1, x1);
        load4(a.buf.pos + 4 * (size_t)s2, x2);
        const float d[3] = {min_image_sep<float>(x1[0], x2[0], R.box, R.box_lo, R.l2s, R.periodic),
                            min_image_sep<float>(x1[1], x2[1], R.box, R.box_lo, R.l2s, R.periodic),
                            min_image_sep<float>(x1[2], x2[2], R.box, R.box_lo, R.l2s, R.periodic)};
        const float r2 = sep_r2(d[0], d[1], d[2]);
        const int t0 = side_of<float>(r2, B.mk2_lo, B.mk2_hi);
        const float rr = sqrtf(r2), u[3] = {d[0] / rr, d[1] / rr, d[2] / rr};
        load_q(a, s1, x1[3], Q);
#pragma unroll
        for (int k = 0; k < 3; k++) w1[k] = Q[3 * k] * u[0] + Q[3 * k + 1] * u[1] + Q[3 * k + 2] * u[2];
        load_q(a, s2, x2[3], Q);
#pragma unroll
        for (int k = 0; k < 3; k++) w2[k] = Q[3 * k] * u[0] + Q[3 * k + 1] * u[1] + Q[3 * k + 2] * u[2];
        const float *va = M.orient[M.ooff[ty1] + ka], *vb = M.orient[M.ooff[ty2] + kb];
        const float c1 = -(va[0] * w1[0] + va[1] * w1[1] + va[2] * w1[2]);
        const float c2 = vb[0] * w2[0] + vb[1] * w2[1] + vb[2] * w2[2];
        bind_patch_edge<float>(a, B, R, M, s1, s2, li1, li2, ty1, ty2, ka, kb, c1, c2, rr, t0, stamp);
    }
}

// single-bond mode, a bond-deciding pass: KernFrenkelOnePatch2::force_and_torque of every pair bound by this
// update's decisions (LangevinRforce.cpp:3940-4030), one thread per pair, into the fixed-point sums of both
// particles (the epilogue then leaves bound pairs alone)
__global__ void __launch_bounds__(kPipeThreads) bound_pairs_kernel(ForceArgs<float> a, const int2 *list_all,
                                                                 long long cap, long long *acc) {
    __shared__ long long segs[kSegs + 1];
    seg_prefix(a.bind_ctr + kSegBound, cap, segs);
    const long long n = segs[kSegs];
    {
        for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
            const int2 e = list_all[seg_slot(segs, cap, q)];
            const int rp = patch_replica(a.bind_reps, a.tb.nrep, e.x);
            const Replica<float> &R = a.tb.reps[rp];
            const BindRep &B = a.bind_reps[rp];
            const Model<float> &M = a.tb.models[R.model];
            int l1, t1, k1, l2, t2, k2;
            patch_owner<float>(B, M, e.x - B.patch_off, l1, t1, k1);
            patch_owner<float>(B, M, e.y - B.patch_off, l2, t2, k2);
            if (l2 < l1) {
                int t;
                t = l1; l1 = l2; l2 = t;
                t = t1; t1 = t2; t2 = t;
                t = k1; k1 = k2; k2 = t;
            }
            const int s1 = a.buf.slot_of[R.off + l1], s2 = a.buf.slot_of[R.off + l2];
            Payload<float> P1, P2;
            P1.load(a.buf.pos, a.buf.rota, a.buf.rotb, s1);
            P2.load(a.buf.pos, a.buf.rota, a.buf.rotb, s2);
            const float dx = min_image_sep<float>(P1.v[0], P2.v[0], R.box, R.box_lo, R.l2s, R.periodic);
            const float dy = min_image_sep<float>(P1.v[1], P2.v[1], R.box, R.box_lo, R.l2s, R.periodic);
            const float dz = min_image_sep<float>(P1.v[2], P2.v[2], R.box, R.box_lo, R.l2s, R.periodic);
            const float rr = sqrtf(dx * dx + dy * dy + dz * dz);
            const int qp = M.pstart[t1][t2] + k1 * M.np[t2] + k2;
            if (rr > M.rmax[qp]) continue;
            const float u[3] = {dx / rr, dy / rr, dz / rr};
            const float *b1 = M.orient[M.ooff[t1] + k1], *b2 = M.orient[M.ooff[t2] + k2];
            float n1[3], n2[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                n1[k] = b1[0] * P1.v[3 + k] + b1[1] * P1.v[6 + k] + b1[2] * P1.v[9 + k];
                n2[k] = b2[0] * P2.v[3 + k] + b2[1] * P2.v[6 + k] + b2[2] * P2.v[9 + k];
            }
            const float ci = -(n1[0] * u[0] + n1[1] * u[1] + n1[2] * u[2]);
            const float cj = n2[0] * u[0] + n2[1] * u[1] + n2[2] * u[2];
            if (!(ci > M.costm[qp] && cj > M.costm[qp])) continue;
            float f[3] = {0.f, 0.f, 0.f}, ta[3] = {0.f, 0.f, 0.f}, tb[3] = {0.f, 0.f, 0.f}, ee = 0.f;
            kf2_pair<float>(M.att[qp], M.dis[qp], M.inv_dis[qp], M.kfac[qp], u, rr, n1, n2, ci, cj, f, ta, tb, ee);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                fixed_add(acc + 6 * (size_t)s1 + k, f[k]);
                fixed_add(acc + 6 * (size_t)s2 + k, -f[k]);
                fixed_add(acc + 6 * (size_t)s1 + 3 + k, ta[k]);
                fixed_add(acc + 6 * (size_t)s2 + 3 + k, tb[k]);
            }
        }
    }
}

// per particle: the summed force and torque (cleared for the next pass), bonds, then the mode's output
// the six sums of a slot (F lab, T lab), read and cleared for the next pass: 48 B, 16-byte aligned
__device__ __forceinline__ void take_sums(long long *acc, size_t s, float F[3], float T[3]) {
    longlong2 *as = reinterpret_cast<longlong2 *>(acc + 6 * s);
    const longlong2 s0 = as[0], s1 = as[1], s2 = as[2];
    F[0] = from_fixed(s0.x); F[1] = from_fixed(s0.y); F[2] = from_fixed(s1.x);
    T[0] = from_fixed(s1.y); T[1] = from_fixed(s2.x); T[2] = from_fixed(s2.y);
    const longlong2 zero = make_longlong2(0, 0);
    as[0] = zero;
    as[1] = zero;
    as[2] = zero;
}
__device__ __forceinline__ void take_sums(double *acc, size_t s, double F[3], double T[3]) {
    double2 *as = reinterpret_cast<double2 *>(acc + 6 * s);
    const double2 s0 = as[0], s1 = as[1], s2 = as[2];
    F[0] = s0.x; F[1] = s0.y; F[2] = s1.x;
    T[0] = s1.y; T[1] = s2.x; T[2] = s2.y;
    const double2 zero = make_double2(0.0, 0.0);
    as[0] = zero;
    as[1] = zero;
    as[2] = zero;
}

template <class real, int MODE, int THREADS>
__global__ void __launch_bounds__(THREADS) pair_epilogue_kernel(ForceArgs<real> a, typename PairAcc<real>::type *acc) {
    {
        const int s = blockIdx.x * blockDim.x + threadIdx.x;  // one particle per thread: many loads in flight
        if (s >= a.tb.ntot) return;
        const int r = replica_of(a.tb, s);
        const Replica<real> &R = a.tb.reps[r];
        real F[3], T[3];
        take_sums(acc, (size_t)s, F, T);
        const int id = a.buf.ident[s];
        real xi[4];
        load4(a.buf.pos + 4 * (size_t)s, xi);
        if (a.bond_start && (a.parts & 1)) {
            real eb = real(0);
            bool big = false;
            bond_forces<real>(a, R, id, xi[0], xi[1], xi[2], F, eb, big);
            if (big) atomicOr(a.flags, 2u);
        }
        if (a.bind_on && !a.bind_listed && (a.parts & 2)) {
            Payload<real> P;
            P.load(a.buf.pos, a.buf.rota, a.buf.rotb, s);
            real eb = real(0);
            bound_patch_forces<real>(a, R, a.tb.models[R.model], r, id, P.v, F, T, eb);
        }
        if (MODE == kModeForces) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                a.outF[3 * (size_t)id + k] = F[k];
                a.outT[3 * (size_t)id + k] = T[k];
            }
        } else {
            real Qi[9];
            load_q(a, s, xi[3], Qi);
            langevin_epilogue<real>(a, R, r, s, id, F, T, Qi, xi[0], xi[1], xi[2]);
        }
    }
}

}  // namespace
}  // namespace mtg
