// mtg_tile.cuh -- the FP32 force/torque + Langevin kernel of the batched path, one CTA per tile of cells.
//
// A tile is a block of cells of one replica: whole x-rows (or a chunk of one) x ty x tz rows.  Per tile:
//   stage   the positions of the tile and its one-cell halo (16 B per particle) are copied into shared
//           memory by cp.async.bulk (TMA bulk copies, one per contiguous row piece) on an mbarrier;
//           the wait is bounded and latches MTG_FLAG_TIMEOUT instead of hanging
//   phase 1 one lane per home particle scans its 27 cells in shared memory; in-range pairs are
//           appended to the warp's pair list by ballot (warp-uniform loops, no atomics)
//   phase 2 all lanes take pairs evenly: WCA core and the home particle's cone test (2a); the pairs
//           that pass are compacted and take the neighbour's orientation, the body-frame cone tests
//           and the Kern-Frenkel force/torque of the in-cone patch potentials (2b)
//   phase 3 one lane per home particle: friction + Philox noise, half-kick, next-step binning
// Forces and torques are summed in 64-bit fixed point in shared memory (integer atomics commute), so
// the result does not depend on the order in which lanes or CTAs visit pairs.
#pragma once

#include "mtg_kernels.cuh"

namespace mtg {
namespace {  // internal linkage

constexpr int kTileThreads = 512;  // one persistent CTA per SM: 15 consumer warps + 1 producer warp
constexpr int kTileWarps = kTileThreads / 32;
constexpr int kConsumerWarps = kTileWarps - 1;
constexpr int kStageBufs = 3;      // ring of staging buffers: the producer runs up to two tiles ahead
constexpr int kTileYZMax = 4;
constexpr int kTileXMax = 32;
constexpr int kStageRows = (kTileYZMax + 2) * (kTileYZMax + 2);                   // 36
constexpr int kStageCells = (kTileXMax + 2) * kStageRows;                           // 1224
constexpr int kStartRowInts = 48;  // prefetched start[] entries of one staged row: run 40 + wrapped cell 8
constexpr int kStartRunInts = 40;
constexpr int kStageCap = 2048;    // staged particles per buffer
constexpr int kWarpPairCap = 640;  // in-range pairs per 32 home particles
constexpr unsigned kWaitSpins = 1u << 20;

// tile descriptor: x = replica | periodic << 30, y = x0 | y0 << 10 | z0 << 20,
// z = sx | ty << 10 | tz << 15 | whole << 20 | simple << 21 | nc << 22, w = the replica's first cell.
// sx = staged cells per row (nc for whole rows, tx + 2 for a chunk), tx = sx - 2 for chunks.

enum StageMode : int { kStaged = 0, kSlots = 1 };

// one staging buffer: a tile's positions (TMA-copied) and cell table, or -- for tiny replicas and tiles
// too crowded to stage -- just the slot ranges of its particles.  A staged particle k of staged cell c
// has global slot cell_lo[c] + (k - cell_sm[c]).
struct StageBuf {
    float4 pos[kStageCap];
    int cell_sm[kStageCells + 1];    // offset of every staged cell in pos[] (+ the total)
    int cell_lo[kStageCells];        // global slot of the first particle of every staged cell
    int row_start[kTileYZMax * kTileYZMax + 1];  // home particles before each home row
    int seg_s0[kTileYZMax * kTileYZMax], seg_n[kTileYZMax * kTileYZMax + 1];  // kSlots: slot runs
    unsigned long long bar;
    int4 desc;
    int mode, total, nhome, nseg;
    // units of the CTA-wide stream this buffer holds, published as ONE 64-bit word so a reader never
    // sees half of an update: bits 0-31 first unit, bits 32-62 unit count, bit 63 mbarrier parity
    unsigned long long range;
    int nunits;                      // unit count of the tile held (producer's copy)
    int done;                        // units of this tile finished by the consumers
};

// pair-list entry: staged particle k (bits 0-10), its staged cell (bits 11-21), home lane (22-26)
__device__ __forceinline__ unsigned pair_entry(int k, int cell, int lane) {
    return (unsigned)k | ((unsigned)cell << 11) | ((unsigned)lane << 22);
}
__device__ __forceinline__ int pair_k(unsigned e) { return (int)(e & 2047u); }
__device__ __forceinline__ int pair_cell(unsigned e) { return (int)((e >> 11) & 2047u); }
__device__ __forceinline__ int pair_h(unsigned e) { return (int)(e >> 22); }

// per-warp scratch: the compacted pair and task lists of 32 home particles and their sums
struct WarpScratch {
    unsigned long long acc[32][6];
    float4 h_qa[32], h_qb[32];       // home orientation rows (Q0..Q3, Q4..Q7); Q8 is pos.w
    int h_k[32], h_slot[32], h_id[32];
    unsigned pair[kWarpPairCap];
};

struct TileShared {
    StageBuf buf[kStageBufs];
    WarpScratch w[kConsumerWarps];
    // start[] entries of the next tiles, copied ahead by the producer (cp.async, 16-byte chunks): per
    // staged row the aligned chunks holding its run's starts and end, then those of its wrapped cell
    __align__(16) int start_rows[2][kStageRows * kStartRowInts];
    int claim;                       // next unit of the CTA-wide stream
    int final_units;                 // -1 until the producer has published its last tile
    int overflow;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
        "r"(bytes)
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

struct TileGeom {
    int rep, x0, y0, z0, sx, ty, tz, whole, simple, nc, periodic, cell_off;
};
__device__ __forceinline__ TileGeom decode_tile(int4 t) {
    TileGeom g;
    g.rep = t.x & 0x3fffffff;
    g.periodic = (t.x >> 30) & 1;
    g.nc = (t.z >> 22) & 1023;
    g.cell_off = t.w;
    g.x0 = t.y & 1023;
    g.y0 = (t.y >> 10) & 1023;
    g.z0 = (t.y >> 20) & 1023;
    g.sx = t.z & 1023;
    g.ty = (t.z >> 10) & 31;
    g.tz = (t.z >> 15) & 31;
    g.whole = (t.z >> 20) & 1;
    g.simple = (t.z >> 21) & 1;
    return g;
}

__device__ __forceinline__ void acc_add(unsigned long long *a, float v) {
    atomicAdd(a, (unsigned long long)to_fixed(v));
}
__device__ __forceinline__ float acc_get(unsigned long long a) { return from_fixed((long long)a); }

// the Langevin epilogue shared with the simple kernel (create_forces_and_torques_sphere + half-kick +
// binning of the next step); F, T are the lab-frame force and torque of slot s
template <class real>
__device__ __forceinline__ void langevin_epilogue(const ForceArgs<real> &a, const Replica<real> &R, int r, int s, int id,
                                                  const real F[3], const real T[3], const real Qi[9], real xi,
                                                  real yi, real zi) {
    Row<real> Mv;
    Mv.load(a.buf.motion + (size_t)s * kRow);
    real p[3] = {Mv.v[0], Mv.v[1], Mv.v[2]}, L[3] = {Mv.v[3], Mv.v[4], Mv.v[5]};
    real xi6[6];
    const int li = id - R.off;
    if (a.ext_noise) {
#pragma unroll
        for (int k = 0; k < 6; k++) xi6[k] = (real)a.ext_noise[6 * (size_t)id + k];
    } else {
        philox_noise6<real>((uint32_t)li, (uint32_t)r, a.draw[0], R.seed_lo, R.seed_hi, xi6);
    }
    real pb[3], fb[3], Ft[3], Tt[3];
#pragma unroll
    for (int k = 0; k < 3; k++) pb[k] = Qi[3 * k] * p[0] + Qi[3 * k + 1] * p[1] + Qi[3 * k + 2] * p[2];
#pragma unroll
    for (int k = 0; k < 3; k++) fb[k] = R.fric_t * pb[k] + R.Rt * xi6[k];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        Ft[k] = F[k] + fb[0] * Qi[k] + fb[1] * Qi[3 + k] + fb[2] * Qi[6 + k];
        Tt[k] = R.fric_r * L[k] + R.Rr * xi6[3 + k] + T[0] * Qi[3 * k] + T[1] * Qi[3 * k + 1] + T[2] * Qi[3 * k + 2];
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

__device__ __forceinline__ void load_q(const ForceArgs<float> &a, int slot, float q8, float Q[9]) {
    float b[4], c[4];
    load4(a.buf.rota + 4 * (size_t)slot, b);
    load4(a.buf.rotb + 4 * (size_t)slot, c);
    Q[0] = b[0]; Q[1] = b[1]; Q[2] = b[2]; Q[3] = b[3];
    Q[4] = c[0]; Q[5] = c[1]; Q[6] = c[2]; Q[7] = c[3]; Q[8] = q8;
}

__device__ __forceinline__ void home_q(const WarpScratch &W, int h, float q8, float Q[9]) {
    const float4 b = W.h_qa[h], c = W.h_qb[h];
    Q[0] = b.x; Q[1] = b.y; Q[2] = b.z; Q[3] = b.w;
    Q[4] = c.x; Q[5] = c.y; Q[6] = c.z; Q[7] = c.w; Q[8] = q8;
}

// Kern-Frenkel force and torques of patch potential q between patch rows oa (of the pair's first
// particle a) and ob (of b); u = (x_a - x_b) / r.  Adds the force on the home particle (a when i_first)
// and the torque on it to f and t.
__device__ __forceinline__ void kf2_potential(const Model<float> &M, int q, int oa, int ob, const float *Qa,
                                              const float *Qb, const float u[3], float rr, bool i_first, float f[3],
                                              float t[3]) {
    const float *b1 = M.orient[oa], *b2 = M.orient[ob];
    float n1[3], n2[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        n1[k] = b1[0] * Qa[k] + b1[1] * Qa[3 + k] + b1[2] * Qa[6 + k];
        n2[k] = b2[0] * Qb[k] + b2[1] * Qb[3 + k] + b2[2] * Qb[6 + k];
    }
    // the cone test already passed in the body frame; the lab-frame cosines feed the force
    const float cos1 = -(n1[0] * u[0] + n1[1] * u[1] + n1[2] * u[2]);
    const float cos2 = n2[0] * u[0] + n2[1] * u[1] + n2[2] * u[2];
    float fk[3] = {0, 0, 0}, tqa[3] = {0, 0, 0}, tqb[3] = {0, 0, 0}, en = 0;
    kf2_pair<float>(M.att[q], M.dis[q], M.inv_dis[q], M.kfac[q], u, rr, n1, n2, cos1, cos2, fk, tqa, tqb, en);
    const float sg = i_first ? 1.f : -1.f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        f[k] += sg * fk[k];
        t[k] += i_first ? tqa[k] : tqb[k];
    }
}

// separation x_home - x_neighbour of pair entry e (minimum image)
__device__ __forceinline__ void pair_sep(const Replica<float> &R, const StageBuf &B, const WarpScratch &W, unsigned e,
                                         float4 &pi, float4 &pj, float d[3]) {
    pi = B.pos[W.h_k[pair_h(e)]];
    pj = B.pos[pair_k(e)];
    d[0] = min_image_sep<float>(pi.x, pj.x, R.box, R.box_lo, R.l2s, R.periodic);
    d[1] = min_image_sep<float>(pi.y, pj.y, R.box, R.box_lo, R.l2s, R.periodic);
    d[2] = min_image_sep<float>(pi.z, pj.z, R.box, R.box_lo, R.l2s, R.periodic);
}

// phase 2a body: WCA core of pair entry e, then the home particle's own cone test from data in shared
// memory.  Its cosines are -(n . Qi (d / r)) in either order of the pair (the ones phase 2b tests up to
// rounding, hence the 1e-5 margin), so a pair none of whose home patches is within the widest cone of
// the home type has no patch potential.  Returns whether the pair goes on to phase 2b.
__device__ __forceinline__ bool pair_core(const Replica<float> &R, const Model<float> &M, const StageBuf &B,
                                          WarpScratch &W, unsigned e, bool &big) {
    const int h = pair_h(e);
    float4 pi, pj;
    float d[3];
    pair_sep(R, B, W, e, pi, pj, d);
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float rr = sqrtf(r2);
    if (rr < R.hs_limit) {
        const float s_ = hs_force_over_r<float>(R, r2);
        big |= fabsf(s_ * rr) > 1e4f;
        unsigned long long *acc = W.acc[h];
        acc_add(acc + 0, s_ * d[0]);
        acc_add(acc + 1, s_ * d[1]);
        acc_add(acc + 2, s_ * d[2]);
    }
    if (!(r2 < R.patch_r2)) return false;
    const int ti = M.n_types == 1 ? 0 : type_of<float>(M, W.h_id[h] - R.off);
    const int nph = M.np[ti];
    if (nph == 0) return false;
    const float inv = 1.f / rr;
    float Qi[9];
    home_q(W, h, pi.w, Qi);
    float w[3];
#pragma unroll
    for (int k = 0; k < 3; k++) w[k] = Qi[3 * k] * (d[0] * inv) + Qi[3 * k + 1] * (d[1] * inv) + Qi[3 * k + 2] * (d[2] * inv);
    const float mca = M.mincos_any[ti] - 1e-5f;
    const int oh = M.ooff[ti];
    bool any = false;
    for (int ia = 0; ia < nph; ia++) {
        const float *v = M.orient[oh + ia];
        any |= -(v[0] * w[0] + v[1] * w[1] + v[2] * w[2]) > mca;
    }
    return any;
}

// phase 2b body: body-frame cone tests and Kern-Frenkel potentials of pair entry e.  The first
// in-cone potential of the pair is evaluated after the cone loops, where the lanes of the warp that
// have one meet again; a pair rarely has a second (then it is evaluated in the loop).
__device__ __forceinline__ void pair_patches(const ForceArgs<float> &a, const Replica<float> &R, const Model<float> &M,
                                             const StageBuf &B, WarpScratch &W, unsigned e) {
    const int h = pair_h(e), kk = pair_k(e), cj = pair_cell(e);
    float4 pi, pj;
    float d[3];
    pair_sep(R, B, W, e, pi, pj, d);
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float rr = sqrtf(r2);
    const int j = B.cell_lo[cj] + (kk - B.cell_sm[cj]);
    const int idi = W.h_id[h];
    const int idj = __ldg(a.buf.ident + j);
    float Qj[9];
    load_q(a, j, pj.w, Qj);
    const bool single = M.n_types == 1;
    const int ti = single ? 0 : type_of<float>(M, idi - R.off);
    const int tj = single ? 0 : type_of<float>(M, idj - R.off);
    if (M.np[tj] == 0) return;
    const bool i_first = idi < idj;
    const float sg = i_first ? 1.f : -1.f, inv = 1.f / rr;
    const float u[3] = {sg * d[0] * inv, sg * d[1] * inv, sg * d[2] * inv};
    float Qi[9];
    home_q(W, h, pi.w, Qi);
    const float *Qa = i_first ? Qi : Qj, *Qb = i_first ? Qj : Qi;
    const int ta = i_first ? ti : tj, tb = i_first ? tj : ti;
    float wa[3], wb[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        wa[k] = Qa[3 * k] * u[0] + Qa[3 * k + 1] * u[1] + Qa[3 * k + 2] * u[2];
        wb[k] = Qb[3 * k] * u[0] + Qb[3 * k + 1] * u[1] + Qb[3 * k + 2] * u[2];
    }
    const int na = M.np[ta], nb = M.np[tb];
    const float mc = M.mincos[ta][tb];
    const int oa = M.ooff[ta], ob = M.ooff[tb], ps = M.pstart[ta][tb];
    unsigned maskb = 0;
    for (int jb = 0; jb < nb; jb++) {
        const float *v = M.orient[ob + jb];
        const float cb = v[0] * wb[0] + v[1] * wb[1] + v[2] * wb[2];
        if (cb > mc) maskb |= 1u << jb;
    }
    if (!maskb) return;
    float f[3] = {0.f, 0.f, 0.f}, t[3] = {0.f, 0.f, 0.f};
    int q1 = -1, ra = 0, rb = 0;
    for (int ia = 0; ia < na; ia++) {
        const float *v = M.orient[oa + ia];
        const float ca = -(v[0] * wa[0] + v[1] * wa[1] + v[2] * wa[2]);
        if (!(ca > mc)) continue;
        for (int jb = 0; jb < nb; jb++) {
            if (!((maskb >> jb) & 1u)) continue;
            const int q = ps + ia * nb + jb;
            const float *w = M.orient[ob + jb];
            const float cb = w[0] * wb[0] + w[1] * wb[1] + w[2] * wb[2];
            if (!(ca > M.costm[q] && cb > M.costm[q]) || rr > M.rmax[q]) continue;
            if (q1 < 0) {
                q1 = q;
                ra = oa + ia;
                rb = ob + jb;
            } else {
                kf2_potential(M, q, oa + ia, ob + jb, Qa, Qb, u, rr, i_first, f, t);
            }
        }
    }
    if (q1 < 0) return;
    kf2_potential(M, q1, ra, rb, Qa, Qb, u, rr, i_first, f, t);
    unsigned long long *acc = W.acc[h];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        acc_add(acc + k, f[k]);
        acc_add(acc + 3 + k, t[k]);
    }
}

// staged-cell wrap: the coordinates here are at most one cell outside [0, nc)
__device__ __forceinline__ int wrap1(int v, int nc) { return v < 0 ? v + nc : (v >= nc ? v - nc : v); }

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

// x layout of a tile's staged rows, the same for every row: this lane's cell (c = lane) and its global
// x, the unwrapped run [ru0, ru1) of consecutive global cells, and the wrapped cell wc (-1 if none)
struct RowLayout {
    int c, gx, ru0, ru1, wc, gx_end, gx_w;
    bool in_row, xok;
};
__device__ __forceinline__ RowLayout row_layout(const TileGeom &g, int lane) {
    RowLayout L;
    const int nc = g.nc, sx = g.sx;
    L.c = lane;
    L.in_row = lane < sx;
    L.gx = g.whole ? lane : g.x0 - 1 + lane;
    L.xok = L.in_row;
    if (L.gx < 0 || L.gx >= nc) {
        if (g.periodic) L.gx = L.gx < 0 ? L.gx + nc : L.gx - nc;
        else L.xok = false;
    }
    // a chunk that starts at x = 0 has its wrapped (or, walled, missing) cell first, one that ends at
    // the box's far side last; a chunk is at most nc - 2 cells wide, so only one end can wrap
    L.ru0 = 0;
    L.ru1 = sx;
    if (!g.whole) {
        if (g.x0 == 0) L.ru0 = 1;
        else if (g.x0 - 1 + sx > nc) L.ru1 = sx - 1;
    }
    L.wc = L.ru0 == 1 ? 0 : (L.ru1 < sx ? sx - 1 : -1);
    L.gx_end = g.whole ? L.ru1 - 1 : g.x0 - 1 + (L.ru1 - 1);  // last cell of the run (inside the box)
    L.gx_w = L.wc == 0 ? nc - 1 : 0;                          // the wrapped cell's global x
    return L;
}

// global index of staged plane sz's first cell, or -1 outside a walled box
__device__ __forceinline__ int plane_base(const TileGeom &g, int sz) {
    int gz = g.z0 - 1 + sz;
    if (gz < 0 || gz >= g.nc) {
        if (!g.periodic) return -1;
        gz = wrap1(gz, g.nc);
    }
    return g.cell_off + g.nc * g.nc * gz;
}
// global index of staged row sy's first cell (x = 0) in plane zb, or -1 outside a walled box
__device__ __forceinline__ int row_base(const TileGeom &g, int zb, int sy) {
    int gy = g.y0 - 1 + sy;
    if (gy < 0 || gy >= g.nc) {
        if (!g.periodic) return -1;
        gy = wrap1(gy, g.nc);
    }
    return zb < 0 ? -1 : zb + g.nc * gy;
}

// staged row r of a tile with nry rows per plane: (sy, sz) without a divide (r < 36, nry <= 6: the
// quotient (r + 0.5) / nry is at least 1 / 12 away from an integer)
__device__ __forceinline__ void row_yz(int r, int nry, float inv_nry, int &sy, int &sz) {
    sz = __float2int_rz(((float)r + 0.5f) * inv_nry);
    sy = r - sz * nry;
}

// Issue the copies of the start[] entries tile `desc` needs into P (cp.async, aligned 16-byte chunks,
// lanes over rows); the caller commits them as one group.  Row r of P (kStartRowInts entries): from
// entry 0 the chunks holding start[first run cell .. last run cell + 1] (the first at entry
// first & 3), from entry kStartRunInts the chunks holding start[wrapped cell], start[wrapped cell + 1]
// (the first at entry kStartRunInts + (wrapped cell & 3)).
__device__ void prefetch_starts(const ForceArgs<float> &a, const int4 desc, int *P, int lane) {
    const TileGeom g = decode_tile(desc);
    if (g.simple) return;
    const int nry = g.ty + 2, nrows = nry * (g.tz + 2);
    const float inv_nry = 1.f / (float)nry;
    const RowLayout L = row_layout(g, lane);  // the lane-independent parts (runs) are what is used here
    const int run_x0 = g.whole ? L.ru0 : g.x0 - 1 + L.ru0;
    const int nrun = L.ru1 - L.ru0;
    const bool wrapped = L.wc >= 0 && g.periodic;
    for (int r = lane; r < nrows; r += 32) {
        int sy, sz;
        row_yz(r, nry, inv_nry, sy, sz);
        const int rowg = row_base(g, plane_base(g, sz), sy);
        if (rowg < 0) continue;
        int *Pr = P + r * kStartRowInts;
        const int f = rowg + run_x0;
        const int c0 = f & ~3, c1 = (f + nrun + 1 + 3) & ~3;  // at most 10 chunks
        for (int c = c0; c < c1; c += 4) cp_async16(Pr + (c - c0), a.start + c);
        if (wrapped) {
            const int gw = rowg + L.gx_w;
            const int w0 = gw & ~3, w1 = (gw + 2 + 3) & ~3;  // at most 2 chunks
            for (int c = w0; c < w1; c += 4) cp_async16(Pr + kStartRunInts + (c - w0), a.start + c);
        }
    }
}

__device__ __forceinline__ int warp_inclusive_scan(int v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Producer warp: build buffer B's table for `tile` and start its bulk copies.  Returns the number of
// 32-particle units of the tile.
//   1  lanes over the flattened staged cells (row-major, x fastest): count and first global slot of
//      every cell, eight cells per lane in flight
//   2  one exclusive scan over the flattened counts (a chunk per lane + a warp scan) -> cell_sm
//   3  lanes over the staged rows: each row is one contiguous run of global slots (consecutive x
//      cells are consecutive in the sorted order) plus, for a chunk at the box edge, one wrapped
//      cell; every lane issues its rows' bulk copies.  Copies are issued only when the whole tile
//      fits, so the bytes the barrier expects are exactly the bytes copied.
__device__ int produce_tile(const ForceArgs<float> &a, const int4 desc, StageBuf &B, const int *P, int lane) {
    const TileGeom g = decode_tile(desc);
    int nhome = 0, mode = kStaged, total = 0;
    unsigned issued = 0;  // bytes of bulk copies this lane issued
    if (g.simple) {
        const Replica<float> &R = a.tb.reps[g.rep];
        mode = kSlots;
        if (lane == 0) {
            B.seg_s0[0] = R.off;
            B.seg_n[0] = 0;
            B.seg_n[1] = R.n;
            B.nseg = 1;
        }
        nhome = R.n;
    } else {
        const int nc = g.nc, sx = g.sx;
        const int nry = g.ty + 2, nrz = g.tz + 2, nrows = nry * nrz, ncell = nrows * sx;
        // -- 1: counts and global starts of the staged cells from the prefetched start[] rows
        const RowLayout L = row_layout(g, lane);
        const int run_x0 = g.whole ? L.ru0 : g.x0 - 1 + L.ru0;
        if (L.in_row) {
            for (int sz = 0; sz < nrz; sz++) {
                const int zb = plane_base(g, sz);
#pragma unroll
                for (int sy = 0; sy < kTileYZMax + 2; sy++) {
                    if (sy >= nry) break;
                    const int r = sz * nry + sy;
                    int lo = 0, cnt = 0;
                    const int rowg = row_base(g, zb, sy);
                    if (L.xok && rowg >= 0) {
                        const int *Pr = P + r * kStartRowInts;
                        const int e = L.c == L.wc ? kStartRunInts + ((rowg + L.gx_w) & 3)
                                                  : ((rowg + run_x0) & 3) + (L.c - L.ru0);
                        lo = Pr[e];
                        cnt = Pr[e + 1] - lo;
                    }
                    B.cell_sm[r * sx + L.c] = cnt;
                    B.cell_lo[r * sx + L.c] = lo;
                }
            }
        }
        __syncwarp();
        // -- 2: exclusive scan of the counts
        const int per = (ncell + 31) >> 5;
        const int j0 = min(lane * per, ncell), j1 = min(j0 + per, ncell);
        int sum = 0;
        for (int j = j0; j < j1; j++) sum += B.cell_sm[j];
        const int inc = warp_inclusive_scan(sum, lane);
        int run = inc - sum;
        for (int j = j0; j < j1; j++) {
            const int cnt = B.cell_sm[j];
            B.cell_sm[j] = run;
            run += cnt;
        }
        total = __shfl_sync(0xffffffffu, inc, 31);
        if (lane == 0) B.cell_sm[ncell] = total;
        __syncwarp();
        const int hx0 = g.whole ? 0 : 1, hx1 = g.whole ? sx : sx - 1;
        const int nhrows = g.ty * g.tz;
        if (total <= kStageCap) {
            // -- 3: copies, lanes over rows: the unwrapped run [ru0, ru1) and the wrapped cell wc
            const int ru0 = L.ru0, ru1 = L.ru1, wc = L.wc;
            bool fenced = false;
            for (int r = lane; r < nrows; r += 32) {
                const int rb = r * sx;
                const int k0 = B.cell_sm[rb + ru0], k1 = B.cell_sm[rb + ru1];
                if (k1 > k0) {
                    if (!fenced) { fence_proxy_async(); fenced = true; }
                    bulk_copy_g2s(&B.pos[k0], a.buf.pos + 4 * (size_t)B.cell_lo[rb + ru0], (unsigned)(k1 - k0) * 16u,
                                  &B.bar);
                    issued += (unsigned)(k1 - k0) * 16u;
                }
                if (wc >= 0) {
                    const int w0 = B.cell_sm[rb + wc], w1 = B.cell_sm[rb + wc + 1];
                    if (w1 > w0) {
                        if (!fenced) { fence_proxy_async(); fenced = true; }
                        bulk_copy_g2s(&B.pos[w0], a.buf.pos + 4 * (size_t)B.cell_lo[rb + wc], (unsigned)(w1 - w0) * 16u,
                                      &B.bar);
                        issued += (unsigned)(w1 - w0) * 16u;
                    }
                }
            }
            // home particles before each home row
            int hn = 0;
            if (lane < nhrows) {
                const int rb = ((1 + lane / g.ty) * nry + (1 + lane % g.ty)) * sx;
                hn = B.cell_sm[rb + hx1] - B.cell_sm[rb + hx0];
            }
            const int hinc = warp_inclusive_scan(hn, lane);
            if (lane < nhrows) B.row_start[lane] = hinc - hn;
            nhome = __shfl_sync(0xffffffffu, hinc, 31);
            if (lane == 0) B.row_start[nhrows] = nhome;
        } else {
            // too crowded to stage: the home rows as slot runs, nothing copied
            mode = kSlots;
            int n = 0, s0 = 0;
            if (lane < nhrows) {
                const int ry = 1 + lane % g.ty, rz = 1 + lane / g.ty;
                const int gy = g.y0 - 1 + ry, gz = g.z0 - 1 + rz;  // home rows are inside the box
                const int c0 = g.cell_off + (g.whole ? 0 : g.x0) + nc * (gy + nc * gz);
                const int c1 = c0 + (hx1 - hx0) - 1;
                s0 = __ldg(a.start + c0);
                n = __ldg(a.start + c1 + 1) - s0;
            }
            const int hinc = warp_inclusive_scan(n, lane);
            if (lane < nhrows) {
                B.seg_s0[lane] = s0;
                B.seg_n[lane] = hinc - n;
            }
            if (lane == nhrows - 1) B.seg_n[nhrows] = hinc;
            if (lane == 0) B.nseg = nhrows;
            nhome = __shfl_sync(0xffffffffu, hinc, 31);
        }
    }
    const int units = (nhome + 31) / 32;
    if (lane == 0) {
        B.desc = desc;
        B.mode = mode;
        B.total = total;
        B.nhome = nhome;
    }
    issued = __reduce_add_sync(0xffffffffu, issued);
    __syncwarp();
    // the single arrival expects exactly the bytes issued (zero when nothing was copied), so the
    // phase always completes
    if (lane == 0) mbar_arrive_expect_tx(&B.bar, issued);
    return units;
}

enum ScanKind : int { kScanExact = 0, kScanBuild = 1, kScanStale = 2 };

// Phase 1: candidate scan in shared memory, one lane per home particle.  A neighbour cell reached across
// a periodic face holds unshifted coordinates; its image shift s (0 or +-L per axis, known from the
// staged cell's unwrapped coordinate) gives the separation (x_i - x_j) - s, which is exactly what the
// minimum-image rule computes for every pair within the force range.  The three cells of a row are at
// most two contiguous segments (split only where an image shift changes).  The loops are warp-uniform
// (each row runs to the longest lane's candidate count), so in-range candidates are appended with one
// ballot per candidate round and no shared-memory atomics.  Returns the warp's pair count.
//   kScanExact  cells sorted this step, pairs within the force range
//   kScanBuild  skin lists, rebuild step: also stores every candidate within the list range as the
//               home's list (staged particle | staged cell << 11) and its length
//   kScanStale  skin lists, cells sorted at the last build and particles moved since: minimum image
template <int KIND>
__device__ __forceinline__ int scan_cells(const ForceArgs<float> &a, const Replica<float> &R, const TileGeom &g,
                                          const StageBuf &B, WarpScratch &W, bool active, int myk, int mycell, int slot,
                                          int lane) {
    const int nry = g.ty + 2;
    int npairs = 0;  // warp-uniform
    int lc = 0;      // KIND == kScanBuild: candidates of this lane's home within the list range
    {
        const float4 pi = active ? B.pos[myk] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int lx = mycell % g.sx, ly = (mycell / g.sx) % nry, lz = mycell / (g.sx * nry);
        const int nc = R.nc;
        const float L = R.box;
        const unsigned lt_mask = (1u << lane) - 1u;
        for (int dz = -1; dz <= 1; dz++) {
            const int gz = g.z0 - 1 + lz + dz;
            const float shz = gz < 0 ? -L : (gz >= nc ? L : 0.f);
            for (int dy = -1; dy <= 1; dy++) {
                const int gy = g.y0 - 1 + ly + dy;
                const float shy = gy < 0 ? -L : (gy >= nc ? L : 0.f);
                const int rowb = ((lz + dz) * nry + (ly + dy)) * g.sx;
                // segments of this row: [c0, c1) unshifted in x, plus one wrapped cell cw (shift shw)
                int c0 = lx - 1, c1 = lx + 2, cw = -1;
                float shw = 0.f;
                if (g.whole) {
                    if (c0 < 0) { c0 = 0; cw = R.periodic ? nc - 1 : -1; shw = -L; }
                    if (c1 > g.sx) { c1 = g.sx; cw = R.periodic ? 0 : -1; shw = L; }
                } else {
                    const int gx0 = g.x0 - 1 + c0, gx1 = g.x0 - 1 + (c1 - 1);
                    if (gx0 < 0) { cw = c0; shw = -L; c0 += 1; }
                    else if (gx1 >= nc) { cw = c1 - 1; shw = L; c1 -= 1; }
                }
                int ka = 0, lena = 0, kb = 0, len = 0, b1 = 0, b2 = 0;
                if (active) {
                    ka = B.cell_sm[rowb + c0];
                    lena = B.cell_sm[rowb + c1] - ka;
                    b1 = c0 + 1 < c1 ? B.cell_sm[rowb + c0 + 1] : 1 << 30;  // cell boundaries inside [c0, c1)
                    b2 = c0 + 2 < c1 ? B.cell_sm[rowb + c0 + 2] : 1 << 30;
                    len = lena;
                    if (cw >= 0) {
                        kb = B.cell_sm[rowb + cw];
                        len += B.cell_sm[rowb + cw + 1] - kb;
                    }
                }
                const int maxlen = __reduce_max_sync(0xffffffffu, len);
                // four candidates per lane per round: their loads are issued together
                for (int t0 = 0; t0 < maxlen; t0 += 4) {
                    float4 pj[4];
                    int kq[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int t = t0 + u;
                        kq[u] = t < lena ? ka + t : kb + (t - lena);
                        pj[u] = B.pos[t < len ? kq[u] : myk];
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int t = t0 + u;
                        float ddx, ddy, ddz;
                        if (KIND == kScanStale) {
                            // positions have moved since the cells were built: plain minimum image
                            ddx = min_image_sep<float>(pi.x, pj[u].x, R.box, R.box_lo, R.l2s, R.periodic);
                            ddy = min_image_sep<float>(pi.y, pj[u].y, R.box, R.box_lo, R.l2s, R.periodic);
                            ddz = min_image_sep<float>(pi.z, pj[u].z, R.box, R.box_lo, R.l2s, R.periodic);
                        } else {
                            const float shx = t < lena ? 0.f : shw;
                            ddx = (pi.x - pj[u].x) - shx;
                            ddy = (pi.y - pj[u].y) - shy;
                            ddz = (pi.z - pj[u].z) - shz;
                        }
                        const float r2 = ddx * ddx + ddy * ddy + ddz * ddz;
                        const bool cand = t < len && kq[u] != myk;
                        const bool hit = cand && r2 < R.rc2;
                        const int cell = t < lena ? rowb + c0 + (kq[u] >= b1) + (kq[u] >= b2) : rowb + cw;
                        if (KIND == kScanBuild && cand && r2 < R.rc2_list) {
                            if (lc < kListCap) a.list[(size_t)lc * a.tb.ntot + slot] = (unsigned)kq[u] | ((unsigned)cell << 11);
                            lc++;
                        }
                        const unsigned m = __ballot_sync(0xffffffffu, hit);
                        if (hit) {
                            const int p = npairs + __popc(m & lt_mask);
                            if (p < kWarpPairCap) W.pair[p] = pair_entry(kq[u], cell, lane);
                        }
                        npairs += __popc(m);
                    }
                }
            }
        }
    }
    if (KIND == kScanBuild && active) a.list_n[slot] = lc;
    return npairs;
}

// Phase 1 on a step that keeps its skin lists: each lane's home tests its stored candidates (the staged
// indices are those of the last build: the cells, hence the staging, are unchanged until the next one).
__device__ __forceinline__ int scan_list(const ForceArgs<float> &a, const Replica<float> &R, const StageBuf &B,
                                         WarpScratch &W, bool active, int myk, int slot, int cnt, int lane) {
    const float4 pi = active ? B.pos[myk] : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned lt_mask = (1u << lane) - 1u;
    const int maxlen = __reduce_max_sync(0xffffffffu, cnt);
    int npairs = 0;
    for (int t0 = 0; t0 < maxlen; t0 += 4) {
        unsigned e[4];
        float4 pj[4];
#pragma unroll
        for (int u = 0; u < 4; u++) e[u] = t0 + u < cnt ? __ldg(a.list + (size_t)(t0 + u) * a.tb.ntot + slot) : 0u;
#pragma unroll
        for (int u = 0; u < 4; u++) pj[u] = B.pos[t0 + u < cnt ? (int)(e[u] & 2047u) : myk];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float ddx = min_image_sep<float>(pi.x, pj[u].x, R.box, R.box_lo, R.l2s, R.periodic);
            const float ddy = min_image_sep<float>(pi.y, pj[u].y, R.box, R.box_lo, R.l2s, R.periodic);
            const float ddz = min_image_sep<float>(pi.z, pj[u].z, R.box, R.box_lo, R.l2s, R.periodic);
            const bool hit = t0 + u < cnt && ddx * ddx + ddy * ddy + ddz * ddz < R.rc2;
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (hit) {
                const int p = npairs + __popc(m & lt_mask);
                if (p < kWarpPairCap) W.pair[p] = pair_entry((int)(e[u] & 2047u), (int)(e[u] >> 11), lane);
            }
            npairs += __popc(m);
        }
    }
    return npairs;
}

// Consumer warp: unit u (32 home particles) of a staged tile -- phases 1-4
template <int MODE>
__device__ void consume_staged_unit(const ForceArgs<float> &a, const StageBuf &B, WarpScratch &W, int u, int lane,
                                    bool &big, int &overflow) {
    const TileGeom g = decode_tile(B.desc);
    const Replica<float> &R = a.tb.reps[g.rep];
    const Model<float> &M = a.tb.models[R.model];
    const int nry = g.ty + 2;
    const int hx0 = g.whole ? 0 : 1, hx1 = g.whole ? g.sx : g.sx - 1;
    const int hidx = 32 * u + lane;
    const bool active = hidx < B.nhome;
    int myk = 0, mycell = 0;
    if (active) {
        int r = 0;
        while (B.row_start[r + 1] <= hidx) r++;
        const int rb = ((1 + r / g.ty) * nry + (1 + r % g.ty)) * g.sx;
        myk = B.cell_sm[rb + hx0] + (hidx - B.row_start[r]);
        int lo = hx0, hi = hx1;  // cell_sm[rb+lo] <= myk < cell_sm[rb+hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (B.cell_sm[rb + mid] <= myk) lo = mid;
            else hi = mid;
        }
        mycell = rb + lo;
        const int slot = B.cell_lo[mycell] + (myk - B.cell_sm[mycell]);
        W.h_k[lane] = myk;
        W.h_slot[lane] = slot;
        W.h_id[lane] = __ldg(a.buf.ident + slot);
        W.h_qa[lane] = __ldg(reinterpret_cast<const float4 *>(a.buf.rota) + slot);
        W.h_qb[lane] = __ldg(reinterpret_cast<const float4 *>(a.buf.rotb) + slot);
    }
#pragma unroll
    for (int k = 0; k < 6; k++) W.acc[lane][k] = 0ull;
    __syncwarp();

    // -- phase 1: the warp's pair list (scan_cells / scan_list)
    const int slot = active ? W.h_slot[lane] : 0;
    int npairs;
    if (!a.skin) {
        npairs = scan_cells<kScanExact>(a, R, g, B, W, active, myk, mycell, slot, lane);
    } else if (*a.skin) {
        npairs = scan_cells<kScanBuild>(a, R, g, B, W, active, myk, mycell, slot, lane);
    } else {
        const int cnt = active ? __ldg(a.list_n + slot) : 0;
        if (__any_sync(0xffffffffu, cnt > kListCap))  // a home had more candidates than its list holds
            npairs = scan_cells<kScanStale>(a, R, g, B, W, active, myk, mycell, slot, lane);
        else
            npairs = scan_list(a, R, B, W, active, myk, slot, cnt, lane);
    }
    __syncwarp();
    if (npairs > kWarpPairCap) {
        // more pairs than the warp's list holds: these 32 particles take the per-thread path
        if (active) simple_particle<float, MODE>(a, W.h_slot[lane]);
        overflow = 1;
        __syncwarp();
        return;
    }
    // -- phase 2a: the warp's pairs spread over its lanes: WCA core and the home cone test.  Pairs that
    // may have a patch potential are compacted in place (an entry is written only after every lane of
    // its round has read its own), so phase 2b runs its global loads on dense rounds.
    int ncand = 0;  // warp-uniform
    {
        const unsigned lt_mask = (1u << lane) - 1u;
        for (int p0 = 0; p0 < npairs; p0 += 32) {
            const int p = p0 + lane;
            unsigned e = 0;
            bool keep = false;
            if (p < npairs) {
                e = W.pair[p];
                keep = pair_core(R, M, B, W, e, big);
            }
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) W.pair[ncand + __popc(m & lt_mask)] = e;
            ncand += __popc(m);
        }
    }
    __syncwarp();
    // -- phase 2b: cone tests and Kern-Frenkel potentials of the remaining pairs
    for (int p = lane; p < ncand; p += 32) pair_patches(a, R, M, B, W, W.pair[p]);
    __syncwarp();
    // -- phase 3: epilogue per home particle
    if (active) {
        const int s = W.h_slot[lane];
        float F[3] = {acc_get(W.acc[lane][0]), acc_get(W.acc[lane][1]), acc_get(W.acc[lane][2])};
        const float T[3] = {acc_get(W.acc[lane][3]), acc_get(W.acc[lane][4]), acc_get(W.acc[lane][5])};
        if (a.bond_start) {
            const float4 ph = B.pos[myk];
            float eb = 0.f;
            bond_forces<float>(a, R, W.h_id[lane], ph.x, ph.y, ph.z, F, eb, big);
        }
        if (MODE == kModeForces) {
            const int id = W.h_id[lane];
            for (int k = 0; k < 3; k++) {
                a.outF[3 * (size_t)id + k] = F[k];
                a.outT[3 * (size_t)id + k] = T[k];
            }
        } else {
            const float4 pi = B.pos[myk];
            float Qi[9];
            home_q(W, lane, pi.w, Qi);
            langevin_epilogue<float>(a, R, g.rep, s, W.h_id[lane], F, T, Qi, pi.x, pi.y, pi.z);
        }
    }
    __syncwarp();
}

// Persistent warp-specialised force kernel.  The last warp of each CTA stages tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... into a ring of three buffers and publishes their 32-particle units
// as consecutive ranges of one CTA-wide unit stream; the other warps claim units from the stream in
// order.  A buffer is restaged only after every unit of its previous tile is done, and claims are
// monotone, so every mbarrier wait below has an unambiguous parity.  All waits are bounded.
template <int MODE>
__global__ void __launch_bounds__(kTileThreads, 1) tile_force_kernel(ForceArgs<float> a, const int4 *tiles, int ntiles) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TileShared &sh = *reinterpret_cast<TileShared *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int b = 0; b < kStageBufs; b++) {
            mbar_init(&sh.buf[b].bar, 1);
            sh.buf[b].range = 0ull;
            sh.buf[b].nunits = 0;
            sh.buf[b].done = 0;
        }
        fence_proxy_async();
        sh.claim = 0;
        sh.final_units = -1;
        sh.overflow = 0;
    }
    __syncthreads();

    if (warp == kTileWarps - 1) {
        // ---------------- producer
        // the start[] entries of tile k are copied (cp.async) during tile k - 1, its descriptor is
        // loaded during tile k - 2
        int cum = 0;
        const int G = (int)gridDim.x;
        int4 cur = (int)blockIdx.x < ntiles ? tiles[blockIdx.x] : make_int4(0, 0, 0, 0);
        int4 nxt = (int)blockIdx.x + G < ntiles ? tiles[blockIdx.x + G] : make_int4(0, 0, 0, 0);
        if ((int)blockIdx.x < ntiles) prefetch_starts(a, cur, sh.start_rows[0], lane);
        cp_async_commit();
        for (int k = 0;; k++) {
            const int tile = blockIdx.x + k * G;
            if (tile >= ntiles) break;
            const int4 desc = cur;
            if (tile + G < ntiles) prefetch_starts(a, nxt, sh.start_rows[(k + 1) & 1], lane);
            cp_async_commit();
            cur = nxt;
            if (tile + 2 * G < ntiles) nxt = tiles[tile + 2 * G];
            StageBuf &B = sh.buf[k % kStageBufs];
            if (k >= kStageBufs) {
                // the previous use's copies have landed (also when no consumer waited on them) ...
                bool landed = false;
                const unsigned prev = (unsigned)((k - kStageBufs) / kStageBufs) & 1u;
                for (unsigned it = 0; it < kWaitSpins && !landed; it++) landed = mbar_try_wait(&B.bar, prev);
                if (!landed) {
                    if (lane == 0) atomicOr(a.flags, 4u);
                    break;
                }
                // ... and the consumers are done with the tile this buffer held
                const int need = B.nunits;
                bool ok = false;
                for (unsigned it = 0; it < (kWaitSpins << 4) && !ok; it++) {
                    ok = ld_volatile(&B.done) >= need;
                    if (!ok) __nanosleep(64);
                }
                if (!ok) {
                    if (lane == 0) atomicOr(a.flags, 4u);
                    break;
                }
                __threadfence_block();
            }
            cp_async_wait_prev();  // this tile's start[] entries have landed (this lane's copies) ...
            __syncwarp();          // ... and every lane's
            const int units = produce_tile(a, desc, B, sh.start_rows[k & 1], lane);
            if (lane == 0) {
                B.done = 0;
                B.nunits = units;
                __threadfence_block();
                const unsigned long long parity = (unsigned long long)((k / kStageBufs) & 1);
                *(volatile unsigned long long *)&B.range =
                    (unsigned long long)(unsigned)cum | ((unsigned long long)(unsigned)units << 32) | (parity << 63);
            }
            cum += units;
            __syncwarp();
        }
        if (lane == 0) *(volatile int *)&sh.final_units = cum;
        cp_async_wait_all();
        // drain: the last use of every buffer has completed (its copies landed) before this CTA exits
        const int nk = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
        for (int b = 0; b < kStageBufs && b < nk; b++) {
            const int klast = b + ((nk - 1 - b) / kStageBufs) * kStageBufs;
            bool ok = false;
            for (unsigned it = 0; it < kWaitSpins && !ok; it++) ok = mbar_try_wait(&sh.buf[b].bar, (unsigned)(klast / kStageBufs) & 1u);
            if (!ok && lane == 0) atomicOr(a.flags, 4u);
        }
    } else {
        // ---------------- consumers
        WarpScratch &W = sh.w[warp];
        bool big = false;
        int overflow = 0;
        for (;;) {
            int U = 0;
            if (lane == 0) U = atomicAdd(&sh.claim, 1);
            U = __shfl_sync(0xffffffffu, U, 0);
            // find the buffer that holds unit U (published by the producer in order)
            int b = -1, ubegin = 0;
            unsigned parity = 0;
            bool stop = false;
            for (unsigned it = 0; it < (kWaitSpins << 4); it++) {
                for (int q = 0; q < kStageBufs; q++) {
                    const unsigned long long rw = *(const volatile unsigned long long *)&sh.buf[q].range;
                    const int beg = (int)(unsigned)(rw & 0xffffffffull);
                    const int cnt = (int)(unsigned)((rw >> 32) & 0x7fffffffull);
                    if (beg <= U && U < beg + cnt) {
                        b = q;
                        ubegin = beg;
                        parity = (unsigned)(rw >> 63);
                    }
                }
                if (b >= 0) break;
                const int fin = ld_volatile(&sh.final_units);
                if (fin >= 0 && U >= fin) {
                    stop = true;
                    break;
                }
                __nanosleep(64);
            }
            if (stop) break;
            if (b < 0) {
                if (lane == 0) atomicOr(a.flags, 4u);
                break;
            }
            StageBuf &B = sh.buf[b];
            bool ready = false;
            for (unsigned it = 0; it < kWaitSpins && !ready; it++) ready = mbar_try_wait(&B.bar, parity);
            ready = __all_sync(0xffffffffu, ready);
            if (!ready) {
                if (lane == 0) atomicOr(a.flags, 4u);
                break;
            }
            const int u = U - ubegin;
            if (B.mode == kStaged) {
                consume_staged_unit<MODE>(a, B, W, u, lane, big, overflow);
            } else {
                const int hidx = 32 * u + lane;
                if (hidx < B.nhome) {
                    int r = 0;
                    while (B.seg_n[r + 1] <= hidx) r++;
                    simple_particle<float, MODE>(a, B.seg_s0[r] + (hidx - B.seg_n[r]));
                }
            }
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                atomicAdd(&B.done, 1);
            }
        }
        if (big) atomicOr(a.flags, 2u);
        if (overflow && lane == 0) atomicOr(a.flags, 8u);
    }
}

}  // namespace
}  // namespace mtg
