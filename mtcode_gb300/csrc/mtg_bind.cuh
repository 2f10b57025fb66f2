// mtg_bind.cuh -- single-bond-per-patch mode: the force pass of Condensate::run_singlebond
// (Condensate/Condensate.cpp:422-618), where every patch holds at most one bond and only bound patch
// pairs exert the Kern-Frenkel force.
//
// Per step (all replicas in every launch):
//   [begin]     one thread: this update's stamp, whether the candidate list is due (every patch_every steps)
//   [candidates] one thread per particle, every patch_every steps (LangevinNVTR::calculate_patch_list,
//               LangevinR.cpp:1702-1852): patch pairs of particle pairs closer than
//               min(list cut, max_check + 1) whose cones pass (c_i - max_ang) + (c_j - max_ang) > -0.4.
//               Entries hold particle ids and patch ids, so they outlive the re-sorting of every step.
//   [edges]     one thread per candidate (LangevinRforce.cpp:2900-3090): the distance / cone / bind-state
//               test; an edge goes into both patches' adjacency (stamped counters: no reset pass).
//   [decide]    one thread per patch: no edge -> unbound; else a breadth-first walk of its component.  The
//               component's smallest patch decides a cluster of two or three (doublet / triplet of the
//               binding model, LangevinRforce.cpp:3160-3480); members of larger components queue for:
//   [large]     one thread per queued patch; the smallest one runs the reference's reduction (drop the
//               highest-scoring edge until no piece exceeds three patches, LangevinRforce.cpp:3560-3880)
//               with its scratch in global memory.
// The bound pairs' forces are added by the force epilogue (bound_patch_forces), from both ends.
//
// Exactness.  Every test that decides a bond is the reference's FP64 expression, evaluated with explicit
// roundings in the reference's operation order on the stored coordinates, so the GPU and an FP64 CPU
// evaluation of the same state take identical decisions.  In FP32 the tests first run in float; only a
// value within a margin of its threshold (far above the float evaluation's error) is re-evaluated in FP64.
#pragma once

#include <cooperative_groups.h>

#include "mtg_kernels.cuh"

namespace mtg {

constexpr int kAdjCap = 8;            // candidate partners of one patch in one update
constexpr int kClusterCap = 128;      // patches of one cluster reduced by one thread
constexpr int kClusterEdges = kClusterCap * kAdjCap / 2;
constexpr int kLargeThreads = 64;     // block of the large-cluster kernel
constexpr unsigned kFlagBind = 0x20u; // a capacity of this mode was exceeded (see MTG_FLAG_BIND)

// binding model in table form: species rule of a patch index, doublet rows (species pairs 11, 12, 13, 22,
// 23, 33; [before * 2 + 0] to unbound, + 1 to bound) and triplet rows (sorted triples 111 ... 333,
// [state * 4 + k])
struct BindModel {
    int rule, div1, div2, np;
    double drate[6][4];
    double trate[10][16];
};

struct BindState {
    const BindRep *reps;
    const BindModel *model;
    const int *patch_slot;        // nrep + 1 global patch offsets
    int nrep;
    int ptot;
    int patch_every;
    int4 *plist;                  // candidates: (id1 < id2, patch of id1, patch of id2), global indices
    long long plist_cap;
    unsigned long long *ctr;      // [0] candidates [1] queued large-cluster patches [2] update stamp
                                  // [3] steps of the run_singlebond loop so far [4] candidates due this update
    unsigned long long *deg;      // per patch: stamp << 32 | edges of this update
    int2 *adj;                    // per patch kAdjCap: (partner patch, candidate << 2 | disp2 class)
    int *boundto;                 // global patch indices
    unsigned char *isbound;
    int *large;                   // queued patches of clusters above three
    int *scratch;                 // large-cluster scratch, one block of kScratchInts per thread
    int scratch_threads;
    unsigned *flags;
    const unsigned long long *draw;
};

namespace {

// ------------------------------------------------------------------ FP64 tests in the reference's order
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

// position and rotation of a slot as doubles (exact conversions of the stored values)
template <class real>
__device__ __forceinline__ void load_state_d(const Buffers<real> &b, int s, double x[3], double q[9]) {
    Payload<real> P;
    P.load(b.pos, b.rota, b.rotb, s);
#pragma unroll
    for (int k = 0; k < 3; k++) x[k] = (double)P.v[k];
#pragma unroll
    for (int k = 0; k < 9; k++) q[k] = (double)P.v[3 + k];
}

// float value v against threshold t: +1 certainly above, -1 certainly below, 0 too close to tell
__device__ __forceinline__ int side(double v, double t, double margin) {
    return v > t + margin ? 1 : (v < t - margin ? -1 : 0);
}

// ------------------------------------------------------------------ candidate list
__device__ __forceinline__ void plist_append(const BindState &S, int4 e) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(S.ctr, (unsigned long long)g.size());
    base = g.shfl(base, 0) + g.thread_rank();
    if ((long long)base < S.plist_cap) S.plist[base] = e;
    else atomicOr(S.flags, kFlagBind);
}

// cells of one axis within `reach` of cell c, each once (all cells when the grid is narrower than the stencil)
__device__ __forceinline__ int axis_cells(int c, int nc, int reach, int periodic, int out[5]) {
    int m = 0;
    if (nc <= 2 * reach) {
        for (int k = 0; k < nc && k < 5; k++) out[m++] = k;
        return m;
    }
    for (int d = -reach; d <= reach; d++) {
        int cc = c + d;
        if (cc < 0 || cc >= nc) {
            if (!periodic) continue;
            cc = cc < 0 ? cc + nc : cc - nc;
        }
        out[m++] = cc;
    }
    return m;
}

__global__ void bind_begin_kernel(BindState S, int force, int advance) {
    if (threadIdx.x || blockIdx.x) return;
    const unsigned long long step = S.ctr[3];
    const int due = force || (step > 0 && S.patch_every > 0 && step % (unsigned long long)S.patch_every == 0);
    S.ctr[4] = due;
    if (due) S.ctr[0] = 0;
    S.ctr[1] = 0;
    S.ctr[2] += 1;
    if (advance) S.ctr[3] = step + 1;
}

// LangevinNVTR::calculate_patch_list on the current (cell-sorted) buffers
template <class real>
__global__ void __launch_bounds__(256) bind_candidates_kernel(ForceArgs<real> a, BindState S) {
    if (!S.ctr[4]) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.tb.ntot) return;
    const int r = find_replica(a.tb.rep_slot, a.tb.nrep, s);
    const Replica<real> &R = a.tb.reps[r];
    const Model<real> &M = a.tb.models[R.model];
    const BindRep &B = S.reps[r];
    const int id = a.buf.ident[s], li = id - R.off, ti = type_of<real>(M, li), na = M.np[ti];
    if (na == 0) return;
    Payload<real> Pi;
    Pi.load(a.buf.pos, a.buf.rota, a.buf.rotb, s);
    const int nc = R.nc;
    int cx[5], cy[5], cz[5];
    const int mx = axis_cells(axis_cell<real>(Pi.v[0], R.cell_scale, nc), nc, B.reach, R.periodic, cx);
    const int my = axis_cells(axis_cell<real>(Pi.v[1], R.cell_scale, nc), nc, B.reach, R.periodic, cy);
    const int mz = axis_cells(axis_cell<real>(Pi.v[2], R.cell_scale, nc), nc, B.reach, R.periodic, cz);
    const double max_dis2 = B.max_dis * B.max_dis;
    for (int iz = 0; iz < mz; iz++)
        for (int iy = 0; iy < my; iy++)
            for (int ix = 0; ix < mx; ix++) {
                const int cell = R.cell_off + cx[ix] + nc * (cy[iy] + nc * cz[iz]);
                const int j0 = __ldg(a.start + cell), j1 = __ldg(a.start + cell + 1);
                for (int j = j0; j < j1; j++) {
                    const int idj = __ldg(a.buf.ident + j);
                    if (idj <= id) continue;   // each pair once, p1 < p2 (LangevinR.cpp:1722-1727)
                    const int lj = idj - R.off, tj = type_of<real>(M, lj), nb = M.np[tj];
                    if (nb == 0) continue;
                    real xj, yj, zj;
                    load_pos(a.buf.pos + 4 * (size_t)j, xj, yj, zj);
                    const real dx = min_image<real>(Pi.v[0] - xj, R.box, R.l2s, R.periodic);
                    const real dy = min_image<real>(Pi.v[1] - yj, R.box, R.l2s, R.periodic);
                    const real dz = min_image<real>(Pi.v[2] - zj, R.box, R.l2s, R.periodic);
                    const double d2f = (double)(dx * dx + dy * dy + dz * dz);
                    // pair list (distance_less_than at the list cut) and dis < max_check + 1
                    int in1 = side(d2f, B.list_cut2, 1e-5 * B.list_cut2), in2 = side(d2f, max_dis2, 1e-5 * max_dis2);
                    if (in1 > 0 || in2 > 0) continue;
                    double xa[3], qa[9], xb[3], qb[9], un[3];
                    bool exact = std::is_same<real, double>::value || in1 == 0 || in2 == 0;
                    double d2 = d2f, dis = 0;
                    if (exact) {
                        load_state_d<real>(a.buf, s, xa, qa);
                        load_state_d<real>(a.buf, j, xb, qb);
                        d2 = exact_dist_vec(B, xa, xb, un);
                        if (!(d2 < B.list_cut2)) continue;
                        dis = __dsqrt_rn(d2);
                        if (!(dis < B.max_dis)) continue;
                        un[0] = __ddiv_rn(un[0], dis); un[1] = __ddiv_rn(un[1], dis); un[2] = __ddiv_rn(un[2], dis);
                    }
                    // cones of every patch pair, float first where it is decisive
                    real Qj[9];
                    {
                        Payload<real> Pj;
                        Pj.load(a.buf.pos, a.buf.rota, a.buf.rotb, j);
#pragma unroll
                        for (int k = 0; k < 9; k++) Qj[k] = Pj.v[3 + k];
                    }
                    const real rr = sqrt(dx * dx + dy * dy + dz * dz);
                    const real u[3] = {dx / rr, dy / rr, dz / rr};
                    real wa[3], wb[3];
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        wa[k] = Pi.v[3 + 3 * k] * u[0] + Pi.v[4 + 3 * k] * u[1] + Pi.v[5 + 3 * k] * u[2];
                        wb[k] = Qj[3 * k] * u[0] + Qj[3 * k + 1] * u[1] + Qj[3 * k + 2] * u[2];
                    }
                    const int oa = M.ooff[ti], ob = M.ooff[tj];
                    for (int ka = 0; ka < na; ka++) {
                        const real *va = M.orient[oa + ka];
                        const real ci = -(va[0] * wa[0] + va[1] * wa[1] + va[2] * wa[2]);
                        for (int kb = 0; kb < nb; kb++) {
                            const real *vb = M.orient[ob + kb];
                            const real cj = vb[0] * wb[0] + vb[1] * wb[1] + vb[2] * wb[2];
                            int pass = side(((double)ci - B.max_ang) + ((double)cj - B.max_ang), -0.4, 4e-5);
                            if (exact || pass == 0) {
                                if (!exact) {
                                    load_state_d<real>(a.buf, s, xa, qa);
                                    load_state_d<real>(a.buf, j, xb, qb);
                                    d2 = exact_dist_vec(B, xa, xb, un);
                                    dis = __dsqrt_rn(d2);
                                    un[0] = __ddiv_rn(un[0], dis); un[1] = __ddiv_rn(un[1], dis); un[2] = __ddiv_rn(un[2], dis);
                                    exact = true;
                                }
                                const double ei = exact_cos(B.orient[oa + ka], qa, un, true);
                                const double ej = exact_cos(B.orient[ob + kb], qb, un, false);
                                pass = __dadd_rn(__dsub_rn(ei, B.max_ang), __dsub_rn(ej, B.max_ang)) > -0.4 ? 1 : -1;
                            }
                            if (pass > 0)
                                plist_append(S, make_int4(id, idj, patch_of<real>(B, M, li, ti, ka),
                                                          patch_of<real>(B, M, lj, tj, kb)));
                        }
                    }
                }
            }
}

// ------------------------------------------------------------------ edges
// slot of this update's adjacency for patch p (stamped counter: a stale stamp counts as zero edges)
__device__ __forceinline__ int adj_take(unsigned long long *deg, int p, unsigned stamp, unsigned *flags) {
    unsigned long long old = deg[p];
    for (int it = 0; it < (1 << 20); it++) {
        const unsigned cnt = (unsigned)(old >> 32) == stamp ? (unsigned)old : 0u;
        const unsigned long long nw = ((unsigned long long)stamp << 32) | (unsigned long long)(cnt + 1u);
        const unsigned long long prev = atomicCAS(deg + p, old, nw);
        if (prev == old) return (int)cnt;
        old = prev;
    }
    atomicOr(flags, kFlagBind);
    return kAdjCap;
}

__device__ __forceinline__ int adj_count(const unsigned long long *deg, int p, unsigned stamp) {
    const unsigned long long w = deg[p];
    const int c = (unsigned)(w >> 32) == stamp ? (int)(unsigned)w : 0;
    return c < kAdjCap ? c : kAdjCap;
}

// the reference's bind-state dependent range (LangevinRforce.cpp:3010-3030): class 0 disp, 1 0.5 disp,
// 2 0.7 disp
__device__ __forceinline__ double disp2_of(double disp, int cls) {
    return cls == 1 ? __dmul_rn(0.5, disp) : (cls == 2 ? __dmul_rn(0.7, disp) : disp);
}

// FP64 edge test of one candidate; with score != null also its score (LangevinRforce.cpp:3040-3060)
template <class real>
__device__ __forceinline__ bool exact_edge(const BindRep &B, const Buffers<real> &b, int s1, int s2, int o1, int o2,
                                           int potn, double disp2, double *score) {
    double xa[3], qa[9], xb[3], qb[9], un[3];
    load_state_d<real>(b, s1, xa, qa);
    load_state_d<real>(b, s2, xb, qb);
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

// the candidate's particles, patch numbers and potential
struct Cand {
    int s1, s2, o1, o2, potn, r;
};

template <class real>
__device__ __forceinline__ Cand cand_of(const ForceArgs<real> &a, const BindState &S, int4 e) {
    Cand c;
    c.r = find_replica(a.tb.rep_slot, a.tb.nrep, e.x);
    const Replica<real> &R = a.tb.reps[c.r];
    const Model<real> &M = a.tb.models[R.model];
    const BindRep &B = S.reps[c.r];
    int l1, t1, k1, l2, t2, k2;
    patch_owner<real>(B, M, e.z - B.patch_off, l1, t1, k1);
    patch_owner<real>(B, M, e.w - B.patch_off, l2, t2, k2);
    c.s1 = a.buf.slot_of[e.x];
    c.s2 = a.buf.slot_of[e.y];
    c.o1 = M.ooff[t1] + k1;
    c.o2 = M.ooff[t2] + k2;
    c.potn = M.pstart[t1][t2] + k1 * M.np[t2] + k2;
    return c;
}

template <class real>
__global__ void __launch_bounds__(256) bind_edge_kernel(ForceArgs<real> a, BindState S) {
    const long long n = (long long)S.ctr[0] < S.plist_cap ? (long long)S.ctr[0] : S.plist_cap;
    const unsigned stamp = (unsigned)S.ctr[2];
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int4 e = S.plist[q];
        const Cand c = cand_of<real>(a, S, e);
        const Replica<real> &R = a.tb.reps[c.r];
        const Model<real> &M = a.tb.models[R.model];
        const BindRep &B = S.reps[c.r];
        const bool b1 = S.isbound[e.z] != 0, b2 = S.isbound[e.w] != 0;
        const bool cond1 = S.boundto[e.z] == e.w && S.boundto[e.w] == e.z;
        const int cls = (b1 && b2) ? (cond1 ? 0 : 1) : (b1 != b2 ? 2 : 0);
        const double disp2 = disp2_of(B.disp[c.potn], cls);
        bool edge;
        if (std::is_same<real, double>::value) {
            edge = exact_edge<real>(B, a.buf, c.s1, c.s2, c.o1, c.o2, c.potn, disp2, nullptr);
        } else {
            // float evaluation; anything within a margin of a threshold is decided in FP64
            Payload<real> P1, P2;
            P1.load(a.buf.pos, a.buf.rota, a.buf.rotb, c.s1);
            P2.load(a.buf.pos, a.buf.rota, a.buf.rotb, c.s2);
            const real dx = min_image<real>(P1.v[0] - P2.v[0], R.box, R.l2s, R.periodic);
            const real dy = min_image<real>(P1.v[1] - P2.v[1], R.box, R.l2s, R.periodic);
            const real dz = min_image<real>(P1.v[2] - P2.v[2], R.box, R.l2s, R.periodic);
            const real r2 = dx * dx + dy * dy + dz * dz;
            int t0 = side((double)r2, B.mk2, 1e-5 * B.mk2);
            if (t0 > 0) continue;
            const real rr = sqrt(r2);
            const real u[3] = {dx / rr, dy / rr, dz / rr};
            const real *v1 = M.orient[c.o1], *v2 = M.orient[c.o2];
            real n1[3], n2[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                n1[k] = v1[0] * P1.v[3 + k] + v1[1] * P1.v[6 + k] + v1[2] * P1.v[9 + k];
                n2[k] = v2[0] * P2.v[3 + k] + v2[1] * P2.v[6 + k] + v2[2] * P2.v[9 + k];
            }
            const real ci = -(n1[0] * u[0] + n1[1] * u[1] + n1[2] * u[2]);
            const real cj = n2[0] * u[0] + n2[1] * u[1] + n2[2] * u[2];
            const int t1 = side((double)ci, B.ctm[c.potn], 2e-5), t2 = side((double)cj, B.ctm[c.potn], 2e-5);
            const int t3 = side((double)rr, disp2, 1e-5 * disp2);
            if (t1 < 0 || t2 < 0 || t3 > 0) continue;
            if (t0 < 0 && t1 > 0 && t2 > 0 && t3 < 0) edge = true;
            else edge = exact_edge<real>(B, a.buf, c.s1, c.s2, c.o1, c.o2, c.potn, disp2, nullptr);
        }
        if (!edge) continue;
        const int k1 = adj_take(S.deg, e.z, stamp, S.flags), k2 = adj_take(S.deg, e.w, stamp, S.flags);
        const int tag = (int)(q << 2) | cls;
        if (k1 < kAdjCap) S.adj[(size_t)e.z * kAdjCap + k1] = make_int2(e.w, tag);
        else atomicOr(S.flags, kFlagBind);
        if (k2 < kAdjCap) S.adj[(size_t)e.w * kAdjCap + k2] = make_int2(e.z, tag);
        else atomicOr(S.flags, kFlagBind);
    }
}

// ------------------------------------------------------------------ binding models
__device__ __forceinline__ int species(const BindModel &m, int idx) {
    switch (m.rule) {
    case 1: return idx < m.div1 ? 1 : 2;
    case 2: return idx < m.div1 ? 1 : (idx < m.div2 ? 2 : 3);
    case 3:
        if (idx < m.div1) return 1;
        if (idx < m.div2) return 2;
        return ((idx - m.div2) % m.np == m.np - 1) ? 3 : 1;
    default: return 1;
    }
}

__device__ __forceinline__ int pair_row(int a, int b) { return a == 1 ? b - 1 : (a == 2 ? b + 1 : 5); }
__device__ __forceinline__ int triple_row(int a, int b, int c) {
    if (a == 1) return b == 1 ? c - 1 : (b == 2 ? c + 1 : 5);
    if (a == 2) return 6 + (b == 2 ? c - 2 : 2);
    return 9;
}

// AbstractBindingModel::doublet (BindingModelSingle.cpp, BindingModelBinary.cpp, BindingModelTernary.cpp:523-560)
__device__ __forceinline__ bool doublet(const BindModel &m, bool before, int i1, int i2, double ran) {
    int s1 = species(m, i1), s2 = species(m, i2);
    if (s2 < s1) { const int t = s1; s1 = s2; s2 = t; }
    const double *rt = m.drate[pair_row(s1, s2)];
    const int st = before ? 1 : 0;
    const double r1 = rt[st * 2 + 0], r2 = rt[st * 2 + 1];
    return !(__dmul_rn(__dadd_rn(r1, r2), ran) < r1);
}

// sort_triplet_and_save_permutation (Basic/basic.h:166-230) -> permutation 0..5 = 123, 132, 312, 213, 231, 321
__device__ __forceinline__ int sort3(int a, int b, int c, int s[3]) {
    if (a <= b) {
        if (b <= c) { s[0] = a; s[1] = b; s[2] = c; return 0; }
        if (a <= c) { s[0] = a; s[1] = c; s[2] = b; return 1; }
        s[0] = c; s[1] = a; s[2] = b; return 2;
    }
    if (a <= c) { s[0] = b; s[1] = a; s[2] = c; return 3; }
    if (b <= c) { s[0] = b; s[1] = c; s[2] = a; return 4; }
    s[0] = c; s[1] = b; s[2] = a; return 5;
}

// save_to_type / inverse_save_to_type (Basic/basic.h:373-470) as slot maps over (12, 23, 13)
__device__ __forceinline__ int save_map(int perm, int k) {
    const int m = (perm == 0 ? 0x210 : perm == 1 ? 0x012 : perm == 2 ? 0x021 : perm == 3 ? 0x120 : perm == 4 ? 0x021 : 0x201);
    return (m >> (4 * k)) & 0xF;
}
__device__ __forceinline__ int unsave_map(int perm, int k) {
    const int m = (perm == 0 ? 0x210 : perm == 1 ? 0x012 : perm == 2 ? 0x021 : perm == 3 ? 0x120 : perm == 4 ? 0x102 : 0x201);
    return (m >> (4 * k)) & 0xF;
}

// AbstractBindingModel::triplet (BindingModelTernary.cpp:791-870): b, c, out over (12, 23, 13)
__device__ __forceinline__ void triplet(const BindModel &m, const bool b[3], const bool c[3], int i1, int i2, int i3,
                                        double ran, bool out[3]) {
    int st[3];
    const int perm = sort3(species(m, i1), species(m, i2), species(m, i3), st);
    bool tb[3], tc[3], ta[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        tb[k] = b[save_map(perm, k)];
        tc[k] = c[save_map(perm, k)];
    }
    const int state = tb[0] ? 0 : (tb[1] ? 1 : (tb[2] ? 2 : 3));
    const double *rt = m.trate[triple_row(st[0], st[1], st[2])];
    const double r1 = tc[0] ? rt[state * 4 + 0] : 0.0 * rt[state * 4 + 0];
    const double r2 = tc[1] ? rt[state * 4 + 1] : 0.0 * rt[state * 4 + 1];
    const double r3 = tc[2] ? rt[state * 4 + 2] : 0.0 * rt[state * 4 + 2];
    const double r4 = rt[state * 4 + 3];
    const double rr = __dmul_rn(__dadd_rn(__dadd_rn(__dadd_rn(r1, r2), r3), r4), ran);
    const double s12 = __dadd_rn(r1, r2), s123 = __dadd_rn(s12, r3);
    ta[0] = ta[1] = ta[2] = false;
    if (rr < r1) ta[0] = true;
    else if (rr >= r1 && rr < s12) ta[1] = true;
    else if (rr >= s12 && rr < s123) ta[2] = true;
#pragma unroll
    for (int k = 0; k < 3; k++) out[k] = ta[unsave_map(perm, k)];
}

// uniform [0, 1) of one binding decision: Philox4x32-10, counter (root patch, draw, replica), key
// (seed_lo + 0x2545F491 (iter + 1), seed_hi ^ 0x6A09E667), 53 bits of the first two output words
__device__ __forceinline__ double bind_uniform(const BindRep &B, int replica, unsigned long long draw, int root,
                                               int iter) {
    const uint2 key = make_uint2(B.seed_lo + 0x2545F491u * (unsigned)(iter + 1), B.seed_hi ^ 0x6A09E667u);
    const uint4 o = philox4x32_10(make_uint4((unsigned)root, (unsigned)draw, (unsigned)(draw >> 32), (unsigned)replica), key);
    const unsigned long long w = ((unsigned long long)o.y << 32) | o.x;
    return (double)(w >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ void set_pair(const BindState &S, int i1, int i2) {
    S.boundto[i1] = i2;
    S.boundto[i2] = i1;
    S.isbound[i1] = 1;
    S.isbound[i2] = 1;
}

__device__ __forceinline__ void apply_doublet(const BindState &S, const BindModel &m, int lo, int i1, int i2, double ran) {
    const bool already = S.boundto[i1] == i2 && S.boundto[i2] == i1 && S.isbound[i1] && S.isbound[i2];
    if (doublet(m, already, i1 - lo, i2 - lo, ran)) set_pair(S, i1, i2);
    else S.isbound[i1] = S.isbound[i2] = 0;
}

// connectivity flags of a triplet from its lowest member's degree / first neighbour and the middle one's
// degree (LangevinRforce.cpp:3230-3280); false where the reference calls error()
__device__ __forceinline__ bool triplet_links(int nb1, int first, int nb2, int m2, int m3, bool c[3]) {
    if (nb1 == 1) {
        if (first == m2) { c[0] = true; c[2] = false; c[1] = true; }
        else if (first == m3) { c[2] = true; c[0] = false; c[1] = true; }
        else return false;
    } else if (nb1 == 2) {
        c[0] = true;
        c[2] = true;
        c[1] = nb2 != 1;
    } else {
        return false;
    }
    return true;
}

__device__ __forceinline__ void apply_triplet(const BindState &S, const BindModel &m, int lo, int i1, int i2, int i3,
                                              const bool c[3], double ran) {
    const bool b[3] = {S.boundto[i1] == i2 && S.boundto[i2] == i1 && S.isbound[i1] && S.isbound[i2],
                       S.boundto[i2] == i3 && S.boundto[i3] == i2 && S.isbound[i2] && S.isbound[i3],
                       S.boundto[i1] == i3 && S.boundto[i3] == i1 && S.isbound[i1] && S.isbound[i3]};
    bool a[3];
    triplet(m, b, c, i1 - lo, i2 - lo, i3 - lo, ran, a);
    if (a[0]) { set_pair(S, i1, i2); S.isbound[i3] = 0; }
    else if (a[1]) { set_pair(S, i2, i3); S.isbound[i1] = 0; }
    else if (a[2]) { set_pair(S, i1, i3); S.isbound[i2] = 0; }
    else S.isbound[i1] = S.isbound[i2] = S.isbound[i3] = 0;
}

// a bond whose partner is not among this update's candidates breaks (LangevinRforce.cpp:3110-3133)
__device__ __forceinline__ void break_check(const BindState &S, int p, int d) {
    if (!S.isbound[p]) return;
    const int bt = S.boundto[p];
    for (int k = 0; k < d; k++)
        if (S.adj[(size_t)p * kAdjCap + k].x == bt) return;
    S.isbound[p] = 0;
}

// ------------------------------------------------------------------ clusters of up to three
__global__ void __launch_bounds__(256) bind_decide_kernel(BindState S) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= S.ptot) return;
    const unsigned stamp = (unsigned)S.ctr[2];
    const int d = adj_count(S.deg, p, stamp);
    if (d == 0) {  // a cluster of one: unbound (LangevinRforce.cpp:3165-3170)
        if (S.isbound[p]) S.isbound[p] = 0;
        return;
    }
    // breadth-first walk of p's component, stopped at a fourth member
    int m[4], nm = 1, lo = p;
    m[0] = p;
    for (int h = 0; h < nm && nm <= 3; h++) {
        const int v = m[h], dv = adj_count(S.deg, v, stamp);
        for (int k = 0; k < dv && nm <= 3; k++) {
            const int w = S.adj[(size_t)v * kAdjCap + k].x;
            bool seen = false;
            for (int t = 0; t < nm; t++) seen |= m[t] == w;
            if (!seen) {
                m[nm++] = w;
                lo = w < lo ? w : lo;
            }
        }
    }
    if (nm > 3) {  // larger cluster: every member queues, the smallest decides
        const unsigned long long at = atomicAdd(S.ctr + 1, 1ull);
        if ((long long)at < (long long)S.ptot) S.large[at] = p;
        return;
    }
    if (lo != p) return;
    const int r = find_replica(S.patch_slot, S.nrep, p);
    const BindRep &B = S.reps[r];
    const BindModel &mod = *S.model;
    for (int t = 0; t < nm; t++) break_check(S, m[t], adj_count(S.deg, m[t], stamp));
    const double ran = bind_uniform(B, r, S.draw[0], p - B.patch_off, 0);
    if (nm == 2) {
        const int i1 = m[0] < m[1] ? m[0] : m[1], i2 = m[0] < m[1] ? m[1] : m[0];
        apply_doublet(S, mod, B.patch_off, i1, i2, ran);
        return;
    }
    int s[3];
    sort3(m[0], m[1], m[2], s);
    bool c[3];
    const int d1 = adj_count(S.deg, s[0], stamp);
    if (!triplet_links(d1, S.adj[(size_t)s[0] * kAdjCap].x, adj_count(S.deg, s[1], stamp), s[1], s[2], c)) {
        atomicOr(S.flags, kFlagBind);
        return;
    }
    apply_triplet(S, mod, B.patch_off, s[0], s[1], s[2], c, ran);
}

// ------------------------------------------------------------------ larger clusters
// scratch of one thread (ints): members, component labels, reduced degrees and neighbours, edges (a, b, score)
constexpr int kScratchInts = kClusterCap * 6 + kClusterEdges * 4;

__device__ __forceinline__ int uf_root(int *lab, int v) {
    while (lab[v] != v) v = lab[v];
    return v;
}

template <class real>
__global__ void __launch_bounds__(kLargeThreads) bind_large_kernel(ForceArgs<real> a, BindState S) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= S.scratch_threads) return;
    int *W = S.scratch + (size_t)tid * kScratchInts;
    int *mem = W, *lab = W + kClusterCap, *lens = W + 2 * kClusterCap, *nbx = W + 3 * kClusterCap;
    int *ea = W + 6 * kClusterCap, *eb = ea + kClusterEdges;
    double *es = reinterpret_cast<double *>(eb + kClusterEdges);   // 8-byte aligned: offsets are even
    const unsigned stamp = (unsigned)S.ctr[2];
    const long long nq = (long long)S.ctr[1] < (long long)S.ptot ? (long long)S.ctr[1] : (long long)S.ptot;
    for (long long qi = tid; qi < nq; qi += S.scratch_threads) {
        const int p = S.large[qi];
        // the whole component, breadth first, up to the capacity
        int nm = 1, lo = p;
        bool over = false;
        mem[0] = p;
        for (int h = 0; h < nm && !over; h++) {
            const int v = mem[h], dv = adj_count(S.deg, v, stamp);
            for (int k = 0; k < dv; k++) {
                const int w = S.adj[(size_t)v * kAdjCap + k].x;
                bool seen = false;
                for (int t = 0; t < nm && !seen; t++) seen = mem[t] == w;
                if (seen) continue;
                if (nm == kClusterCap) { over = true; break; }
                mem[nm++] = w;
                lo = w < lo ? w : lo;
            }
        }
        if (over) {
            atomicOr(S.flags, kFlagBind);
            continue;
        }
        if (lo != p) continue;
        // members in increasing order (SingleHistogram, GraphAlgorithms.cpp:2-48)
        for (int i = 1; i < nm; i++) {
            const int v = mem[i];
            int j = i - 1;
            while (j >= 0 && mem[j] > v) { mem[j + 1] = mem[j]; j--; }
            mem[j + 1] = v;
        }
        const int r = find_replica(S.patch_slot, S.nrep, p);
        const BindRep &B = S.reps[r];
        const BindModel &mod = *S.model;
        for (int t = 0; t < nm; t++) break_check(S, mem[t], adj_count(S.deg, mem[t], stamp));
        // local edges (a < b) with their FP64 scores, sorted by (a, b) (RecapitulateEdges,
        // LangevinRforceUtil.cpp:508-572)
        int ne = 0;
        for (int j = 0; j < nm; j++) {
            const int v = mem[j], dv = adj_count(S.deg, v, stamp);
            for (int k = 0; k < dv; k++) {
                const int2 ad = S.adj[(size_t)v * kAdjCap + k];
                if (ad.x < v) continue;   // each edge from its lower patch
                int f2 = 0;
                while (f2 < nm && mem[f2] != ad.x) f2++;
                const Cand c = cand_of<real>(a, S, S.plist[ad.y >> 2]);
                double scr = 0;
                exact_edge<real>(B, a.buf, c.s1, c.s2, c.o1, c.o2, c.potn, disp2_of(B.disp[c.potn], ad.y & 3), &scr);
                int t = ne++;
                while (t > 0 && (ea[t - 1] > j || (ea[t - 1] == j && eb[t - 1] > f2))) {
                    ea[t] = ea[t - 1]; eb[t] = eb[t - 1]; es[t] = es[t - 1];
                    t--;
                }
                ea[t] = j; eb[t] = f2; es[t] = scr;
            }
        }
        // drop the first highest-scoring edge, then again while a piece has more than three patches
        bool first = true;
        int ncomp_big = 0;
        for (int guard = 0; guard <= kClusterEdges && ne > 0; guard++) {
            if (!first) {
                ncomp_big = 0;
                for (int v = 0; v < nm; v++) lab[v] = v;
                for (int q = 0; q < ne; q++) {
                    const int x = uf_root(lab, ea[q]), y = uf_root(lab, eb[q]);
                    if (x < y) lab[y] = x;
                    else if (y < x) lab[x] = y;
                }
                for (int v = 0; v < nm; v++) lens[v] = 0;
                for (int v = 0; v < nm; v++) lens[uf_root(lab, v)]++;
                for (int v = 0; v < nm; v++) ncomp_big = lens[v] > ncomp_big ? lens[v] : ncomp_big;
                if (ncomp_big <= 3) break;
            }
            first = false;
            int mx = 0;
            for (int q = 1; q < ne; q++)
                if (es[mx] < es[q]) mx = q;
            for (int q = mx; q + 1 < ne; q++) { ea[q] = ea[q + 1]; eb[q] = eb[q + 1]; es[q] = es[q + 1]; }
            ne--;
        }
        // components of what is left, labelled by their smallest member
        for (int v = 0; v < nm; v++) lab[v] = v;
        for (int q = 0; q < ne; q++) {
            const int x = uf_root(lab, ea[q]), y = uf_root(lab, eb[q]);
            if (x < y) lab[y] = x;
            else if (y < x) lab[x] = y;
        }
        for (int v = 0; v < nm; v++) lab[v] = uf_root(lab, v);
        // reduced adjacency (PairHistogram) and the second bond check against it
        for (int v = 0; v < nm; v++) lens[v] = 0;
        bool bad = false;
        for (int q = 0; q < ne; q++) {
            if (lens[ea[q]] >= 3 || lens[eb[q]] >= 3) { bad = true; break; }
            nbx[3 * ea[q] + lens[ea[q]]++] = eb[q];
            nbx[3 * eb[q] + lens[eb[q]]++] = ea[q];
        }
        if (bad) {
            atomicOr(S.flags, kFlagBind);
            continue;
        }
        for (int v = 0; v < nm; v++) {
            const int g = mem[v];
            if (!S.isbound[g]) continue;
            bool inside = false;
            for (int k = 0; k < lens[v]; k++) inside |= S.boundto[g] == mem[nbx[3 * v + k]];
            if (!inside) S.isbound[g] = 0;
        }
        // the pieces in order of their smallest member
        int it = 0;
        for (int v = 0; v < nm; v++) {
            if (lab[v] != v) continue;
            int pm[3], np_ = 0;
            for (int w = v; w < nm && np_ <= 3; w++)
                if (lab[w] == v) {
                    if (np_ < 3) pm[np_] = w;
                    np_++;
                }
            if (np_ == 1) {
                S.isbound[mem[pm[0]]] = 0;
            } else if (np_ == 2) {
                apply_doublet(S, mod, B.patch_off, mem[pm[0]], mem[pm[1]], bind_uniform(B, r, S.draw[0], p - B.patch_off, it));
                it++;
            } else if (np_ == 3) {
                bool c[3];
                if (!triplet_links(lens[pm[0]], nbx[3 * pm[0]], lens[pm[1]], pm[1], pm[2], c)) {
                    atomicOr(S.flags, kFlagBind);
                    break;
                }
                apply_triplet(S, mod, B.patch_off, mem[pm[0]], mem[pm[1]], mem[pm[2]], c,
                              bind_uniform(B, r, S.draw[0], p - B.patch_off, it));
                it++;
            } else {
                atomicOr(S.flags, kFlagBind);
                break;
            }
        }
    }
}

}  // namespace

}  // namespace mtg
