// mtg_bind.cuh -- single-bond-per-patch mode: the force pass of Condensate::run_singlebond
// (Condensate/Condensate.cpp:422-618), where every patch holds at most one bond and only bound patch
// pairs exert the Kern-Frenkel force.
//
// Per step (all replicas in every launch):
//   [begin]    one thread: this update's stamp; whether the candidate list is due (every patch_every steps
//              of the run_singlebond loop).  When it is, the scatter stores every particle's position and
//              rotation at the start of the step (the snapshot the candidate list is evaluated on);
//              otherwise particles carry their snapshot along.
//   [edges]    inside the force pass's pair loop (bind_pair_edges in mtg_kernels.cuh): every patch pair
//              that passes the current edge test and the candidate-list condition on the snapshot goes into
//              both patches' adjacency (stamped counters, no reset pass).
//   [decide]   one thread per patch: no edge -> unbound; else a breadth-first walk of its component.  The
//              component's smallest patch decides a cluster of two or three (doublet / triplet of the
//              binding model, LangevinRforce.cpp:3160-3480); members of larger components queue for:
//   [large]    one thread per queued patch; the smallest one runs the reference's reduction (drop the
//              highest-scoring edge until no piece exceeds three patches, LangevinRforce.cpp:3560-3880)
//              with its scratch in global memory.
// The bound pairs' forces are then added by the force epilogue (bound_patch_forces), from both ends.
#pragma once

#include <cooperative_groups.h>

#include "mtg_kernels.cuh"

namespace mtg {

constexpr int kClusterCap = 128;      // patches of one cluster reduced by one thread
constexpr int kClusterEdges = kClusterCap * kAdjCap / 2;
constexpr int kLargeThreads = 64;     // block of the large-cluster kernel

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
    unsigned long long *ctr;      // [1] queued large-cluster patches [2] update stamp [3] steps of the
                                  // run_singlebond loop so far [4] candidate list due this update
                                  // [5] patches with an edge (touched) [6] pairs listed for the edge pass
    unsigned long long *deg;      // per patch: stamp << 32 | edges of this update
    int2 *adj;                    // per patch kAdjCap: (partner patch, disp2 class)
    int *boundto;                 // global patch indices
    unsigned char *isbound;
    int *large;                   // queued patches of clusters above three
    int *touched;                 // patches with at least one edge in this update (kSegs segments of tcap)
    long long tcap;
    int2 *bound;                  // pairs bound by this update's decisions (kSegs segments of bcap), or null
    long long bcap;
    int *scratch;                 // large-cluster scratch, one block of kScratchInts per thread
    int scratch_threads;
    unsigned *flags;
    const unsigned long long *draw;
};

namespace {

__global__ void bind_begin_kernel(BindState S, int force, int advance) {
    if (threadIdx.x || blockIdx.x) return;
    const unsigned long long step = S.ctr[3];
    S.ctr[4] = force || (step > 0 && S.patch_every > 0 && step % (unsigned long long)S.patch_every == 0);
    S.ctr[1] = 0;
    for (int k = kSegPairs; k < kBindCounters; k++) S.ctr[k] = 0;
    S.ctr[2] += 1;
    if (advance) S.ctr[3] = step + 1;
}

// the candidate list is due now, at the current positions (a pass that does not move particles)
template <class real>
__global__ void __launch_bounds__(256) bind_snapshot_kernel(int ntot, Buffers<real> b) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ntot; s += gridDim.x * blockDim.x) {
        Payload<real> P;
        P.load(b.pos, b.rota, b.rotb, s);
        P.store(b.snap_a, b.snap_b, b.snap_c, b.ident[s]);   // by global index
    }
}

__device__ __forceinline__ int adj_count(const unsigned long long *deg, int p, unsigned stamp) {
    const unsigned long long w = deg[p];
    const int c = (unsigned)(w >> 32) == stamp ? (int)(unsigned)w : 0;
    return c < kAdjCap ? c : kAdjCap;
}

// slots, patch-vector rows and potential of the patch pair (w1, w2), w1 of the lower particle index
struct PatchPair {
    int s1, s2, o1, o2, potn;
};

template <class real>
__device__ __forceinline__ PatchPair patch_pair_of(const ForceArgs<real> &a, const BindRep &B, const Model<real> &M,
                                                   int off, int w1, int w2) {
    int l1, t1, k1, l2, t2, k2;
    patch_owner<real>(B, M, w1 - B.patch_off, l1, t1, k1);
    patch_owner<real>(B, M, w2 - B.patch_off, l2, t2, k2);
    if (l2 < l1) {
        int t;
        t = l1; l1 = l2; l2 = t;
        t = t1; t1 = t2; t2 = t;
        t = k1; k1 = k2; k2 = t;
    }
    PatchPair pp;
    pp.s1 = a.buf.slot_of[off + l1];
    pp.s2 = a.buf.slot_of[off + l2];
    pp.o1 = M.ooff[t1] + k1;
    pp.o2 = M.ooff[t2] + k2;
    pp.potn = M.pstart[t1][t2] + k1 * M.np[t2] + k2;
    return pp;
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
    if (S.bound) seg_append<int2>(S.bound, S.ctr + kSegBound, S.bcap, make_int2(i1, i2), S.flags);
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

// ------------------------------------------------------------------ clusters
// a patch without an edge is a cluster of one: unbound (LangevinRforce.cpp:3110-3133, 3165-3170)
// A thread takes 16 patches: their bound flags as one 16-byte word (the array is a cudaMalloc'd base and
// groups start at multiples of 16), then the adjacency counter of each bound one.
__global__ void __launch_bounds__(256) bind_unbind_kernel(BindState S) {
    const unsigned stamp = (unsigned)S.ctr[2];
    const int ngroups = (S.ptot + 15) / 16;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += gridDim.x * blockDim.x) {
        const int p0 = 16 * g;
        if (p0 + 16 <= S.ptot) {
            const uint4 v = *reinterpret_cast<const uint4 *>(S.isbound + p0);
            if (!(v.x | v.y | v.z | v.w)) continue;
            const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int b = 0; b < 16; b++)
                if (((w[b >> 2] >> (8 * (b & 3))) & 0xffu) && adj_count(S.deg, p0 + b, stamp) == 0) S.isbound[p0 + b] = 0;
        } else {
            for (int p = p0; p < S.ptot; p++)
                if (S.isbound[p] && adj_count(S.deg, p, stamp) == 0) S.isbound[p] = 0;
        }
    }
}

// clusters of two or three: the walk from one patch with an edge
__device__ __forceinline__ void decide_one(const BindState &S, int p, unsigned stamp) {
    const int d = adj_count(S.deg, p, stamp);
    // a patch with a partner below it is not its component's smallest patch, so it decides nothing (a cluster
    // of two or three is decided by its smallest patch, a larger one queued by a patch below all its partners):
    // it leaves before the walk
    for (int k = 0; k < d; k++)
        if (S.adj[(size_t)p * kAdjCap + k].x < p) return;
    if (d == 1) {
        // the common cluster, a doublet: p's one partner w has p as its one partner.  Both bond states are read
        // with w's degree, so the decision waits on memory once after p's own row.  The bond-breaking checks
        // of the general path leave no trace here: the decision writes both bound flags, and "already bound"
        // needs the two bound to each other, which no check breaks
        const int w = S.adj[(size_t)p * kAdjCap].x;
        const int dw = adj_count(S.deg, w, stamp);
        const bool bp = S.isbound[p] != 0, bw = S.isbound[w] != 0;
        const int btp = S.boundto[p], btw = S.boundto[w];
        const int r = find_replica(S.patch_slot, S.nrep, p);
        if (dw == 1) {
            const BindRep &B = S.reps[r];
            const double ran = bind_uniform(B, r, S.draw[0], p - B.patch_off, 0);
            const bool already = bp && bw && btp == w && btw == p;
            if (doublet(*S.model, already, p - B.patch_off, w - B.patch_off, ran)) set_pair(S, p, w);
            else S.isbound[p] = S.isbound[w] = 0;
            return;
        }
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
    if (nm > 3) {  // larger cluster: its smallest patch decides; patches below all their partners (p) queue
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
        atomicOr(S.flags, kFlagBind | kBindWhyRef);
        return;
    }
    apply_triplet(S, mod, B.patch_off, s[0], s[1], s[2], c, ran);
}

__global__ void __launch_bounds__(256) bind_decide_kernel(BindState S) {
    __shared__ long long segs[kSegs + 1];
    seg_prefix(S.ctr + kSegTouched, S.tcap, segs);
    const unsigned stamp = (unsigned)S.ctr[2];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < segs[kSegs]; i += (long long)gridDim.x * blockDim.x)
        decide_one(S, S.touched[seg_slot(segs, S.tcap, i)], stamp);
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
                if (w < p) { lo = w; break; }   // not the smallest: another queued patch decides
                if (nm == kClusterCap) { over = true; break; }
                mem[nm++] = w;
            }
            if (lo != p) break;
        }
        if (lo != p) continue;
        if (over) {
            atomicOr(S.flags, kFlagBind | kBindWhyCluster);
            continue;
        }
        // members in increasing order (SingleHistogram, GraphAlgorithms.cpp:2-48)
        for (int i = 1; i < nm; i++) {
            const int v = mem[i];
            int j = i - 1;
            while (j >= 0 && mem[j] > v) { mem[j + 1] = mem[j]; j--; }
            mem[j + 1] = v;
        }
        const int r = find_replica(S.patch_slot, S.nrep, p);
        const BindRep &B = S.reps[r];
        const Replica<real> &R = a.tb.reps[r];
        const Model<real> &M = a.tb.models[R.model];
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
                const PatchPair c = patch_pair_of<real>(a, B, M, R.off, v, ad.x);
                double scr = 0;
                exact_edge<real>(B, a.buf.pos, a.buf.rota, a.buf.rotb, c.s1, c.s2, c.o1, c.o2, c.potn,
                                 disp2_of(B.disp[c.potn], ad.y), &scr);
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
            atomicOr(S.flags, kFlagBind | kBindWhyRef);
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
                    atomicOr(S.flags, kFlagBind | kBindWhyRef);
                    break;
                }
                apply_triplet(S, mod, B.patch_off, mem[pm[0]], mem[pm[1]], mem[pm[2]], c,
                              bind_uniform(B, r, S.draw[0], p - B.patch_off, it));
                it++;
            } else {
                atomicOr(S.flags, kFlagBind | kBindWhyRef);
                break;
            }
        }
    }
}

// ------------------------------------------------------------------ random initial binding
// LangevinNVTR::setup_random_binding (LangevinRforceUtil.cpp:749-1010): every candidate patch pair that passes
// this update's edge test is an edge with score scr1 + scr2 + scr3 + scr4, scr4 = -log(1e-10 + the binding
// model's calculate_score); the edges are shuffled and taken in that order, each binding its two patches when
// both are unbound and its score is below 4.  The reference shuffles with std::random_device; here the order is
// ascending (Philox priority of the replica-local patch pair, lower patch, higher patch), seeded, so the result
// is reproducible and the oracle's greedy walk in the same order matches it.  Taking edges in a fixed order is
// the greedy matching of that order, which rounds of mutual choices reach on the GPU: every unbound patch picks
// its first live edge, and an edge both ends picked binds (the first live edge of the whole replica always is
// one, so every round binds, and the edges bound are the ones the greedy walk binds).

// -log(1e-10 + calculate_score(wp1, wp2, before)) per doublet row and prior state, computed on the host
struct SetupScores {
    double scr4[6][2];
};

// the doublet row calculate_score reads for (wp1 of the lower particle, wp2): BindingModelSingle one row;
// BindingModelBinary 11 if both are below div, 12 if only wp1 is, else 22 (BindingModelBinary.cpp:194-230);
// BindingModelTernary the sorted species pair (BindingModelTernary.cpp:596-640)
__device__ __forceinline__ int score_row(const BindModel &m, int i1, int i2) {
    if (m.rule == 0) return 0;
    if (m.rule == 1) return (i1 < m.div1 && i2 < m.div1) ? 0 : (i1 < m.div1 ? 1 : 3);
    int s1 = species(m, i1), s2 = species(m, i2);
    if (s2 < s1) { const int t = s1; s1 = s2; s2 = t; }
    return pair_row(s1, s2);
}

__device__ __forceinline__ uint32_t setup_priority(uint64_t seed, uint32_t replica, uint32_t lo, uint32_t hi) {
    return philox4x32_10(make_uint4(lo, hi, replica, 0x53455455u), make_uint2((uint32_t)seed, (uint32_t)(seed >> 32))).x;
}

// per adjacency entry of this update: whether the edge can bind (edge test and score below 4) and its priority
template <class real>
__global__ void __launch_bounds__(256) setup_edges_kernel(ForceArgs<real> a, BindState S, SetupScores sc,
                                                          uint64_t seed, uint32_t *prio, unsigned char *ok) {
    const unsigned stamp = (unsigned)S.ctr[2];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.ptot; p += gridDim.x * blockDim.x) {
        const int dp = adj_count(S.deg, p, stamp);
        if (!dp) continue;
        const int r = find_replica(S.patch_slot, S.nrep, p);
        const BindRep &B = S.reps[r];
        const Replica<real> &R = a.tb.reps[r];
        const Model<real> &M = a.tb.models[R.model];
        for (int k = 0; k < dp; k++) {
            const int2 ad = S.adj[(size_t)p * kAdjCap + k];
            const int q = ad.x;
            const PatchPair c = patch_pair_of<real>(a, B, M, R.off, p, q);
            double scr = 0;
            bool e = exact_edge<real>(B, a.buf.pos, a.buf.rota, a.buf.rotb, c.s1, c.s2, c.o1, c.o2, c.potn,
                                      disp2_of(B.disp[c.potn], ad.y), &scr);
            // wp1 is the patch of the lower particle index (the candidate list's order)
            int l1, t1, k1, l2, t2, k2;
            patch_owner<real>(B, M, p - B.patch_off, l1, t1, k1);
            patch_owner<real>(B, M, q - B.patch_off, l2, t2, k2);
            const int wp1 = (l1 < l2 ? p : q) - B.patch_off, wp2 = (l1 < l2 ? q : p) - B.patch_off;
            const bool before = S.isbound[p] && S.isbound[q] && S.boundto[p] == q && S.boundto[q] == p;
            e = e && __dadd_rn(scr, sc.scr4[score_row(*S.model, wp1, wp2)][before ? 1 : 0]) < 4.0;
            const int lo = (p < q ? p : q) - B.patch_off, hi = (p < q ? q : p) - B.patch_off;
            ok[(size_t)p * kAdjCap + k] = e ? 1 : 0;
            prio[(size_t)p * kAdjCap + k] = setup_priority(seed, (uint32_t)r, (uint32_t)lo, (uint32_t)hi);
        }
    }
}

// one round, first half: every unbound patch's first live edge (to an unbound patch), in (priority, lower
// patch, higher patch) order
__global__ void __launch_bounds__(256) setup_choose_kernel(BindState S, const uint32_t *prio, const unsigned char *ok,
                                                           int *best) {
    const unsigned stamp = (unsigned)S.ctr[2];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.ptot; p += gridDim.x * blockDim.x) {
        int b = -1;
        uint32_t bp = 0u;
        int blo = 0, bhi = 0;
        if (!S.isbound[p]) {
            const int dp = adj_count(S.deg, p, stamp);
            for (int k = 0; k < dp; k++) {
                const size_t e = (size_t)p * kAdjCap + k;
                const int q = S.adj[e].x;
                if (!ok[e] || S.isbound[q]) continue;
                const uint32_t pr = prio[e];
                const int lo = p < q ? p : q, hi = p < q ? q : p;
                if (b < 0 || pr < bp || (pr == bp && (lo < blo || (lo == blo && hi < bhi)))) {
                    b = q;
                    bp = pr;
                    blo = lo;
                    bhi = hi;
                }
            }
        }
        best[p] = b;
    }
}

// second half: an edge both of whose ends chose it binds; `bound` counts this round's bonds
__global__ void __launch_bounds__(256) setup_commit_kernel(BindState S, const int *best, unsigned long long *bound) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.ptot; p += gridDim.x * blockDim.x) {
        const int q = best[p];
        if (q <= p || best[q] != p) continue;
        S.isbound[p] = 1;
        S.isbound[q] = 1;
        S.boundto[p] = q;
        S.boundto[q] = p;
        atomicAdd(bound, 1ull);
    }
}

}  // namespace

}  // namespace mtg
