// mtg_pairs.cuh -- neighbour-pair export (MD::calculatepairs_parallel, MD.cpp:1100-1176) for one replica.
//
// Not on the step path (the step never materialises pairs); it exists so the pair SET of the cell
// list can be compared bit for bit with the reference.  The inclusion test is evaluated in FP64 with
// explicitly rounded operations, in the order of cube::distance_less_than (geometry.h:145-162), on the
// stored coordinates, so both sides decide every borderline pair identically.
#pragma once

#include "mtg_kernels.cuh"

namespace mtg {
namespace {  // internal linkage: every translation unit keeps its own kernels

struct PairGrid {
    int off;        // first slot of the replica
    int n;          // particles of the replica
    int nc;         // cells per side (side >= rc)
    double box;
    double scale;   // unused by the FP64 cell test (kept for symmetry with Replica)
    int periodic;
    double rc;
};

__device__ __forceinline__ int pair_axis_cell(double x, int nc, double box) {
    // cube::assign_box: fasterfloor(n * x / l), clamped to [0, n-1]
    double t = __ddiv_rn(__dmul_rn((double)nc, x), box);
    int m = t > 0.0 ? (int)t : (int)t - 1;
    m = m < 0 ? 0 : m;
    return m > nc - 1 ? nc - 1 : m;
}

__device__ __forceinline__ bool distance_less_than(const double xi[3], const double xj[3], double box, int periodic,
                                                   double val) {
    const double v2 = __dmul_rn(val, val);
    const double half = __dmul_rn(box, 0.5);
    double temp = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double dx = __dsub_rn(xi[k], xj[k]);
        if (periodic && fabs(dx) > half) dx = dx >= 0.0 ? __dsub_rn(dx, box) : __dadd_rn(dx, box);
        dx = __dmul_rn(dx, dx);
        if (dx > v2) return false;
        temp = __dadd_rn(temp, dx);
    }
    return temp < v2;
}

template <class real>
__device__ __forceinline__ void load_pos_d(const real *pos, int s, double x[3]) {
    real a, b, c;
    load_pos(pos + 4 * (size_t)s, a, b, c);
    x[0] = (double)a; x[1] = (double)b; x[2] = (double)c;
}

template <class real>
__global__ void pair_bin_kernel(PairGrid g, Buffers<real> in, int2 *bin, int *count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        double x[3];
        load_pos_d<real>(in.pos, g.off + i, x);
        int key = pair_axis_cell(x[0], g.nc, g.box) + g.nc * (pair_axis_cell(x[1], g.nc, g.box) +
                                                              g.nc * pair_axis_cell(x[2], g.nc, g.box));
        int rank = atomicAdd(count + key, 1);
        bin[i] = make_int2(key, rank);
    }
}

__global__ void pair_fill_kernel(PairGrid g, const int2 *bin, const int *start, int *members) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        int2 kb = bin[i];
        members[start[kb.x] + kb.y] = g.off + i;
    }
}

// visits every candidate partner j (any order) of slot s; calls f(local_j) for pairs within rc, j > i
template <class real, class Fn>
__device__ __forceinline__ void pair_visit(const PairGrid &g, const Buffers<real> &in, const int *start,
                                           const int *members, int s, int li, Fn f) {
    double xi[3];
    load_pos_d<real>(in.pos, s, xi);
    const int cx = pair_axis_cell(xi[0], g.nc, g.box), cy = pair_axis_cell(xi[1], g.nc, g.box),
              cz = pair_axis_cell(xi[2], g.nc, g.box);
    const int lo = g.nc >= 3 ? -1 : 0, hi = g.nc >= 2 ? 1 : 0;  // de-duplicated stencil (geometry.h:596-606)
    for (int dz = lo; dz <= hi; dz++)
        for (int dy = lo; dy <= hi; dy++)
            for (int dx = lo; dx <= hi; dx++) {
                int a = (cx + dx + g.nc) % g.nc, b = (cy + dy + g.nc) % g.nc, c = (cz + dz + g.nc) % g.nc;
                int cell = a + g.nc * (b + g.nc * c);
                for (int q = start[cell]; q < start[cell + 1]; q++) {
                    const int t = members[q];
                    const int lj = in.ident[t] - g.off;
                    if (lj <= li) continue;
                    double xj[3];
                    load_pos_d<real>(in.pos, t, xj);
                    // the reference tests (lower index, higher index) in that order
                    if (distance_less_than(xi, xj, g.box, g.periodic, g.rc)) f(lj);
                }
            }
}

template <class real>
__global__ void pair_count_kernel(PairGrid g, Buffers<real> in, const int *start, const int *members, int *cnt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int s = g.off + i;
        const int li = in.ident[s] - g.off;
        int c = 0;
        pair_visit<real>(g, in, start, members, s, li, [&](int) { c++; });
        cnt[li] = c;
    }
}

template <class real>
__global__ void pair_write_kernel(PairGrid g, Buffers<real> in, const int *start, const int *members, const int *offs,
                                  int32_t *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int s = g.off + i;
        const int li = in.ident[s] - g.off;
        int w = offs[li];
        pair_visit<real>(g, in, start, members, s, li, [&](int lj) {
            out[2 * (size_t)w] = li;
            out[2 * (size_t)w + 1] = lj;
            w++;
        });
    }
}

// ------------------------------------------------------------------ analysis passes on the pair grid

// cube::distance (geometry.h:107-121) with explicit FP64 roundings: dx = x_i - x_j, one image correction
// dx - SIGN(l, dx) when |dx| > l / 2, sqrt of the summed squares (symmetric in i, j bit for bit)
__device__ __forceinline__ double cube_distance(const double xi[3], const double xj[3], double box, int periodic) {
    const double half = __dmul_rn(box, 0.5);
    double temp = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double dx = __dsub_rn(xi[k], xj[k]);
        if (periodic && fabs(dx) > half) dx = dx >= 0.0 ? __dsub_rn(dx, box) : __dadd_rn(dx, box);
        temp = __dadd_rn(temp, __dmul_rn(dx, dx));
    }
    return __dsqrt_rn(temp);
}

// calcg1 (MDBase/Analysis/PairCorrelation.cpp:9-153): every unordered pair of the stencil once, bin
// floor(r / dr) when below nbins.  Counts go to a block histogram in shared memory (nbins <= smem_bins)
// or straight to global memory.
template <class real>
__global__ void pair_hist_kernel(PairGrid g, Buffers<real> in, const int *start, const int *members, double dr,
                                 int nbins, int smem_bins, unsigned long long *hist) {
    extern __shared__ unsigned long long hs[];
    const bool local = nbins <= smem_bins;
    if (local)
        for (int b = threadIdx.x; b < nbins; b += blockDim.x) hs[b] = 0ull;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int s = g.off + i;
        const int li = in.ident[s] - g.off;
        double xi[3];
        load_pos_d<real>(in.pos, s, xi);
        const int cx = pair_axis_cell(xi[0], g.nc, g.box), cy = pair_axis_cell(xi[1], g.nc, g.box),
                  cz = pair_axis_cell(xi[2], g.nc, g.box);
        const int lo = g.nc >= 3 ? -1 : 0, hi = g.nc >= 2 ? 1 : 0;
        for (int dz = lo; dz <= hi; dz++)
            for (int dy = lo; dy <= hi; dy++)
                for (int dx = lo; dx <= hi; dx++) {
                    int a = (cx + dx + g.nc) % g.nc, b = (cy + dy + g.nc) % g.nc, c = (cz + dz + g.nc) % g.nc;
                    int cell = a + g.nc * (b + g.nc * c);
                    for (int q = start[cell]; q < start[cell + 1]; q++) {
                        const int t = members[q];
                        if (in.ident[t] - g.off <= li) continue;
                        double xj[3];
                        load_pos_d<real>(in.pos, t, xj);
                        const double r = cube_distance(xi, xj, g.box, g.periodic);
                        const double f = floor(__ddiv_rn(r, dr));
                        if (f < (double)nbins) {
                            const int bin = (int)f;
                            if (local) atomicAdd(hs + bin, 1ull);
                            else atomicAdd(hist + bin, 1ull);
                        }
                    }
                }
    }
    __syncthreads();
    if (local)
        for (int b = threadIdx.x; b < nbins; b += blockDim.x)
            if (hs[b]) atomicAdd(hist + b, hs[b]);
}

// Connected components of the pairs closer than g.rc (distance_graph, AnalyzeGrowth.cpp:136-171) by
// union-find over local indices: a root is only ever hooked under a smaller root (compare-and-swap on
// the root's entry), so parent[i] <= i, every walk ends, and a component's final root is its smallest
// index -- the label ConnectedComponentsParallel_Old (GraphAlgorithms.cpp:672-800) converges to.
__device__ __forceinline__ int uf_find(const int *parent, int a, int limit, bool &ok) {
    for (int it = 0; it < limit; it++) {
        const int p = *(const volatile int *)(parent + a);
        if (p == a) return a;
        a = p;
    }
    ok = false;
    return a;
}

__global__ void uf_init_kernel(int n, int *parent) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) parent[i] = i;
}

// limit: the bound on every parent walk and on the compare-and-swap retries of one hook, which wait on the
// progress of other threads' hooks (n + 1 always suffices; a smaller caller limit may give up early).  A loop
// that reaches it stops, latches MTG_FLAG_TIMEOUT and the kernel returns normally.
template <class real>
__global__ void uf_hook_kernel(PairGrid g, Buffers<real> in, const int *start, const int *members, int *parent,
                               unsigned *flags, int limit) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int s = g.off + i;
        const int li = in.ident[s] - g.off;
        bool ok = true;
        pair_visit<real>(g, in, start, members, s, li, [&](int lj) {
            int u = li, v = lj;
            bool done = false;
            for (int it = 0; it < limit && ok; it++) {
                u = uf_find(parent, u, limit, ok);
                v = uf_find(parent, v, limit, ok);
                if (!ok) break;
                if (u == v) { done = true; break; }
                if (u < v) { const int t = u; u = v; v = t; }
                const int old = atomicCAS(parent + u, u, v);
                if (old == u) { done = true; break; }
                u = old;
            }
            if (!done) ok = false;
        });
        if (!ok) atomicOr(flags, 4u);
    }
}

__global__ void uf_label_kernel(int n, const int *parent, int32_t *labels, unsigned *flags, int limit) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool ok = true;
        labels[i] = uf_find(parent, i, limit, ok);
        if (!ok) atomicOr(flags, 4u);
    }
}

}  // namespace
}  // namespace mtg
