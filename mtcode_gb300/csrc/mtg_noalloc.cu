// mtg_noalloc.cu -- neighbour-pair build that allocates nothing (mtg_pairs_noalloc).
//
// Some callers cannot allocate device memory at the time they need the pair list: code running
// inside another framework's memory pool or allocator hooks, a process whose device memory is
// reserved up front by its host application, or a driver loop that must not call into the CUDA
// allocator between steps.  For them this entry point works only on buffers the caller owns plus one
// fixed scratch area that lives inside this library: a file-scope __device__ array of
// kNoAllocScratchBytes bytes, which every GPU that loads the library holds until the process exits.
//
// Host code cannot use the array's symbol as a device address (on the host it names a stand-in
// object), so on the first call on each device this file asks the runtime for the array's device
// address with cudaGetSymbolAddress, with that device current, and passes the address to the
// kernels.  That first call should therefore come before any stream capture.  The address is kept for
// the life of the process, so the library must not be used across cudaDeviceReset on that device (the
// reset unloads the module that holds the array).
//
// All calls share the one scratch area and it keeps the last call's contents: each call clears the
// parts that must start at zero, and calls whose work overlaps on the GPU (different streams, or
// different host threads on the same device) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/mtcode_gb300.h"
#include "mtg_pairs.cuh"

namespace {

constexpr int kNoAllocMaxParticles = MTG_NOALLOC_MAX_PARTICLES;
constexpr int kNoAllocMaxCells = MTG_NOALLOC_MAX_CELLS;

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr int kNoAllocMaxBlocks = kNoAllocMaxCells / mtg::kScanTile + 2;
// scratch layout: cell histogram and starts, cell block sums, per-particle (cell, rank),
// members in cell order, per-particle pair counts and offsets, particle block sums
constexpr size_t kOffCount = 0;
constexpr size_t kOffStart = kOffCount + align256(sizeof(int) * (kNoAllocMaxCells + 1));
constexpr size_t kOffCellBlk = kOffStart + align256(sizeof(int) * (kNoAllocMaxCells + 1));
constexpr size_t kOffBin = kOffCellBlk + align256(sizeof(int) * kNoAllocMaxBlocks);
constexpr size_t kOffMembers = kOffBin + align256(sizeof(int2) * kNoAllocMaxParticles);
constexpr size_t kOffPcnt = kOffMembers + align256(sizeof(int) * kNoAllocMaxParticles);
constexpr size_t kOffPoff = kOffPcnt + align256(sizeof(int) * (kNoAllocMaxParticles + 1));
constexpr size_t kOffPartBlk = kOffPoff + align256(sizeof(int) * (kNoAllocMaxParticles + 1));
constexpr size_t kNoAllocScratchBytes = kOffPartBlk + align256(sizeof(int) * kNoAllocMaxBlocks);
// 1,836,544 bytes with 4096-entry scan tiles: the figure the documentation quotes
static_assert(kNoAllocScratchBytes == 1836544, "the documented scratch size no longer matches the layout");

__device__ __align__(256) static unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kMaxDevices] = {};
// the status is the whole report: this entry point keeps no error text
mtg_status fail(mtg_status st, const std::string &) { return st; }

// device address of the scratch array on the current device (looked up once per device)
mtg_status scratch_address(int device, unsigned char **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(MTG_ERR_CUDA, std::string("mtg_pairs_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_ptr[device] = p;
    }
    *out = static_cast<unsigned char *>(g_noalloc_ptr[device]);
    return MTG_OK;
}

struct NoAllocGrid {
    const double *x;  // n x 3, row-major (the reference's matrix<double> layout)
    int n, nc;
    double box, rc;
    int periodic;
};

__device__ __forceinline__ void load_x(const NoAllocGrid &g, int i, double v[3]) {
    v[0] = g.x[3 * (size_t)i];
    v[1] = g.x[3 * (size_t)i + 1];
    v[2] = g.x[3 * (size_t)i + 2];
}

__global__ void noalloc_bin(NoAllocGrid g, int2 *bin, int *count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        double v[3];
        load_x(g, i, v);
        const int key = mtg::pair_axis_cell(v[0], g.nc, g.box) +
                        g.nc * (mtg::pair_axis_cell(v[1], g.nc, g.box) + g.nc * mtg::pair_axis_cell(v[2], g.nc, g.box));
        bin[i] = make_int2(key, atomicAdd(count + key, 1));
    }
}

__global__ void noalloc_fill(NoAllocGrid g, const int2 *bin, const int *start, int *members) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int2 kb = bin[i];
        members[start[kb.x] + kb.y] = i;
    }
}

// partners j > i of particle i within rc, in the reference's inclusion test; f(j) for each
template <class Fn>
__device__ __forceinline__ void noalloc_visit(const NoAllocGrid &g, const int *start, const int *members, int i, Fn f) {
    double xi[3];
    load_x(g, i, xi);
    const int cx = mtg::pair_axis_cell(xi[0], g.nc, g.box), cy = mtg::pair_axis_cell(xi[1], g.nc, g.box),
              cz = mtg::pair_axis_cell(xi[2], g.nc, g.box);
    const int lo = g.nc >= 3 ? -1 : 0, hi = g.nc >= 2 ? 1 : 0;
    for (int dz = lo; dz <= hi; dz++)
        for (int dy = lo; dy <= hi; dy++)
            for (int dx = lo; dx <= hi; dx++) {
                const int a = (cx + dx + g.nc) % g.nc, b = (cy + dy + g.nc) % g.nc, c = (cz + dz + g.nc) % g.nc;
                const int cell = a + g.nc * (b + g.nc * c);
                for (int q = start[cell]; q < start[cell + 1]; q++) {
                    const int j = members[q];
                    if (j <= i) continue;
                    double xj[3];
                    load_x(g, j, xj);
                    if (mtg::distance_less_than(xi, xj, g.box, g.periodic, g.rc)) f(j);
                }
            }
}

__global__ void noalloc_count(NoAllocGrid g, const int *start, const int *members, int *pcnt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        int c = 0;
        noalloc_visit(g, start, members, i, [&](int) { c++; });
        pcnt[i] = c;
    }
}

__global__ void noalloc_write(NoAllocGrid g, const int *start, const int *members, const int *poff, int32_t *pairs,
                              int64_t cap) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        int64_t w = poff[i];
        noalloc_visit(g, start, members, i, [&](int j) {
            if (w < cap) {
                pairs[2 * w] = i;
                pairs[2 * w + 1] = j;
            }
            w++;
        });
    }
}

__global__ void noalloc_total(const int *poff, int n, int64_t *npairs) { *npairs = (int64_t)poff[n]; }

void run_scan(int *count, int n, int *blocks, int *start, cudaStream_t st) {
    const int nblk = n > 0 ? (n + mtg::kScanTile - 1) / mtg::kScanTile : 1;
    mtg::scan_reduce_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(count, n, blocks);
    mtg::scan_top_kernel<<<1, mtg::kScanThreads, 0, st>>>(blocks, nblk, start, n, nullptr, 0);
    mtg::scan_down_kernel<<<nblk, mtg::kScanThreads, 0, st>>>(count, n, blocks, start);
}

}  // namespace

extern "C" {

mtg_status mtg_pairs_noalloc(const double *x_dev, int n, double box, int periodic, double rc, int32_t *pairs_dev,
                             int64_t cap, int64_t *npairs_dev, void *stream) {
    if (n < 0 || !(box > 0) || !(rc > 0) || !npairs_dev || (n > 0 && !x_dev) || cap < 0 || (cap > 0 && !pairs_dev))
        return fail(MTG_ERR_ARG, "mtg_pairs_noalloc: invalid argument");
    if (n > kNoAllocMaxParticles)
        return fail(MTG_ERR_ARG, "mtg_pairs_noalloc: n = " + std::to_string(n) + " exceeds the maximum of " +
                                     std::to_string(kNoAllocMaxParticles) + " particles");
    const double cells = std::floor(box / (rc * (1 + 1e-12)));
    const int nc = cells < 1 ? 1 : (cells > 1e4 ? 10000 : (int)cells);
    const long long ncell = (long long)nc * nc * nc;
    if (ncell > kNoAllocMaxCells)
        return fail(MTG_ERR_ARG, "mtg_pairs_noalloc: box / rc gives " + std::to_string(ncell) +
                                     " cells, more than the maximum of " + std::to_string(kNoAllocMaxCells));
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices)
        return fail(MTG_ERR_NODEVICE, "mtg_pairs_noalloc: no current CUDA device");
    unsigned char *scratch = nullptr;
    mtg_status st0 = scratch_address(device, &scratch);
    if (st0 != MTG_OK) return st0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int *count = reinterpret_cast<int *>(scratch + kOffCount);
    int *start = reinterpret_cast<int *>(scratch + kOffStart);
    int *cellblk = reinterpret_cast<int *>(scratch + kOffCellBlk);
    int2 *bin = reinterpret_cast<int2 *>(scratch + kOffBin);
    int *members = reinterpret_cast<int *>(scratch + kOffMembers);
    int *pcnt = reinterpret_cast<int *>(scratch + kOffPcnt);
    int *poff = reinterpret_cast<int *>(scratch + kOffPoff);
    int *partblk = reinterpret_cast<int *>(scratch + kOffPartBlk);
    // the histogram must start at zero; everything else is written before it is read
    if (cudaMemsetAsync(count, 0, sizeof(int) * (ncell + 1), st) != cudaSuccess)
        return fail(MTG_ERR_CUDA, "mtg_pairs_noalloc: cudaMemsetAsync failed");
    NoAllocGrid g{x_dev, n, nc, box, rc, periodic ? 1 : 0};
    const int blocks = n > 0 ? (n + 255) / 256 : 1;
    if (n > 0) noalloc_bin<<<blocks, 256, 0, st>>>(g, bin, count);
    run_scan(count, (int)ncell, cellblk, start, st);
    if (n > 0) {
        noalloc_fill<<<blocks, 256, 0, st>>>(g, bin, start, members);
        noalloc_count<<<blocks, 256, 0, st>>>(g, start, members, pcnt);
    }
    run_scan(pcnt, n, partblk, poff, st);
    if (n > 0 && cap > 0) noalloc_write<<<blocks, 256, 0, st>>>(g, start, members, poff, pairs_dev, cap);
    noalloc_total<<<1, 1, 0, st>>>(poff, n, npairs_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MTG_ERR_CUDA, std::string("mtg_pairs_noalloc: ") + cudaGetErrorString(e));
    return MTG_OK;
}

}  // extern "C"
