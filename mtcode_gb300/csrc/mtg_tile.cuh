// mtg_tile.cuh -- the FP32 force/torque + Langevin kernel of the batched path, one CTA per tile of cells.
//
// A tile is a block of cells of one replica: whole x-rows (or a chunk of one) x ty x tz rows.  Per tile:
//   stage   the positions of the tile and its one-cell halo (16 B per particle) are copied into shared
//           memory by cp.async.bulk (TMA bulk copies, one per contiguous row piece) on an mbarrier;
//           the wait is bounded and latches MTG_FLAG_TIMEOUT instead of hanging
//   phase 1 one thread per home particle scans its 27 cells in shared memory and appends every pair
//           within the force range to a shared pair list           (cheap, the only divergent loop)
//   phase 2 all threads take pairs evenly: WCA core, body-frame cone tests; every in-cone patch
//           potential is appended to a shared task list
//   phase 3 all threads take tasks evenly: Kern-Frenkel force/torque (the transcendental part)
//   phase 4 one thread per home particle: friction + Philox noise, half-kick, next-step binning
// Forces and torques are summed in 64-bit fixed point in shared memory (integer atomics commute), so
// the result does not depend on the order in which lanes or CTAs visit pairs.
#pragma once

#include "mtg_kernels.cuh"

namespace mtg {
namespace {  // internal linkage

constexpr int kTileThreads = 256;
constexpr int kTileYZMax = 4;
constexpr int kTileXMax = 32;
constexpr int kStageCells = (kTileXMax + 2) * (kTileYZMax + 2) * (kTileYZMax + 2);  // 1224
constexpr int kStageCap = 1536;   // staged particles per tile
constexpr int kPairCap = 2560;    // in-range pairs per chunk of home particles
constexpr int kTaskCap = 1024;    // in-cone patch potentials per chunk
constexpr unsigned kWaitSpins = 1u << 20;

// tile descriptor: x = replica, y = x0 | y0 << 10 | z0 << 20, z = sx | ty << 10 | tz << 15 | whole << 20 | simple << 21
// sx = staged cells per row (nc for whole rows, tx + 2 for a chunk), tx = sx - 2 for chunks.
struct TileShared {
    unsigned long long bar;
    int nstage, npairs, ntasks, nhome, abort_flag, overflow;
    int row_start[kTileYZMax * kTileYZMax + 1];  // prefix of home particles over home rows
    int cell_sm[kStageCells + 1];
    int cell_slot[kStageCells];
    float4 stage[kStageCap];
    unsigned long long acc[kTileThreads][6];
    int h_slot[kTileThreads], h_id[kTileThreads];
    short h_k[kTileThreads], h_cell[kTileThreads];
    int pair_slot[kPairCap];
    short pair_k[kPairCap];
    unsigned char pair_home[kPairCap];
    unsigned task[kTaskCap];
    int scan_ws[33];
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

struct TileGeom {
    int rep, x0, y0, z0, sx, ty, tz, whole, simple;
};
__device__ __forceinline__ TileGeom decode_tile(int4 t) {
    TileGeom g;
    g.rep = t.x;
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
    atomicAdd(a, (unsigned long long)__float2ll_rn(v * 4294967296.0f));
}
__device__ __forceinline__ float acc_get(unsigned long long a) {
    return __ll2float_rn((long long)a) * 2.3283064365386963e-10f;
}

// global cell of staged cell (sx_, sy, sz) in tile g, or -1 when it lies outside a walled box
__device__ __forceinline__ int staged_global_cell(const TileGeom &g, const Replica<float> &R, int sx_, int sy, int sz) {
    const int nc = R.nc;
    int gx = g.whole ? sx_ : g.x0 - 1 + sx_;
    int gy = g.y0 - 1 + sy, gz = g.z0 - 1 + sz;
    if (R.periodic) {
        gx = (gx + nc) % nc;
        gy = (gy + nc) % nc;
        gz = (gz + nc) % nc;
    } else if (gx < 0 || gx >= nc || gy < 0 || gy >= nc || gz < 0 || gz >= nc) {
        return -1;
    }
    return R.cell_off + gx + nc * (gy + nc * gz);
}

// the Langevin epilogue shared with the simple kernel (create_forces_and_torques_sphere + half-kick +
// binning of the next step); F, T are the lab-frame force and torque of slot s
__device__ __forceinline__ void langevin_epilogue(const ForceArgs<float> &a, const Replica<float> &R, int r, int s, int id,
                                                  const float F[3], const float T[3], const float Qi[9], float xi,
                                                  float yi, float zi) {
    Row<float> Mv;
    Mv.load(a.buf.motion + (size_t)s * kRow);
    float p[3] = {Mv.v[0], Mv.v[1], Mv.v[2]}, L[3] = {Mv.v[3], Mv.v[4], Mv.v[5]};
    float xi6[6];
    const int li = id - R.off;
    if (a.ext_noise) {
#pragma unroll
        for (int k = 0; k < 6; k++) xi6[k] = (float)a.ext_noise[6 * (size_t)id + k];
    } else {
        philox_noise6<float>((uint32_t)li, (uint32_t)r, a.draw[0], R.seed_lo, R.seed_hi, xi6);
    }
    float pb[3], fb[3], Ft[3], Tt[3];
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
    float xn[3] = {xi, yi, zi}, pn[3] = {p[0], p[1], p[2]};
    drift_position<float>(R, xn, pn, Ft);
    if (!(isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]))) {
        atomicOr(a.flags, 1u);
        xn[0] = xn[1] = xn[2] = 0.f;
    }
    const int key = cell_of<float>(R, xn[0], xn[1], xn[2]);
    const int rank = aggregated_rank(a.count, key);
    a.bin[s] = make_int2(key, rank);
}

__device__ __forceinline__ void load_q(const ForceArgs<float> &a, int slot, float q8, float Q[9]) {
    float b[4], c[4];
    load4(a.buf.rota + 4 * (size_t)slot, b);
    load4(a.buf.rotb + 4 * (size_t)slot, c);
    Q[0] = b[0]; Q[1] = b[1]; Q[2] = b[2]; Q[3] = b[3];
    Q[4] = c[0]; Q[5] = c[1]; Q[6] = c[2]; Q[7] = c[3]; Q[8] = q8;
}

// one in-cone patch potential q of pair p (phase 3, or immediately when the task list is full)
__device__ __noinline__ void eval_task(const ForceArgs<float> &a, const Replica<float> &R, const Model<float> &M,
                                       TileShared &sh, int p, int q) {
    const int h = sh.pair_home[p];
    const int kk = sh.pair_k[p], j = sh.pair_slot[p];
    const int ki = sh.h_k[h], si = sh.h_slot[h], idi = sh.h_id[h];
    const int idj = __ldg(a.buf.ident + j);
    const float4 pi = sh.stage[ki], pj = sh.stage[kk];
    float d[3] = {min_image<float>(pi.x - pj.x, R.box, R.l2s, R.periodic),
                  min_image<float>(pi.y - pj.y, R.box, R.l2s, R.periodic),
                  min_image<float>(pi.z - pj.z, R.box, R.l2s, R.periodic)};
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float rr = sqrtf(r2);
    const bool i_first = idi < idj;
    const float sg = i_first ? 1.f : -1.f, inv = 1.f / rr;
    const float u[3] = {sg * d[0] * inv, sg * d[1] * inv, sg * d[2] * inv};
    float Qi[9], Qj[9];
    load_q(a, si, pi.w, Qi);
    load_q(a, j, pj.w, Qj);
    const float *Qa = i_first ? Qi : Qj, *Qb = i_first ? Qj : Qi;
    const int ta = type_of<float>(M, (i_first ? idi : idj) - R.off);
    const int tb = type_of<float>(M, (i_first ? idj : idi) - R.off);
    const int nb = M.np[tb];
    const int rel = q - M.pstart[ta][tb];
    const int ia = rel / nb, ib = rel - ia * nb;
    const float *b1 = M.orient[M.ooff[ta] + ia], *b2 = M.orient[M.ooff[tb] + ib];
    float n1[3], n2[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        n1[k] = b1[0] * Qa[k] + b1[1] * Qa[3 + k] + b1[2] * Qa[6 + k];
        n2[k] = b2[0] * Qb[k] + b2[1] * Qb[3 + k] + b2[2] * Qb[6 + k];
    }
    // the cone test already passed in the body frame; the lab-frame cosines feed the force
    const float ci = -(n1[0] * u[0] + n1[1] * u[1] + n1[2] * u[2]);
    const float cj = n2[0] * u[0] + n2[1] * u[1] + n2[2] * u[2];
    float f[3] = {0, 0, 0}, tqa[3] = {0, 0, 0}, tqb[3] = {0, 0, 0}, e = 0;
    kf2_pair<float>(M.att[q], M.dis[q], M.inv_dis[q], M.kfac[q], u, rr, n1, n2, ci, cj, f, tqa, tqb, e);
    unsigned long long *acc = sh.acc[h];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        acc_add(acc + k, sg * f[k]);
        acc_add(acc + 3 + k, i_first ? tqa[k] : tqb[k]);
    }
}

// phase 2 body: WCA core + cone tests of pair p; in-cone potentials become tasks
__device__ __forceinline__ void eval_pair(const ForceArgs<float> &a, const Replica<float> &R, const Model<float> &M,
                                          TileShared &sh, int p, bool &big) {
    const int h = sh.pair_home[p];
    const int kk = sh.pair_k[p], j = sh.pair_slot[p];
    const int ki = sh.h_k[h];
    const float4 pi = sh.stage[ki], pj = sh.stage[kk];
    float d[3] = {min_image<float>(pi.x - pj.x, R.box, R.l2s, R.periodic),
                  min_image<float>(pi.y - pj.y, R.box, R.l2s, R.periodic),
                  min_image<float>(pi.z - pj.z, R.box, R.l2s, R.periodic)};
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float rr = sqrtf(r2);
    unsigned long long *acc = sh.acc[h];
    if (rr < R.hs_limit) {
        const float s_ = hs_force_over_r<float>(R, r2);
        big |= fabsf(s_ * rr) > 1e4f;
        acc_add(acc + 0, s_ * d[0]);
        acc_add(acc + 1, s_ * d[1]);
        acc_add(acc + 2, s_ * d[2]);
    }
    if (!(r2 < R.patch_r2)) return;
    const int idi = sh.h_id[h];
    const int idj = __ldg(a.buf.ident + j);
    const bool single = M.n_types == 1;
    const int ti = single ? 0 : type_of<float>(M, idi - R.off);
    const int tj = single ? 0 : type_of<float>(M, idj - R.off);
    if (M.np[ti] == 0 || M.np[tj] == 0) return;
    const bool i_first = idi < idj;
    const float sg = i_first ? 1.f : -1.f, inv = 1.f / rr;
    const float u[3] = {sg * d[0] * inv, sg * d[1] * inv, sg * d[2] * inv};
    float Qi[9], Qj[9];
    load_q(a, sh.h_slot[h], pi.w, Qi);
    load_q(a, j, pj.w, Qj);
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
            const int t = atomicAdd(&sh.ntasks, 1);
            if (t < kTaskCap) sh.task[t] = ((unsigned)p << 8) | (unsigned)q;
            else eval_task(a, R, M, sh, p, q);
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(kTileThreads) tile_force_kernel(ForceArgs<float> a, const int4 *tiles, int ntiles) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TileShared &sh = *reinterpret_cast<TileShared *>(smem_raw);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&sh.bar, 1);
        fence_proxy_async();
        sh.overflow = 0;
    }
    __syncthreads();
    unsigned phase = 0;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const TileGeom g = decode_tile(tiles[tile]);
        const Replica<float> &R = a.tb.reps[g.rep];
        const Model<float> &M = a.tb.models[R.model];

        if (g.simple) {
            // replicas with fewer than three cells per side: every particle by the per-thread path
            for (int s = R.off + tid; s < R.off + R.n; s += kTileThreads) simple_particle<float, MODE>(a, s);
            __syncthreads();
            continue;
        }
        const int nrows_y = g.ty + 2, nrows_z = g.tz + 2;
        const int ncells_staged = g.sx * nrows_y * nrows_z;

        // ---- staged cell table: counts, block-wide exclusive scan -> shared offsets
        constexpr int kItems = (kStageCells + kTileThreads - 1) / kTileThreads;
        int cnt[kItems], gc[kItems];
        int local = 0;
#pragma unroll
        for (int it = 0; it < kItems; it++) {
            const int c = tid * kItems + it;
            cnt[it] = 0;
            gc[it] = -1;
            if (c < ncells_staged) {
                const int sx_ = c % g.sx, sy = (c / g.sx) % nrows_y, sz = c / (g.sx * nrows_y);
                gc[it] = staged_global_cell(g, R, sx_, sy, sz);
                if (gc[it] >= 0) cnt[it] = __ldg(a.start + gc[it] + 1) - __ldg(a.start + gc[it]);
            }
            local += cnt[it];
        }
        int total;
        int off = block_exclusive_scan(local, sh.scan_ws, total);
#pragma unroll
        for (int it = 0; it < kItems; it++) {
            const int c = tid * kItems + it;
            if (c < ncells_staged) {
                sh.cell_sm[c] = off;
                sh.cell_slot[c] = gc[it] >= 0 ? __ldg(a.start + gc[it]) : 0;
            }
            off += cnt[it];
        }
        if (tid == 0) {
            sh.cell_sm[ncells_staged] = total;
            sh.nstage = total;
        }
        __syncthreads();

        if (total > kStageCap) {
            // too crowded to stage: the per-thread path over the home rows (slots are contiguous per row)
            const int hx0 = g.whole ? 0 : 1, hx1 = g.whole ? g.sx : g.sx - 1;
            for (int rz = 1; rz <= g.tz; rz++)
                for (int ry = 1; ry <= g.ty; ry++) {
                    const int base = (rz * nrows_y + ry) * g.sx;
                    const int s0 = sh.cell_slot[base + hx0];
                    const int s1 = sh.cell_slot[base + hx1 - 1] + (sh.cell_sm[base + hx1] - sh.cell_sm[base + hx1 - 1]);
                    for (int s = s0 + tid; s < s1; s += kTileThreads) simple_particle<float, MODE>(a, s);
                }
            __syncthreads();
            continue;
        }

        // ---- TMA bulk copies of the staged positions (one per contiguous piece of a staged row)
        if (tid == 0) {
            fence_proxy_async();
            mbar_arrive_expect_tx(&sh.bar, (unsigned)total * 16u);
        }
        __syncthreads();
        if (tid < nrows_y * nrows_z) {
            fence_proxy_async();  // this thread's earlier generic reads of the buffer precede the copies
            const int base = tid * g.sx;
            int c = 0;
            while (c < g.sx) {
                // extend the piece while the global cells stay consecutive
                const int g0 = sh.cell_slot[base + c];
                int e = c + 1;
                const int gcell0 = staged_global_cell(g, R, c, tid % nrows_y, tid / nrows_y);
                if (gcell0 < 0) { c = e; continue; }
                while (e < g.sx) {
                    const int gce = staged_global_cell(g, R, e, tid % nrows_y, tid / nrows_y);
                    if (gce != gcell0 + (e - c)) break;
                    e++;
                }
                const int bytes = (sh.cell_sm[base + e] - sh.cell_sm[base + c]) * 16;
                if (bytes > 0)
                    bulk_copy_g2s(&sh.stage[sh.cell_sm[base + c]], a.buf.pos + 4 * (size_t)g0, (unsigned)bytes, &sh.bar);
                c = e;
            }
        }
        // bounded wait for the copies
        bool done = false;
        for (unsigned it = 0; it < kWaitSpins && !done; it++) done = mbar_try_wait(&sh.bar, phase);
        if (__syncthreads_or(!done)) {
            if (tid == 0) atomicOr(a.flags, 4u);
            for (unsigned it = 0; it < kWaitSpins && !done; it++) done = mbar_try_wait(&sh.bar, phase);
            return;
        }
        phase ^= 1u;

        // ---- home particles: the inner rows, contiguous in shared memory per row
        const int hx0 = g.whole ? 0 : 1, hx1 = g.whole ? g.sx : g.sx - 1;
        if (tid == 0) {
            int acc_rows = 0;
            for (int r = 0; r < g.ty * g.tz; r++) {
                const int ry = 1 + r % g.ty, rz = 1 + r / g.ty;
                const int base = (rz * nrows_y + ry) * g.sx;
                sh.row_start[r] = acc_rows;
                acc_rows += sh.cell_sm[base + hx1] - sh.cell_sm[base + hx0];
            }
            sh.row_start[g.ty * g.tz] = acc_rows;
            sh.nhome = acc_rows;
        }
        __syncthreads();
        const int nhome = sh.nhome;
        bool big = false;

        for (int c0 = 0; c0 < nhome; c0 += kTileThreads) {
            const int nchunk = min(kTileThreads, nhome - c0);
            // -- locate this thread's home particle
            int myk = -1, mycell = -1;
            if (tid < nchunk) {
                const int hidx = c0 + tid;
                int r = 0;
                while (sh.row_start[r + 1] <= hidx) r++;
                const int ry = 1 + r % g.ty, rz = 1 + r / g.ty;
                const int base = (rz * nrows_y + ry) * g.sx;
                myk = sh.cell_sm[base + hx0] + (hidx - sh.row_start[r]);
                int lo = hx0, hi = hx1;  // cell_sm[base+lo] <= myk < cell_sm[base+hi]
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (sh.cell_sm[base + mid] <= myk) lo = mid;
                    else hi = mid;
                }
                mycell = base + lo;
                const int slot = sh.cell_slot[mycell] + (myk - sh.cell_sm[mycell]);
                sh.h_k[tid] = (short)myk;
                sh.h_cell[tid] = (short)mycell;
                sh.h_slot[tid] = slot;
                sh.h_id[tid] = __ldg(a.buf.ident + slot);
#pragma unroll
                for (int k = 0; k < 6; k++) sh.acc[tid][k] = 0ull;
            }
            if (tid == 0) {
                sh.npairs = 0;
                sh.ntasks = 0;
            }
            __syncthreads();

            // -- phase 1: candidate scan in shared memory
            if (tid < nchunk) {
                const float4 pi = sh.stage[myk];
                const int lx = mycell % g.sx, ly = (mycell / g.sx) % nrows_y, lz = mycell / (g.sx * nrows_y);
                for (int dz = -1; dz <= 1; dz++)
                    for (int dy = -1; dy <= 1; dy++) {
                        const int rowb = ((lz + dz) * nrows_y + (ly + dy)) * g.sx;
                        for (int dx = -1; dx <= 1; dx++) {
                            int cx = lx + dx;
                            if (g.whole) {
                                if (cx < 0 || cx >= g.sx) {
                                    if (!R.periodic) continue;
                                    cx = cx < 0 ? cx + g.sx : cx - g.sx;
                                }
                            }
                            const int cell = rowb + cx;
                            const int k0 = sh.cell_sm[cell], k1 = sh.cell_sm[cell + 1];
                            for (int kk = k0; kk < k1; kk++) {
                                if (kk == myk) continue;
                                const float4 pj = sh.stage[kk];
                                const float dx_ = min_image<float>(pi.x - pj.x, R.box, R.l2s, R.periodic);
                                const float dy_ = min_image<float>(pi.y - pj.y, R.box, R.l2s, R.periodic);
                                const float dz_ = min_image<float>(pi.z - pj.z, R.box, R.l2s, R.periodic);
                                if (dx_ * dx_ + dy_ * dy_ + dz_ * dz_ < R.rc2) {
                                    const int p = atomicAdd(&sh.npairs, 1);
                                    if (p < kPairCap) {
                                        sh.pair_k[p] = (short)kk;
                                        sh.pair_slot[p] = sh.cell_slot[cell] + (kk - k0);
                                        sh.pair_home[p] = (unsigned char)tid;
                                    }
                                }
                            }
                        }
                    }
            }
            __syncthreads();
            if (sh.npairs > kPairCap) {
                // more pairs than the list holds: this chunk goes through the per-thread path instead
                if (tid < nchunk) simple_particle<float, MODE>(a, sh.h_slot[tid]);
                if (tid == 0) sh.overflow = 1;
                __syncthreads();
                continue;
            }
            const int npairs = sh.npairs;

            // -- phase 2: pairs spread over all threads
            for (int p = tid; p < npairs; p += kTileThreads) eval_pair(a, R, M, sh, p, big);
            __syncthreads();
            // -- phase 3: in-cone patch potentials spread over all threads
            const int ntasks = min(sh.ntasks, kTaskCap);
            for (int t = tid; t < ntasks; t += kTileThreads) eval_task(a, R, M, sh, (int)(sh.task[t] >> 8), (int)(sh.task[t] & 255u));
            __syncthreads();

            // -- phase 4: epilogue per home particle
            if (tid < nchunk) {
                const int s = sh.h_slot[tid];
                const float F[3] = {acc_get(sh.acc[tid][0]), acc_get(sh.acc[tid][1]), acc_get(sh.acc[tid][2])};
                const float T[3] = {acc_get(sh.acc[tid][3]), acc_get(sh.acc[tid][4]), acc_get(sh.acc[tid][5])};
                if (MODE == kModeForces) {
                    const int id = sh.h_id[tid];
                    for (int k = 0; k < 3; k++) {
                        a.outF[3 * (size_t)id + k] = F[k];
                        a.outT[3 * (size_t)id + k] = T[k];
                    }
                } else {
                    const float4 pi = sh.stage[myk];
                    float Qi[9];
                    load_q(a, s, pi.w, Qi);
                    langevin_epilogue(a, R, g.rep, s, sh.h_id[tid], F, T, Qi, pi.x, pi.y, pi.z);
                }
            }
            __syncthreads();
        }
        if (big) atomicOr(a.flags, 2u);
    }
    if (tid == 0 && sh.overflow) atomicOr(a.flags, 8u);
}

}  // namespace
}  // namespace mtg
