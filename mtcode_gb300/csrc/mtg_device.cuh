// mtg_device.cuh -- device-side data layout and per-pair physics of the GB300 patchy-Langevin step.
//
// HBM layout (one handle, all replicas concatenated; "slot" = position in cell-sorted order):
//   pos[slot]      4 reals   (x, y, z, Q8)       the only array neighbour scans read (16 B in FP32)
//   rota[slot]     4 reals   (Q0, Q1, Q2, Q3)    read for in-range pairs only
//   rotb[slot]     4 reals   (Q4, Q5, Q6, Q7)
//   motion[slot]   12 reals  (px, py, pz, Lx | Ly, Lz, F~x, F~y | F~z, T~x, T~y, T~z)
//   ident[slot]    int32 global particle index (replica offset + reference particle index)
//   disp_{x,y,z}   FP64 unwrapped displacement (SoA, optional)
//   bin[slot]      int2 (global cell, rank inside the cell) of the particle's NEXT position
//   cell_count / cell_start   per global cell (replica cell blocks are contiguous)
// Every element is 16 B (FP32) or 32 B (FP64) aligned, so rows move as float4/double2 vectors.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mtg {

constexpr int kMaxTypes = 4;
constexpr int kMaxOrient = 16;
constexpr int kMaxPots = 64;
constexpr int kRow = 12;  // reals per motion row

// ------------------------------------------------------------------ per-replica constants
template <class real>
struct Replica {
    int n;            // particles
    int off;          // first slot / global particle index
    int cell_off;     // first global cell
    int nc;           // cells per side of the force grid
    uint32_t nc_mul;  // n / nc = umulhi(n, nc_mul) >> nc_sh for 0 <= n < nc^3 (nc_magic)
    int nc_sh;
    int periodic;
    int model;        // index into the model table
    uint32_t seed_lo, seed_hi;
    real box, half_box, l2s;   // cube::l, l/2, (l/2)^2
    real box_lo;               // FP32: l - (float)l, the part of the double box length a float drops (0 in FP64)
    real cell_scale;           // nc / box  (cube::assign_box: n * x / l)
    real dt, half_dt, c1;      // dt, dt/2, dt/m
    real fric_t, fric_r;       // -gamma/m, -gammar/I
    real Rt, Rr;               // sqrt(2 gamma kT / dt), sqrt(2 gammar kT / dt)
    real inertia;
    real hs_limit, hs_4eps, hs_s6, hs_s12, hs_eps;  // HSPotential: 1.12246 sigma, 4 eps, sigma^6, sigma^12
    real max_dist2;            // LangevinNVTR::max_distance_check
    real rc2;                  // squared force range (max of HS range and patch range)
    real patch_r2;             // squared range of any patch force: min(max_dist2, (1.4 dis_max)^2)
    real rc2_list;             // skin lists: squared list range (force range + skin, padded for rounding)
    real rc2_find, rc2_list_find;   // pair finding's ranges: rc2 / rc2_list widened by the rounding of its cheaper
                                    // separation, (x_a - x_b) - shift; the pair kernels keep the exact test
    real half_skin2;           // skin lists: (skin / 2)^2, the displacement that forces a rebuild
    real bond_r;               // ComboPatch::max_check
};

// n / nc for a cell key 0 <= n < nc^3 of replica R's force grid, without an integer division
template <class real>
__device__ __forceinline__ int div_nc(const Replica<real> &R, int n) {
    return (int)(__umulhi((unsigned)n, R.nc_mul) >> R.nc_sh);
}

// ------------------------------------------------------------------ single-bond-per-patch mode, per replica
// Patch numbering (GeneralPatch, GeneralPatch.cpp:285-320) and the constants of the bond tests.  The FP64
// values are the reference's thresholds; the float pairs bracket them by a margin far above the error of
// a float evaluation, so that a float value outside [lo, hi] decides like the FP64 test.
struct BindRep {
    int patch_off, npatch;
    int pbase[kMaxTypes + 1];     // first local patch of each type; pbase[n_types] = patches of the replica
    int periodic;
    uint32_t seed_lo, seed_hi;
    double box, l2s;              // cube::l, (l/2)^2
    double orient[kMaxOrient][3]; // body-frame patch vectors
    double ctm[kMaxPots];         // cos(thetam) of each potential
    double disp[kMaxPots];        // interaction_distance = 1.4 dis (potentialtheta.h:416)
    double mk2;                   // ComboPatch::max_check^2
    double max_dis;               // max_check + 1 (calculate_patch_list)
    double list_cut2;             // squared pair-list cut the candidates come from (run_singlebond: 2.5 sigma)
    double max_ang;               // ComboPatch::max_ang
    float ctm_lo[kMaxPots], ctm_hi[kMaxPots];   // cos(thetam) -+ 2e-5
    float disp_f[kMaxPots];                     // interaction_distance in float
    float mk2_lo, mk2_hi;                       // max_check^2 (1 -+ 1e-5)
    float memb2_lo, memb2_hi;                   // min(list_cut^2, (max_check + 1)^2) (1 -+ 1e-5)
    float ang_lo, ang_hi;                       // -0.4 -+ 4e-5 for (c_i - max_ang) + (c_j - max_ang)
    float max_ang_f;
};

// ------------------------------------------------------------------ patch model (GeneralPatch form)
template <class real>
struct Model {
    int n_types;
    int np[kMaxTypes];            // patches per type
    int ncum[kMaxTypes];          // cumulative particle counts
    int ooff[kMaxTypes];          // first orientation row of each type
    int pstart[kMaxTypes][kMaxTypes];  // first potential of type pair (k1 <= k2)
    real orient[kMaxOrient][3];
    real att[kMaxPots], dis[kMaxPots], inv_dis[kMaxPots], rmax[kMaxPots], costm[kMaxPots], kfac[kMaxPots];
    real mincos[kMaxTypes][kMaxTypes];  // smallest cos(thetam) of a type pair (early cone reject)
    real mincos_any[kMaxTypes];         // smallest cos(thetam) of a type with any type
};

// ------------------------------------------------------------------ vector moves of 12-real rows
template <class real> struct Row;
template <> struct Row<float> {
    float v[12];
    __device__ __forceinline__ void load(const float *p) {
        const float4 *q = reinterpret_cast<const float4 *>(p);
        float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        v[8] = c.x; v[9] = c.y; v[10] = c.z; v[11] = c.w;
    }
    __device__ __forceinline__ void store(float *p) const {
        float4 *q = reinterpret_cast<float4 *>(p);
        q[0] = make_float4(v[0], v[1], v[2], v[3]);
        q[1] = make_float4(v[4], v[5], v[6], v[7]);
        q[2] = make_float4(v[8], v[9], v[10], v[11]);
    }
};
template <> struct Row<double> {
    double v[12];
    __device__ __forceinline__ void load(const double *p) {
        const double2 *q = reinterpret_cast<const double2 *>(p);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            double2 a = __ldg(q + k);
            v[2 * k] = a.x; v[2 * k + 1] = a.y;
        }
    }
    __device__ __forceinline__ void store(double *p) const {
        double2 *q = reinterpret_cast<double2 *>(p);
#pragma unroll
        for (int k = 0; k < 6; k++) q[k] = make_double2(v[2 * k], v[2 * k + 1]);
    }
};

// four consecutive reals (one 16-byte vector in FP32, two in FP64)
__device__ __forceinline__ void load4(const float *p, float v[4]) {
    float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void load4(const double *p, double v[4]) {
    double2 a = __ldg(reinterpret_cast<const double2 *>(p)), b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void store4(float *p, float a, float b, float c, float d) {
    *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void store4(double *p, double a, double b, double c, double d) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(a, b);
    reinterpret_cast<double2 *>(p)[1] = make_double2(c, d);
}

// position of a slot (pos array: x, y, z, Q8)
__device__ __forceinline__ void load_pos(const float *p, float &x, float &y, float &z) {
    float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    x = a.x; y = a.y; z = a.z;
}
__device__ __forceinline__ void load_pos(const double *p, double &x, double &y, double &z) {
    double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    x = a.x; y = a.y; z = __ldg(p + 2);
}

// position + orientation of one slot in logical order v = (x, y, z, Q0..Q8)
template <class real>
struct Payload {
    real v[12];
    __device__ __forceinline__ void load(const real *pos, const real *rota, const real *rotb, size_t s) {
        real a[4], b[4], c[4];
        load4(pos + 4 * s, a);
        load4(rota + 4 * s, b);
        load4(rotb + 4 * s, c);
        v[0] = a[0]; v[1] = a[1]; v[2] = a[2]; v[11] = a[3];
        v[3] = b[0]; v[4] = b[1]; v[5] = b[2]; v[6] = b[3];
        v[7] = c[0]; v[8] = c[1]; v[9] = c[2]; v[10] = c[3];
    }
    __device__ __forceinline__ void store(real *pos, real *rota, real *rotb, size_t d) const {
        store4(pos + 4 * d, v[0], v[1], v[2], v[11]);
        store4(rota + 4 * d, v[3], v[4], v[5], v[6]);
        store4(rotb + 4 * d, v[7], v[8], v[9], v[10]);
    }
};

// ------------------------------------------------------------------ correctly rounded, uncontracted ops
// The integrator uses explicit roundings so that the binning pass and the scatter pass compute the
// identical next position, and so that the FP64 path rounds like the reference's x + c1 * p.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

template <class real> __device__ __forceinline__ real rsqrt_(real a);
template <> __device__ __forceinline__ float rsqrt_(float a) { return rsqrtf(a); }
template <> __device__ __forceinline__ double rsqrt_(double a) { return 1.0 / sqrt(a); }

// fasterfloor (Basic/basic.h:58)
template <class real>
__device__ __forceinline__ int fasterfloor(real x) { return x > real(0) ? (int)x : (int)x - 1; }

// cube::assign_box (geometry.h:508-520) for one axis
template <class real>
__device__ __forceinline__ int axis_cell(real x, real scale, int nc) {
    int m = fasterfloor<real>(mul_rn(x, scale));
    m = m < 0 ? 0 : m;
    return m > nc - 1 ? nc - 1 : m;
}

// cube::correct_position_and_momentum (geometry.h:403-446) for one coordinate.  The periodic wrap
// repeats like the reference's while-loops but is bounded (a non-finite coordinate is left as is
// and reported by the caller).
template <class real>
__device__ __forceinline__ void wrap_coord(real &x, real &p, real l, int periodic) {
    if (periodic) {
        if (x < real(0)) {
            for (int it = 0; it < 8 && x < real(0); it++) x = add_rn(x, l);
        } else if (x > l) {
            for (int it = 0; it < 8 && x > l; it++) x = sub_rn(x, l);
        }
    } else {
        if (x < real(0)) { x = -x; p = -p; }
        else if (x > l) { x = sub_rn(l, sub_rn(x, l)); p = -p; }
    }
}

// minimum image as cube::distance_vector (geometry.h:277-294): one correction when dx^2 > (l/2)^2
template <class real>
__device__ __forceinline__ real min_image(real dx, real l, real l2s, int periodic) {
    if (periodic && dx * dx > l2s) dx = dx >= real(0) ? dx - l : dx + l;
    return dx;
}

// The minimum-image separation x_a - x_b by the same rule.  FP64 forms it as the reference does, (x_a - x_b) -+ l.
// FP32 forms the corrected separation as ((x_a - l) - x_b) - l_lo or (x_a - (x_b - l)) + l_lo, l + l_lo being
// the double box length: the coordinate next to the far face lies in [l/2, l], so its difference with l is exact
// (Sterbenz), and the separation carries one rounding of its own size and the box length to double precision --
// (x_a - x_b) -+ (float)l would carry a rounding of the box length's size and the float box's own error (each up
// to 4e-6 at l = 130: 3e-6 relative at r = 1.5, 4e-5 in a WCA force).
template <class real>
__device__ __forceinline__ real min_image_sep(real xa, real xb, real l, real l_lo, real l2s, int periodic) {
    real dx = xa - xb;
    if (periodic && dx * dx > l2s) {
        if constexpr (sizeof(real) == 4) dx = dx >= real(0) ? ((xa - l) - xb) - l_lo : (xa - (xb - l)) + l_lo;
        else dx = dx >= real(0) ? dx - l : dx + l;
    }
    return dx;
}

// ------------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Six unit-variance uniform values for (particle, replica, draw):
// xi = 3.464101615 u - 1.732050808, u = (w >> 8) 2^-24  (matrix2.cpp:1807-1821 shape, U[0,1) here).
template <class real>
__device__ __forceinline__ void philox_noise6(uint32_t local, uint32_t replica, uint64_t draw,
                                              uint32_t seed_lo, uint32_t seed_hi, real xi[6]) {
    uint2 key = make_uint2(seed_lo, seed_hi);
    uint4 a = philox4x32_10(make_uint4(local, (uint32_t)draw, (uint32_t)(draw >> 32), 2u * replica), key);
    uint4 b = philox4x32_10(make_uint4(local, (uint32_t)draw, (uint32_t)(draw >> 32), 2u * replica + 1u), key);
    uint32_t w[6] = {a.x, a.y, a.z, a.w, b.x, b.y};
#pragma unroll
    for (int k = 0; k < 6; k++) {
        real u = real(w[k] >> 8) * real(1.0 / 16777216.0);
        xi[k] = real(3.464101615) * u - real(1.732050808);
    }
}

// ------------------------------------------------------------------ pair accumulators
// FP32: per-particle sums are kept in 64-bit fixed point (2^-32 resolution).  Integer addition is
// associative, so a particle's force does not depend on the order in which its neighbours are
// visited -- and that order (the within-cell order of the counting sort) is not deterministic.
// FP64: plain double sums.
template <class real> struct Acc3;
// 64-bit fixed point with 32 fraction bits, converted with 32-bit instructions only (64-bit integer <->
// float conversions run on GB300's narrow FP64 pipe).  to_fixed(v) equals round-to-nearest-even of
// v * 2^32 for |v| < 2^31: the floor part is exact and v - floor(v) is exact, so one rounding of the
// fraction * 2^32 (< 2^32) is the rounding of the whole.  from_fixed rounds the fraction to 24 bits first,
// so it can differ from a correctly rounded conversion by one unit in the last place; it is a fixed
// function of the sum, which is what order independence needs.
__device__ __forceinline__ long long to_fixed(float v) {
    const float a = fabsf(v);
    const float h = floorf(a);                                      // exact
    const unsigned hi = __float2uint_rz(h);
    const unsigned lo = __float2uint_rn((a - h) * 4294967296.0f);   // a - h exact, < 1 - 2^-24: fits
    const long long m = (long long)(((unsigned long long)hi << 32) + (unsigned long long)lo);
    return v < 0.f ? -m : m;
}
__device__ __forceinline__ float from_fixed(long long a) {
    const int hi = (int)(a >> 32);
    const unsigned lo = (unsigned)(unsigned long long)a;
    return fmaf(__uint2float_rn(lo), 2.3283064365386963e-10f, __int2float_rn(hi));
}

template <> struct Acc3<float> {
    long long v[3];
    __device__ __forceinline__ void zero() { v[0] = v[1] = v[2] = 0; }
    __device__ __forceinline__ void add(float a, float b, float c) {
        v[0] += to_fixed(a);
        v[1] += to_fixed(b);
        v[2] += to_fixed(c);
    }
    __device__ __forceinline__ float get(int k) const { return from_fixed(v[k]); }
};
template <> struct Acc3<double> {
    double v[3];
    __device__ __forceinline__ void zero() { v[0] = v[1] = v[2] = 0; }
    __device__ __forceinline__ void add(double a, double b, double c) { v[0] += a; v[1] += b; v[2] += c; }
    __device__ __forceinline__ double get(int k) const { return v[k]; }
};

// ------------------------------------------------------------------ physics of one pair

// HSPotential::force (potential.h:106-118) divided by r: 4 eps (12 s^12/r^14 - 6 s^6/r^8), written in
// terms of r^2 so no power of a rounded square root enters; the caller applies the r < 1.12246 sigma cut.
template <class real>
__device__ __forceinline__ real hs_force_over_r(const Replica<real> &R, real r2) {
    real inv2 = real(1) / r2;
    real s6 = R.hs_s6 * inv2 * inv2 * inv2;  // (sigma/r)^6
    return R.hs_4eps * inv2 * (real(12) * s6 * s6 - real(6) * s6);
}

// ---- float-float arithmetic (Dekker; Knuth's two-sum; the product error from an FMA), for the FP32 WCA core.
// Every operation is an explicit round-to-nearest intrinsic, so no contraction changes the error terms.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ FF ff_fast_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const FF s = ff_two_sum(a.hi, b.hi);
    return ff_fast_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const FF p = ff_two_prod(a.hi, b.hi);
    return ff_fast_sum(p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo)));
}
__device__ __forceinline__ FF ff_mul(FF a, float b) {
    const FF p = ff_two_prod(a.hi, b);
    return ff_fast_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
// 1 / a: the rounded reciprocal of a.hi and one Newton correction with the residual 1 - a r0 kept exactly
__device__ __forceinline__ FF ff_rcp(FF a) {
    const float r0 = __frcp_rn(a.hi);
    const FF p = ff_two_prod(a.hi, r0);
    const float e = __fmaf_rn(-a.lo, r0, __fsub_rn(__fsub_rn(1.0f, p.hi), p.lo));   // 1 - p.hi is exact
    return ff_fast_sum(r0, __fmul_rn(r0, e));
}

// The WCA core force of one pair in FP32 as float-float components: force = hi + lo per axis, from the exact
// separation d (x_a - x_b).  |d|^2, 1/|d|^2, the powers and the force law run in float-float, so the pair force
// carries about 1e-12 relative error instead of single precision's ~1e-7: the net force of a particle whose pair
// forces of tens of eps/sigma cancel stays accurate (the sums are fixed point, 2^-32).  Same law as
// hs_force_over_r: 4 eps (12 s^12/r^14 - 6 s^6/r^8) times d.
__device__ __forceinline__ void hs_force_ff(const Replica<float> &R, const float d[3], float hi[3], float lo[3]) {
    const FF r2 = ff_add(ff_add(ff_two_prod(d[0], d[0]), ff_two_prod(d[1], d[1])), ff_two_prod(d[2], d[2]));
    const FF inv = ff_rcp(r2);
    const FF s6 = ff_mul(ff_mul(ff_mul(inv, inv), inv), R.hs_s6);                      // (sigma / r)^6
    const FF t = ff_add(ff_mul(ff_mul(s6, s6), 12.0f), ff_mul(s6, -6.0f));           // 12 s^12 - 6 s^6
    const FF g = ff_mul(ff_mul(inv, t), R.hs_4eps);                                  // force / r
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const FF v = ff_mul(g, d[k]);
        hi[k] = v.hi;
        lo[k] = v.lo;
    }
}

// shifted WCA energy used for the energy observable
template <class real>
__device__ __forceinline__ real wca_energy(const Replica<real> &R, real r2) {
    real s2 = R.hs_s6 / (r2 * r2 * r2);  // (sigma/r)^6
    return R.hs_4eps * (s2 * s2 - s2) + R.hs_eps;
}

// Patch (KernFrenkelOnePatch2::force_and_torque, potentialtheta.h:517-750) for one in-cone potential.
// u = (x_a - x_b)/r (a = lower reference index), n1/n2 = lab-frame patch vectors of a/b,
// ci = -n1.u, cj = n2.u.  Adds the force on a to f, the torques on a/b to ta/tb, the energy to e.
template <class real>
__device__ __forceinline__ void kf2_pair(real att, real dis, real inv_dis, real kfac, const real u[3], real r,
                                         const real n1[3], const real n2[3], real ci, real cj, real f[3], real ta[3],
                                         real tb[3], real &e) {
    if (ci > real(1)) ci = real(0.999999);
    if (cj > real(1)) cj = real(0.999999);
    real thi = acos(ci), thj = acos(cj);
    real sai, cai, saj, caj;
    sincos(kfac * thi, &sai, &cai);
    sincos(kfac * thj, &saj, &caj);
    real fang = cai * caj;
    real fac = r * inv_dis;
    real fac2 = fac * fac, fac4 = fac2 * fac2, fac8 = fac4 * fac4, fac10 = fac2 * fac8;
    real ex = exp(real(-0.5) * fac10);
    real pot = -att * ex;
    real potf = real(-5) * att * fac8 * (fac * inv_dis) * ex;
    // d1/d2 of the reference: zero when |c^2 - 1| < 1e-5, else -1/sqrt(1 - c^2)
    real d1 = fabs(ci * ci - real(1)) < real(1e-5) ? real(0) : -rsqrt_<real>((real(1) - ci) * (real(1) + ci));
    real d2 = fabs(cj * cj - real(1)) < real(1e-5) ? real(0) : -rsqrt_<real>((real(1) - cj) * (real(1) + cj));
    real gi = -kfac * pot * sai * d1 * caj;
    real gj = -kfac * pot * saj * d2 * cai;
    real fp = fang * potf, gir = gi / r, gjr = gj / r;
#pragma unroll
    for (int k = 0; k < 3; k++) f[k] += fp * u[k] + gir * (n1[k] + ci * u[k]) - gjr * (n2[k] - cj * u[k]);
    // torque on a: gi (n1 x u); torque on b: gj (u x n2)
    ta[0] += gi * (n1[1] * u[2] - n1[2] * u[1]);
    ta[1] += gi * (n1[2] * u[0] - n1[0] * u[2]);
    ta[2] += gi * (n1[0] * u[1] - n1[1] * u[0]);
    tb[0] += gj * (u[1] * n2[2] - u[2] * n2[1]);
    tb[1] += gj * (u[2] * n2[0] - u[0] * n2[2]);
    tb[2] += gj * (u[0] * n2[1] - u[1] * n2[0]);
    e += pot * fang;
}

template <class real>
__device__ __forceinline__ int type_of(const Model<real> &M, int local) {
    int t = 0;
#pragma unroll
    for (int k = 0; k < kMaxTypes - 1; k++)
        if (k < M.n_types - 1 && local >= M.ncum[k]) t = k + 1;
    return t;
}

// patch_pair for types with at most four patches each: the cosines stay in registers and the in-cone
// potentials (i, j) are collected in a 16-bit mask (bit 4 i + j) and evaluated in ascending bit order,
// which is patch_pair's loop order, so sums and counts are the same bit for bit.
template <class real>
__device__ __forceinline__ void patch_pair4(const Model<real> &M, int ta_, int tb_, const real *Qa, const real *Qb,
                                            const real u[3], real r, real bond_r, real f[3], real tqa[3],
                                            real tqb[3], real &e, int &bonds) {
    const int na = M.np[ta_], nb = M.np[tb_];
    real wa[3], wb[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        wa[k] = Qa[3 * k] * u[0] + Qa[3 * k + 1] * u[1] + Qa[3 * k + 2] * u[2];
        wb[k] = Qb[3 * k] * u[0] + Qb[3 * k + 1] * u[1] + Qb[3 * k + 2] * u[2];
    }
    const real mc = M.mincos[ta_][tb_];
    const int oa = M.ooff[ta_], ob = M.ooff[tb_];
    real ca[4], cb[4];
    unsigned ma = 0u, mb = 0u;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        ca[i] = real(0);
        cb[i] = real(0);
        if (i < na) {
            const real *v = M.orient[oa + i];
            ca[i] = -(v[0] * wa[0] + v[1] * wa[1] + v[2] * wa[2]);
            if (ca[i] > mc) ma |= 1u << i;
        }
        if (i < nb) {
            const real *v = M.orient[ob + i];
            cb[i] = v[0] * wb[0] + v[1] * wb[1] + v[2] * wb[2];
            if (cb[i] > mc) mb |= 1u << i;
        }
    }
    if (!ma || !mb) return;
    const int ps = M.pstart[ta_][tb_];
    unsigned m = 0u;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (!((ma >> i) & 1u)) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (j >= nb) continue;
            const int q = ps + i * nb + j;
            const real cm = M.costm[q];
            if (!(ca[i] > cm && cb[j] > cm)) continue;
            if (r < bond_r) bonds++;
            if (!(r > M.rmax[q])) m |= 1u << (4 * i + j);
        }
    }
    while (m) {
        const int bit = __ffs(m) - 1;
        m &= m - 1u;
        const int i = bit >> 2, j = bit & 3;
        const real ci = i == 0 ? ca[0] : (i == 1 ? ca[1] : (i == 2 ? ca[2] : ca[3]));
        const real cj = j == 0 ? cb[0] : (j == 1 ? cb[1] : (j == 2 ? cb[2] : cb[3]));
        const int q = ps + i * nb + j;
        const real *b1 = M.orient[oa + i], *b2 = M.orient[ob + j];
        real n1[3], n2[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            n1[k] = b1[0] * Qa[k] + b1[1] * Qa[3 + k] + b1[2] * Qa[6 + k];
            n2[k] = b2[0] * Qb[k] + b2[1] * Qb[3 + k] + b2[2] * Qb[6 + k];
        }
        kf2_pair<real>(M.att[q], M.dis[q], M.inv_dis[q], M.kfac[q], u, r, n1, n2, ci, cj, f, tqa, tqb, e);
    }
}

// All potentials of the canonical pair (a, b): Qa/Qb lab->body rows, u = (x_a - x_b)/r.
// Returns the number of in-cone potentials; adds force on a, torques on a/b, energy, bonds.
template <class real>
__device__ __forceinline__ void patch_pair(const Model<real> &M, int ta_, int tb_, const real *Qa, const real *Qb,
                                           const real u[3], real r, real bond_r, real f[3], real tqa[3],
                                           real tqb[3], real &e, int &bonds) {
    const int na = M.np[ta_], nb = M.np[tb_];
    if (na <= 4 && nb <= 4) {
        patch_pair4<real>(M, ta_, tb_, Qa, Qb, u, r, bond_r, f, tqa, tqb, e, bonds);
        return;
    }
    // body-frame images of u: c_i(patch) = -n_body . (Qa u), c_j = n_body . (Qb u)
    real wa[3], wb[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        wa[k] = Qa[3 * k] * u[0] + Qa[3 * k + 1] * u[1] + Qa[3 * k + 2] * u[2];
        wb[k] = Qb[3 * k] * u[0] + Qb[3 * k + 1] * u[1] + Qb[3 * k + 2] * u[2];
    }
    const real mc = M.mincos[ta_][tb_];
    real ca[kMaxOrient], cb[kMaxOrient];
    bool anya = false, anyb = false;
    const int oa = M.ooff[ta_], ob = M.ooff[tb_];
    for (int i = 0; i < na; i++) {
        const real *nbv = M.orient[oa + i];
        ca[i] = -(nbv[0] * wa[0] + nbv[1] * wa[1] + nbv[2] * wa[2]);
        anya |= ca[i] > mc;
    }
    for (int j = 0; j < nb; j++) {
        const real *nbv = M.orient[ob + j];
        cb[j] = nbv[0] * wb[0] + nbv[1] * wb[1] + nbv[2] * wb[2];
        anyb |= cb[j] > mc;
    }
    if (!(anya && anyb)) return;
    const int ps = M.pstart[ta_][tb_];
    for (int i = 0; i < na; i++) {
        if (!(ca[i] > mc)) continue;
        for (int j = 0; j < nb; j++) {
            const int q = ps + i * nb + j;
            const real cm = M.costm[q];
            if (!(ca[i] > cm && cb[j] > cm)) continue;
            if (r < bond_r) bonds++;
            if (r > M.rmax[q]) continue;
            // lab-frame patch vectors n = Q^T n_body
            const real *b1 = M.orient[oa + i], *b2 = M.orient[ob + j];
            real n1[3], n2[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                n1[k] = b1[0] * Qa[k] + b1[1] * Qa[3 + k] + b1[2] * Qa[6 + k];
                n2[k] = b2[0] * Qb[k] + b2[1] * Qb[3 + k] + b2[2] * Qb[6 + k];
            }
            kf2_pair<real>(M.att[q], M.dis[q], M.inv_dis[q], M.kfac[q], u, r, n1, n2, ca[i], cb[j], f, tqa, tqb, e);
        }
    }
}

}  // namespace mtg
