// LangevinNVTRGPU.hpp -- header-only C++ adapter that gives the reference's LangevinNVTR interface
// (MDBase/Rotational/LangevinR.h:59-270) to the GB300 C ABI (mtcode_gb300.h).
//
// A maintainer of osmanovicdino/mtcode replaces the step loop of Condensate::run
// (Condensate/Condensate.cpp:335-378) by
//
//     LangevinNVTRGPU<matrix<double>> gpu(geo_l, /*periodic*/ true, N, model);
//     gpu.setdt(dt); gpu.setkT(kT); gpu.setgamma(g); gpu.setgammar(gr);
//     gpu.initialize(pos, mom, orient, angmom);        // LangevinNVTR::initialize(x, p, Q, L)
//     gpu.init_forces();                               // the F, T, RT before the loop (:312-334)
//     for (i ...) { gpu.measured_temperature(meas); gpu.step(1); if (i % every == 0) gpu.getdat(pos); ... }
//
// The matrix type only needs operator()(i, j), getNsafe() and getncols(), so the same header works
// with the reference's matrix<T> (DataStructures/matrix2.h) and with any other row-major container.
// Every failure throws std::runtime_error with the library's message (the reference's error()
// would block on stdin, Basic/basic.h:61-71).
#ifndef MTCODE_GB300_LANGEVINNVTRGPU_HPP
#define MTCODE_GB300_LANGEVINNVTRGPU_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "mtcode_gb300.h"

// Names here avoid the reference's object-like macros (Basic/basic.h defines check, min, mathematica,
// convert, ...), so this header can follow the reference's own includes.
namespace mtg_adapter {

inline void require_ok(mtg_system *h, mtg_status st, const char *what) {
    if (st != MTG_OK)
        throw std::runtime_error(std::string(what) + ": " + mtg_status_string(st) + " -- " + mtg_last_error(h));
}

template <class M>
void to_rows(M &m, int n, int c, std::vector<double> &out) {
    out.resize((size_t)n * c);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < c; k++) out[(size_t)c * i + k] = m(i, k);
}

template <class M>
void from_rows(const std::vector<double> &in, int n, int c, M &m) {
    for (int i = 0; i < n; i++)
        for (int k = 0; k < c; k++) m(i, k) = in[(size_t)c * i + k];
}

// Binding models of the reference (MDBase/Bindings) in the C ABI's table form.  Templates, so this header
// needs none of the reference's headers: any object with the reference's public members converts.
// BindingModelSingle: on_rate, off_rate.
template <class BMS>
mtg_binding_model binding_single_from(const BMS &bm) {
    mtg_binding_model m;
    mtg_binding_single(&m, bm.on_rate, bm.off_rate);
    return m;
}

template <class Vec>
void copy_rates(const Vec &v, double *out, int count) {
    for (int k = 0; k < count; k++) out[k] = k < v.getsize() ? v.gpcons(k) : 0.0;
}

// BindingModelBinary: div and its rate vectors; its 122 / 222 triplets take the rate to none-bound from
// tripr111 (BindingModelBinary.cpp triplet)
template <class BMB>
mtg_binding_model binding_binary_from(const BMB &bm) {
    mtg_binding_model m{};
    m.species_rule = 1;
    m.div1 = bm.div;
    m.np = 1;
    copy_rates(bm.doubr11, m.drate[0], 4);
    copy_rates(bm.doubr12, m.drate[1], 4);
    copy_rates(bm.doubr22, m.drate[3], 4);
    copy_rates(bm.tripr111, m.trate[0], 16);
    copy_rates(bm.tripr112, m.trate[1], 16);
    copy_rates(bm.tripr122, m.trate[3], 16);
    copy_rates(bm.tripr222, m.trate[6], 16);
    for (int r : {3, 6})
        for (int st = 0; st < 4; st++) m.trate[r][4 * st + 3] = m.trate[0][4 * st + 3];
    return m;
}

template <class BMT>
void ternary_rates(const BMT &bm, mtg_binding_model &m) {
    copy_rates(bm.doubr11, m.drate[0], 4);
    copy_rates(bm.doubr12, m.drate[1], 4);
    copy_rates(bm.doubr13, m.drate[2], 4);
    copy_rates(bm.doubr22, m.drate[3], 4);
    copy_rates(bm.doubr23, m.drate[4], 4);
    copy_rates(bm.doubr33, m.drate[5], 4);
    copy_rates(bm.tripr111, m.trate[0], 16);
    copy_rates(bm.tripr112, m.trate[1], 16);
    copy_rates(bm.tripr113, m.trate[2], 16);
    copy_rates(bm.tripr122, m.trate[3], 16);
    copy_rates(bm.tripr123, m.trate[4], 16);
    copy_rates(bm.tripr133, m.trate[5], 16);
    copy_rates(bm.tripr222, m.trate[6], 16);
    copy_rates(bm.tripr223, m.trate[7], 16);
    copy_rates(bm.tripr233, m.trate[8], 16);
    copy_rates(bm.tripr333, m.trate[9], 16);
}

// BindingModelTernary<SortingFunctionUniform> / <SortingFunctionNonUniform> (BindingModelTernary.h:6-30)
template <class BMT>
mtg_binding_model binding_ternary_uniform_from(const BMT &bm) {
    mtg_binding_model m{};
    m.species_rule = 2;
    m.div1 = bm.func.div1;
    m.div2 = bm.func.div2;
    m.np = 1;
    ternary_rates(bm, m);
    return m;
}

template <class BMT>
mtg_binding_model binding_ternary_nonuniform_from(const BMT &bm) {
    mtg_binding_model m{};
    m.species_rule = 3;
    m.div1 = bm.func.div1;
    m.div2 = bm.func.div2;
    m.np = bm.func.np;
    ternary_rates(bm, m);
    return m;
}

// Patch models of the reference (MDBase/Potentials/ComboPatch) in the C ABI's GeneralPatch form, read from
// the objects' public members, so a driver passes its own ComboPatch instead of filling arrays by hand.
// TetrahedralPatch(str, dis, ang) (TetrahedralPatch.cpp:4-44)
template <class TP>
mtg_patch_model model_from_tetrahedral(const TP &tp) {
    mtg_patch_model m;
    mtg_model_tetrahedral(&m, tp.str, tp.dis, tp.ang);
    return m;
}
// BivalentPatch(str, dis, ang) (BivalentPatch.cpp:4-34)
template <class BP>
mtg_patch_model model_from_bivalent(const BP &bp) {
    mtg_patch_model m;
    mtg_model_bivalent(&m, bp.str, bp.dis, bp.ang);
    return m;
}
// GeneralPatch (GeneralPatch.cpp:7-121): no_types, no_patches_per_type[], num_per_type[] (cumulative), the
// orient rows (patch unit vectors, types contiguous) and the params rows (att, dis, thetam) per potential, in
// the order GeneralPatch enumerates potential_bundle -- the C ABI's own order, so the rows copy unchanged
template <class GP>
mtg_patch_model model_from_general(GP &gp) {
    mtg_patch_model m{};
    if (gp.no_types < 1 || gp.no_types > MTG_MAX_TYPES)
        throw std::runtime_error("model_from_general: " + std::to_string(gp.no_types) + " particle types (1 to " +
                                 std::to_string(MTG_MAX_TYPES) + " supported)");
    m.n_types = gp.no_types;
    int norient = 0;
    for (int k = 0; k < gp.no_types; k++) {
        m.patches_per_type[k] = gp.no_patches_per_type[k];
        m.count_per_type[k] = gp.num_per_type[k];
        norient += gp.no_patches_per_type[k];
    }
    const int npots = gp.params.getnrows();
    if (norient > MTG_MAX_ORIENT || npots > MTG_MAX_POTS)
        throw std::runtime_error("model_from_general: more patch vectors or potentials than the C ABI holds");
    for (int i = 0; i < norient; i++)
        for (int c = 0; c < 3; c++) m.orient[i][c] = gp.orient(i, c);
    for (int q = 0; q < npots; q++)
        for (int c = 0; c < 3; c++) m.params[q][c] = gp.params(q, c);
    return m;
}

}  // namespace mtg_adapter

template <class Matrix>
class LangevinNVTRGPU {
  public:
    // cube(l, pb, 3) + the ComboPatch in GeneralPatch form (mtg_model_tetrahedral / _bivalent or a
    // filled mtg_patch_model); precision MTG_FP32 (batched path) or MTG_FP64 (plain path)
    LangevinNVTRGPU(double box, bool periodic, int n, const mtg_patch_model &model, int precision = MTG_FP32,
                    int device = 0)
        : precision_(precision), device_(device) {
        mtg_replica_defaults(&desc_);
        desc_.n = n;
        desc_.box = box;
        desc_.periodic = periodic ? 1 : 0;
        desc_.model = model;
        if (desc_.model.n_types == 1 && desc_.model.count_per_type[0] == 0) desc_.model.count_per_type[0] = n;
    }
    ~LangevinNVTRGPU() { mtg_destroy(h_); }
    LangevinNVTRGPU(const LangevinNVTRGPU &) = delete;
    LangevinNVTRGPU &operator=(const LangevinNVTRGPU &) = delete;

    // LangevinNVTR setters (LangevinR.h:109-134, LangevinR.cpp:130-144); effective at initialize()
    void setdt(double v) { desc_.dt = v; }
    void setkT(double v) { desc_.kT = v; }
    void setgamma(double v) { desc_.gamma = v; }
    void setgammar(double v) { desc_.gammar = v; }
    void setm(double v) { desc_.mass = v; }
    void setinertia(double v) { desc_.inertia = v; }
    void setmaxdistance(double v) { desc_.max_dist2 = v; }    // LangevinR.h:136-138
    void sethardcore(double eps, double sigma) { desc_.hs_eps = eps; desc_.hs_sigma = sigma; }  // HSPotential(eps, sigma)
    void setseed(uint64_t s) { desc_.seed = s; }

    // LangevinNVTR::initialize(positions, momenta, orientations, angular_momenta) (LangevinR.cpp:309-325)
    void initialize(Matrix &x, Matrix &p, Matrix &Q, Matrix &L) {
        if (!h_) create();
        const int n = desc_.n;
        mtg_adapter::to_rows(x, n, 3, bx_);
        mtg_adapter::to_rows(p, n, 3, bp_);
        mtg_adapter::to_rows(Q, n, 9, bq_);
        mtg_adapter::to_rows(L, n, 3, bl_);
        mtg_adapter::require_ok(h_, mtg_set_state(h_, bx_.data(), bp_.data(), bl_.data(), bq_.data(), nullptr, nullptr),
                           "initialize");
    }

    // F, T, RT and create_forces_and_torques_sphere before the loop (Condensate.cpp:312-334)
    void init_forces() { mtg_adapter::require_ok(h_, mtg_init_forces(h_), "init_forces"); }

    // nsteps of the loop body (Condensate.cpp:335-378); asynchronous
    void step(int nsteps = 1) { mtg_adapter::require_ok(h_, mtg_step(h_, nsteps), "step"); }

    // MD::calculateforces(pairs, HSPotential) + calculate_forces_and_torques3D(pairs, ComboPatch, F, T)
    void calculate_forces_and_torques3D(Matrix &F, Matrix &T) {
        const int n = desc_.n;
        std::vector<double> f((size_t)n * 3), t((size_t)n * 3);
        mtg_adapter::require_ok(h_, mtg_forces(h_, f.data(), t.data(), nullptr), "calculate_forces_and_torques3D");
        mtg_adapter::from_rows(f, n, 3, F);
        mtg_adapter::from_rows(t, n, 3, T);
    }

    // ---- the loop body one method at a time, with the reference's signatures (Condensate.cpp:335-378):
    //   advancemom_halfstep(F, T); advance_pos(); rotate(); F = calculateforces(pairs, HS); T = 0;
    //   calculate_forces_and_torques3D(pairs, patches, F, T); create_forces_and_torques_sphere(F, T, R);
    //   advancemom_halfstep(F, T);
    // Pair lists and potentials are accepted for the signatures' sake: the GPU's own cell list finds every pair
    // within the force range (the pair set of any caller list that covers that range), and the potentials are
    // the handle's (sethardcore, and the patch model given at construction).

    // MD::calculatepairs_parallel(boxlist, rc) (MD.h:83): a new P x 2 matrix of the pairs (i < j) closer than rc,
    // which the caller deletes (Condensate.cpp:348-349)
    template <class IntMatrix>
    IntMatrix *calculatepairs_parallel(IntMatrix &boxlist, double rc) {
        (void)boxlist;
        int64_t np = 0;
        mtg_status st = mtg_pairs(h_, 0, rc, nullptr, 0, &np);
        if (st != MTG_OK && st != MTG_ERR_CAPACITY) mtg_adapter::require_ok(h_, st, "calculatepairs_parallel");
        std::vector<int32_t> buf((size_t)(np > 0 ? np : 1) * 2);
        mtg_adapter::require_ok(h_, mtg_pairs(h_, 0, rc, buf.data(), np, &np), "calculatepairs_parallel");
        IntMatrix *out = new IntMatrix((int)np, 2);
        for (int64_t i = 0; i < np; i++) {
            (*out)((int)i, 0) = buf[2 * i];
            (*out)((int)i, 1) = buf[2 * i + 1];
        }
        return out;
    }

    // MD::calculateforces(pairs, HSPotential) (MD.h:110): the WCA core forces (plus any setbonds bonds)
    template <class IntMatrix, class Potential>
    Matrix calculateforces(IntMatrix &pairs, Potential &pot) {
        (void)pairs;
        (void)pot;
        const int n = desc_.n;
        std::vector<double> f((size_t)n * 3);
        mtg_adapter::require_ok(h_, mtg_calculateforces(h_, f.data()), "calculateforces");
        Matrix F(n, 3);
        mtg_adapter::from_rows(f, n, 3, F);
        return F;
    }

    // LangevinNVTR::calculate_forces_and_torques3D(pairs, ComboPatch, F, T) (LangevinR.h:247): ADDS the patch
    // forces to F and the lab-frame torques to T
    template <class IntMatrix, class Combo>
    void calculate_forces_and_torques3D(IntMatrix &pairs, Combo &patches, Matrix &F, Matrix &T) {
        (void)pairs;
        (void)patches;
        const int n = desc_.n;
        std::vector<double> f, t;
        mtg_adapter::to_rows(F, n, 3, f);
        mtg_adapter::to_rows(T, n, 3, t);
        mtg_adapter::require_ok(h_, mtg_calculate_forces_and_torques3D(h_, f.data(), t.data()),
                                "calculate_forces_and_torques3D");
        mtg_adapter::from_rows(f, n, 3, F);
        mtg_adapter::from_rows(t, n, 3, T);
    }

    // LangevinNVTR::create_forces_and_torques_sphere(F, T, R) (LangevinR.h:244): F (lab), T (lab) in; F~ (lab)
    // and T~ (body) out, with the caller's n x 6 noise R
    template <class RMatrix>
    void create_forces_and_torques_sphere(Matrix &F, Matrix &T, RMatrix &R) {
        const int n = desc_.n;
        std::vector<double> f, t, r;
        mtg_adapter::to_rows(F, n, 3, f);
        mtg_adapter::to_rows(T, n, 3, t);
        mtg_adapter::to_rows(R, n, 6, r);
        mtg_adapter::require_ok(h_, mtg_create_forces_and_torques_sphere(h_, f.data(), t.data(), r.data()),
                                "create_forces_and_torques_sphere");
        mtg_adapter::from_rows(f, n, 3, F);
        mtg_adapter::from_rows(t, n, 3, T);
    }
    // the same with the handle's counter-based Philox noise in place of R
    void create_forces_and_torques_sphere(Matrix &F, Matrix &T) {
        const int n = desc_.n;
        std::vector<double> f, t;
        mtg_adapter::to_rows(F, n, 3, f);
        mtg_adapter::to_rows(T, n, 3, t);
        mtg_adapter::require_ok(h_, mtg_create_forces_and_torques_sphere(h_, f.data(), t.data(), nullptr),
                                "create_forces_and_torques_sphere");
        mtg_adapter::from_rows(f, n, 3, F);
        mtg_adapter::from_rows(t, n, 3, T);
    }

    // LangevinNVTR::advancemom_halfstep(F, T) (LangevinR.h:259): F lab, T body
    void advancemom_halfstep(Matrix &F, Matrix &T) {
        const int n = desc_.n;
        std::vector<double> f, t;
        mtg_adapter::to_rows(F, n, 3, f);
        mtg_adapter::to_rows(T, n, 3, t);
        mtg_adapter::require_ok(h_, mtg_advancemom_halfstep(h_, f.data(), t.data()), "advancemom_halfstep");
    }

    // LangevinNVT::advance_pos() (Langevin.h:57) and LangevinNVTR::rotate() (LangevinR.h:233)
    void advance_pos() { mtg_adapter::require_ok(h_, mtg_advance_pos(h_), "advance_pos"); }
    void rotate() { mtg_adapter::require_ok(h_, mtg_rotate(h_), "rotate"); }

    // the bonded term of the polymer drivers: F += MD::calculateforces(bonds, HarmonicPotential(k, r0))
    // (mainActivePolymer.cpp:390-402) on every force pass; bonds is any B x 2 int matrix (e.g. matrix<int>)
    template <class IntMatrix>
    void setbonds(IntMatrix &bonds, double k, double r0) {
        if (!h_) create();
        const int nb = bonds.getNsafe();
        std::vector<int32_t> b((size_t)nb * 2);
        for (int i = 0; i < nb; i++) {
            b[2 * (size_t)i] = bonds(i, 0);
            b[2 * (size_t)i + 1] = bonds(i, 1);
        }
        mtg_adapter::require_ok(h_, mtg_set_bonds(h_, nb ? b.data() : nullptr, nb, k, r0), "setbonds");
    }

    // Condensate::run_singlebond (Condensate.cpp:422-618): from now on each force pass keeps one bond per
    // patch, decided by the binding model (mtg_adapter::binding_*_from converts the reference's models), and
    // only bound patch pairs exert the Kern-Frenkel force.  The candidate list is rebuilt every patch_every
    // steps from pairs closer than list_cut (run_singlebond: 10 steps, 2.5 sigma).
    void setsinglebond(const mtg_binding_model &bm, int patch_every = 10, double list_cut = 2.5) {
        if (!h_) create();
        mtg_single_bond sb;
        mtg_single_bond_defaults(&sb);
        sb.model = bm;
        sb.patch_every = patch_every;
        sb.list_cut = list_cut;
        mtg_adapter::require_ok(h_, mtg_set_single_bond(h_, &sb), "setsinglebond");
    }

    // BinaryBindStore (Bindings/BinaryBindStore.h): isbound / boundto of every patch, in and out; any
    // vectors with operator[] and getsize() (e.g. vector1<bool>, vector1<int>)
    template <class BoolVec, class IntVec>
    void setbindings(BoolVec &isbound, IntVec &boundto) {
        const int64_t np = mtg_num_patches(h_);
        std::vector<int32_t> bt((size_t)np);
        std::vector<uint8_t> ib((size_t)np);
        for (int64_t i = 0; i < np; i++) {
            bt[(size_t)i] = boundto[(int)i];
            ib[(size_t)i] = isbound[(int)i] ? 1 : 0;
        }
        mtg_adapter::require_ok(h_, mtg_set_bind_state(h_, bt.data(), ib.data()), "setbindings");
    }
    template <class BoolVec, class IntVec>
    void getbindings(BoolVec &isbound, IntVec &boundto) {
        const int64_t np = mtg_num_patches(h_);
        std::vector<int32_t> bt((size_t)np);
        std::vector<uint8_t> ib((size_t)np);
        mtg_adapter::require_ok(h_, mtg_get_bind_state(h_, bt.data(), ib.data()), "getbindings");
        for (int64_t i = 0; i < np; i++) {
            boundto[(int)i] = bt[(size_t)i];
            isbound[(int)i] = ib[(size_t)i] != 0;
        }
    }

    // LangevinNVTR::setup_random_binding(pairs, divs, iny, bo, bm) (LangevinRforceUtil.cpp:749-1010), as
    // run_singlebond calls it before its loop (Condensate.cpp:478-484): the candidate list of the current state
    // (the device's own, from every pair within the list cut: the caller's pairs and divs are not read), the
    // edges that can bind, taken in a random order, each binding two unbound patches; bo (a BinaryBindStore or
    // anything with isbound / boundto members) receives the bond state.  The order is seeded (mtg_setup_random_binding)
    // where the reference draws it from std::random_device.
    template <class Pairs, class Divs, class Patches, class BindStore, class BindingModel>
    void setup_random_binding(Pairs &, Divs &, Patches &, BindStore &bo, BindingModel &, uint64_t seed = 0) {
        mtg_adapter::require_ok(h_, mtg_setup_random_binding(h_, seed), "setup_random_binding");
        getbindings(bo.isbound, bo.boundto);
    }

    // LangevinNVTR::calculate_forces_and_torques3D_onlyone_nonlets (LangevinRforce.cpp:2874-4030) at the
    // current state, with the candidate list rebuilt first: decides the bonds, then F = calculateforces(HS)
    // + bound-pair forces and T = bound-pair torques, as run_singlebond's first call (Condensate.cpp:455-460)
    void calculate_forces_and_torques3D_onlyone_nonlets(Matrix &F, Matrix &T) {
        const int n = desc_.n;
        std::vector<double> f((size_t)n * 3), t((size_t)n * 3);
        mtg_adapter::require_ok(h_, mtg_bind_update(h_, f.data(), t.data()), "calculate_forces_and_torques3D_onlyone_nonlets");
        mtg_adapter::from_rows(f, n, 3, F);
        mtg_adapter::from_rows(t, n, 3, T);
    }

    // MD::calculatepairs_parallel(boxes, rc) -> pairs (i < j), P x 2, into any resizable int matrix
    template <class IntMatrix>
    void calculatepairs_parallel(double rc, IntMatrix &pairs_out) {
        int64_t np = 0;
        mtg_status st = mtg_pairs(h_, 0, rc, nullptr, 0, &np);
        if (st != MTG_OK && st != MTG_ERR_CAPACITY) mtg_adapter::require_ok(h_, st, "calculatepairs_parallel");
        std::vector<int32_t> buf((size_t)(np > 0 ? np : 1) * 2);
        mtg_adapter::require_ok(h_, mtg_pairs(h_, 0, rc, buf.data(), np, &np), "calculatepairs_parallel");
        pairs_out.resize(np, 2);
        for (int64_t i = 0; i < np; i++) {
            pairs_out(i, 0) = buf[2 * i];
            pairs_out(i, 1) = buf[2 * i + 1];
        }
    }

    // LangevinNVTR::measured_temperature(vector1<double>&) (LangevinR.cpp:170-193); any vec with operator[]
    template <class Vec>
    void measured_temperature(Vec &ret) {
        double t[6];
        mtg_adapter::require_ok(h_, mtg_temperature(h_, t), "measured_temperature");
        for (int k = 0; k < 6; k++) ret[k] = t[k];
    }

    // nsteps of the loop body, each followed by measured_temperature of that step, with no host round trip
    // between steps: out holds nsteps x n_replicas x 6 (step-major) when the call returns
    void step_measured(int nsteps, double *out) {
        mtg_adapter::require_ok(h_, mtg_step_temperatures(h_, nsteps, out), "step_measured");
    }

    // getdat / getmom / getorientation / getangmom (LangevinR.h:190-196), into caller matrices
    void getdat(Matrix &x) { get(0, x); }
    void getmom(Matrix &p) { get(1, p); }
    void getorientation(Matrix &Q) { get(3, Q); }
    void getangmom(Matrix &L) { get(2, L); }

    mtg_system *handle() { return h_; }

  private:
    void create() {
        mtg_config cfg{};
        cfg.precision = precision_;
        cfg.n_replicas = 1;
        cfg.replicas = &desc_;
        cfg.device = device_;
        cfg.track_displacement = 1;
        cfg.force_kernel = 0;
        mtg_status st = mtg_create(&cfg, &h_);
        if (st != MTG_OK) throw std::runtime_error(std::string("mtg_create: ") + mtg_last_error(nullptr));
    }
    void get(int which, Matrix &m) {
        const int n = desc_.n, w = which == 3 ? 9 : 3;
        std::vector<double> b((size_t)n * w);
        double *ptr[4] = {nullptr, nullptr, nullptr, nullptr};
        ptr[which] = b.data();
        mtg_adapter::require_ok(h_, mtg_get_state(h_, ptr[0], ptr[1], ptr[2], ptr[3], nullptr, nullptr), "get_state");
        mtg_adapter::from_rows(b, n, w, m);
    }

    mtg_replica_desc desc_;
    int precision_, device_;
    mtg_system *h_ = nullptr;
    std::vector<double> bx_, bp_, bq_, bl_;
};

#endif  // MTCODE_GB300_LANGEVINNVTRGPU_HPP
