// LangevinNVTRGPU_reference.hpp -- the drop-in as a subclass of the reference's own integrator:
// mtg_dropin::LangevinNVTRGPU derives from LangevinNVTR (MDBase/Rotational/LangevinR.h:59-270) and redeclares
// the methods of Condensate::run's loop body (Condensate/Condensate.cpp:288-378) with the reference's
// signatures, running each on the GB300 through the C ABI.  A driver changes the type of its integrator object
// and keeps its loop:
//
//     mtg_dropin::LangevinNVTRGPU b(geo, *pots);          // was: LangevinNVTR b(geo);
//     b.setdt(dt); b.setkT(kT); b.setgamma(g); b.setgammar(gr);
//     b.initialize(dat, mom, orient, angmom);
//     matrix<int> *pairs = b.calculatepairs_parallel(boxes, 3.5);
//     F = b.calculateforces(*pairs, wsa);
//     b.calculate_forces_and_torques3D(*pairs, *pots, F, T);
//     generate_uniform_random_matrix(RT);
//     b.create_forces_and_torques_sphere(F, T, RT);
//     for (...) { b.advancemom_halfstep(F, T); b.advance_pos(); b.rotate(); F = b.calculateforces(*pairs, wsa);
//                 T.reset(0); b.calculate_forces_and_torques3D(*pairs, *pots, F, T); generate_uniform_random_matrix(RT);
//                 b.create_forces_and_torques_sphere(F, T, RT); b.advancemom_halfstep(F, T); }
//
// Include it after the reference's own headers (it needs LangevinNVTR, cube, matrix<>, vector1<>, potential,
// HSPotential and the ComboPatch family).  The state lives on the device: the base class's host copies (dat,
// mom, orient, angmom) are refreshed by this class's getters, and calls made through a LangevinNVTR& to methods
// the base does not declare virtual reach the base's CPU code, not this class.  Parameters (setdt, setkT,
// setgamma, setgammar, setm, setmaxdistance) take effect when the device handle is created, at the first call
// after initialize.
#ifndef MTCODE_GB300_LANGEVINNVTRGPU_REFERENCE_HPP
#define MTCODE_GB300_LANGEVINNVTRGPU_REFERENCE_HPP

#include <memory>

#include "LangevinNVTRGPU.hpp"

namespace mtg_dropin {

// the ComboPatch of a driver in the C ABI's GeneralPatch form (TetrahedralPatch, BivalentPatch, GeneralPatch)
inline mtg_patch_model patch_model_of(ComboPatch &patches, int n) {
    mtg_patch_model m;
    if (TetrahedralPatch *t = dynamic_cast<TetrahedralPatch *>(&patches)) m = mtg_adapter::model_from_tetrahedral(*t);
    else if (BivalentPatch *b = dynamic_cast<BivalentPatch *>(&patches)) m = mtg_adapter::model_from_bivalent(*b);
    else if (GeneralPatch *g = dynamic_cast<GeneralPatch *>(&patches)) m = mtg_adapter::model_from_general(*g);
    else throw std::runtime_error("mtg_dropin: the patch model must be a TetrahedralPatch, BivalentPatch or GeneralPatch");
    if (m.n_types == 1 && m.count_per_type[0] == 0) m.count_per_type[0] = n;
    return m;
}

class LangevinNVTRGPU : public LangevinNVTR {
  public:
    // LangevinNVTR(cube&) (LangevinR.cpp:41-69) and the patch model the force routines will be given.
    // precision: MTG_FP64 (the reference's arithmetic, the default) or MTG_FP32 (the batched path's).
    LangevinNVTRGPU(cube &a, ComboPatch &patches, int precision = MTG_FP64, int device = 0)
        : LangevinNVTR(a), patches_(&patches), precision_(precision), device_(device) {}

    // HSPotential(eps, sigma) of calculateforces; HSPotential(1, 1) unless set here or seen by calculateforces
    // before the device handle exists
    void sethardcore(double eps, double sigma) {
        hs_eps_ = eps;
        hs_sigma_ = sigma;
    }

    // LangevinNVTR::initialize(x, p, Q, L) (LangevinR.cpp:309-325): the base's host copies, then the device state
    void initialize(matrix<double> &x, matrix<double> &p, matrix<double> &Q, matrix<double> &L) {
        LangevinNVTR::initialize(x, p, Q, L);
        gpu_.reset();
        pending_ = true;
    }

    // MD::calculatepairs_parallel(boxlist, rc) (MD.h:83): new P x 2 matrix, the caller deletes it
    matrix<int> *calculatepairs_parallel(matrix<int> &boxlist, double rc) {
        return gpu().calculatepairs_parallel(boxlist, rc);
    }

    // MD::calculateforces(pairs, potential) (MD.h:110) for the WCA core HSPotential the handle holds
    matrix<double> calculateforces(matrix<int> &pairs, potential &iny) {
        if (HSPotential *hs = dynamic_cast<HSPotential *>(&iny)) {
            if (!gpu_) sethardcore(hs->epsilon, hs->sigma);
            else if (hs->epsilon != hs_eps_ || hs->sigma != hs_sigma_)
                throw std::runtime_error("mtg_dropin: calculateforces was given an HSPotential other than the handle's");
        } else {
            throw std::runtime_error("mtg_dropin: calculateforces runs the HSPotential core only");
        }
        return gpu().calculateforces(pairs, iny);
    }

    // LangevinNVTR::calculate_forces_and_torques3D(pairs, ComboPatch, F, T) (LangevinR.h:247): adds to F and T
    void calculate_forces_and_torques3D(matrix<int> &pairs, ComboPatch &iny, matrix<double> &F, matrix<double> &T) {
        if (&iny != patches_) throw std::runtime_error("mtg_dropin: a different ComboPatch than the constructor's");
        gpu().calculate_forces_and_torques3D(pairs, iny, F, T);
    }

    // LangevinNVTR::create_forces_and_torques_sphere(F, T, R) (LangevinR.h:244)
    void create_forces_and_torques_sphere(matrix<double> &F, matrix<double> &T, matrix<double> &R) {
        gpu().create_forces_and_torques_sphere(F, T, R);
    }

    // LangevinNVTR::advancemom_halfstep(F, T) (LangevinR.h:259), LangevinNVT::advance_pos(), LangevinNVTR::rotate()
    void advancemom_halfstep(matrix<double> &F, matrix<double> &T) {
        gpu().advancemom_halfstep(F, T);
        stale_ = true;
    }
    void advance_pos() {
        gpu().advance_pos();
        stale_ = true;
    }
    void rotate() {
        gpu().rotate();
        stale_ = true;
    }

    // LangevinNVTR::measured_temperature(vector1<double>&) (LangevinR.cpp:170-193)
    void measured_temperature(vector1<double> &out) { gpu().measured_temperature(out); }

    // the state, read back from the device into the base's host copies
    matrix<double> getdat() {
        sync();
        return *dat;
    }
    matrix<double> getmom() {
        sync();
        return *mom;
    }
    matrix<double> &getorientation() {
        sync();
        return *orient;
    }
    matrix<double> &getangmom() {
        sync();
        return *angmom;
    }

    // the standalone adapter behind this class (for mtg_step-style fused steps: gpu().init_forces(); gpu().step(n))
    ::LangevinNVTRGPU<matrix<double>> &gpu() {
        if (!gpu_) create();
        return *gpu_;
    }

  private:
    void create() {
        const int n = dat->getNsafe();
        mtg_patch_model model = patch_model_of(*patches_, n);
        gpu_.reset(new ::LangevinNVTRGPU<matrix<double>>(geo.l, geo.pb[0], n, model, precision_, device_));
        gpu_->setdt(dt);
        gpu_->setkT(kT);
        gpu_->setgamma(gamma);
        gpu_->setgammar(gammar);
        gpu_->setm(m);
        gpu_->setinertia(im[0]);
        gpu_->setmaxdistance(max_distance_check);
        gpu_->sethardcore(hs_eps_, hs_sigma_);
        if (pending_) {
            gpu_->initialize(*dat, *mom, *orient, *angmom);
            pending_ = false;
        }
        stale_ = false;
    }
    void sync() {
        if (!gpu_ || !stale_) return;
        gpu_->getdat(*dat);
        gpu_->getmom(*mom);
        gpu_->getorientation(*orient);
        gpu_->getangmom(*angmom);
        stale_ = false;
    }

    ComboPatch *patches_;
    int precision_, device_;
    double hs_eps_ = 1.0, hs_sigma_ = 1.0;
    bool pending_ = false, stale_ = false;
    std::unique_ptr<::LangevinNVTRGPU<matrix<double>>> gpu_;
};

}  // namespace mtg_dropin

#endif  // MTCODE_GB300_LANGEVINNVTRGPU_REFERENCE_HPP
