// reference_dropin.cpp -- compile check: the adapter instantiated with the REFERENCE's own types
// (matrix<double>, matrix<int>, vector1<double>, TetrahedralPatch), exactly as Condensate::run would
// use it.  Built by tests/test_adapter.py only where the reference sources are present.
#include <stdlib.h>
#include <iostream>
#include <fstream>
#include <vector>
#include <algorithm>
#include <sstream>
#include <string>
#include <iomanip>
#include <random>
#include <chrono>
#include <unistd.h>
#include <execinfo.h>
#include <signal.h>
#include <sys/stat.h>
typedef int omp_int_t;
inline omp_int_t omp_get_thread_num() { return 0; }
inline omp_int_t omp_get_max_threads() { return 1; }
inline omp_int_t omp_get_num_threads() { return 1; }
using namespace std;
#include "Basic/basic.h"
#include "DataStructures/vector1.h"
#include "DataStructures/matrix2.h"
#include "DataStructures/matrix2.cpp"
#include "MDBase/MD.h"
#include "MDBase/Langevin.h"
#include "Condensate/Condensate.h"

#include "LangevinNVTRGPU.hpp"
#include "LangevinNVTRGPU_reference.hpp"

// Condensate::run's loop with the step on the GPU; the reference's TetrahedralPatch parameters feed
// the GeneralPatch-form model of the C ABI
void run_on_gpu(double l, int N, matrix<double> &dat, int runtime, TetrahedralPatch &pots) {
    mtg_patch_model model;
    mtg_model_tetrahedral(&model, pots.str, pots.dis, pots.ang);
    LangevinNVTRGPU<matrix<double>> obj(l, true, N, model);
    obj.setdt(0.005);
    obj.setkT(1.0);
    matrix<double> mom(N, 3), ang(N, 3), orient(N, 9);
    for (int i = 0; i < N; i++) orient(i, 0) = orient(i, 4) = orient(i, 8) = 1.0;
    obj.initialize(dat, mom, orient, ang);
    matrix<double> F(N, 3), T(N, 3);
    obj.calculate_forces_and_torques3D(F, T);
    matrix<int> pairs;
    obj.calculatepairs_parallel(3.5, pairs);
    // the bonded drivers' bond list is the reference's own matrix<int> (mainActivePolymer.cpp:390)
    matrix<int> bp2(N - 1, 2);
    for (int i = 0; i + 1 < N; i++) {
        bp2(i, 0) = i;
        bp2(i, 1) = i + 1;
    }
    obj.setbonds(bp2, 100.0, 1.0);
    obj.init_forces();
    vector1<double> meas(6);
    for (int i = 0; i < runtime; i++) {
        obj.measured_temperature(meas);
        obj.step(1);
    }
    obj.getdat(dat);
    obj.getorientation(orient);
}

// Condensate::run_singlebond's loop with the force pass on the GPU: the reference's binding models and
// BinaryBindStore go through the adapter unchanged
void run_singlebond_on_gpu(double l, int N, matrix<double> &dat, int runtime, TetrahedralPatch &pots) {
    mtg_patch_model model;
    mtg_model_tetrahedral(&model, pots.str, pots.dis, pots.ang);
    LangevinNVTRGPU<matrix<double>> obj(l, true, N, model);
    obj.sethardcore(3.0, 1.0);   // HSPotential wsa(3.0, size_mol) (Condensate.cpp:440)
    BindingModelSingle single(1.0, 0.1);
    BindingModelBinary binary(2 * N);
    binary.setup_equilibrium();
    SortingFunctionUniform fu;
    fu.div1 = N;
    fu.div2 = 2 * N;
    BindingModelTernary<SortingFunctionUniform> ternary(fu);
    SortingFunctionNonUniform fn;
    fn.div1 = N;
    fn.div2 = 2 * N;
    fn.np = 3;
    BindingModelTernary<SortingFunctionNonUniform> ternary2(fn);
    mtg_binding_model tables[4] = {mtg_adapter::binding_single_from(single), mtg_adapter::binding_binary_from(binary),
                                   mtg_adapter::binding_ternary_uniform_from(ternary),
                                   mtg_adapter::binding_ternary_nonuniform_from(ternary2)};
    obj.setsinglebond(tables[0]);
    matrix<double> mom(N, 3), ang(N, 3), orient(N, 9);
    for (int i = 0; i < N; i++) orient(i, 0) = orient(i, 4) = orient(i, 8) = 1.0;
    obj.initialize(dat, mom, orient, ang);
    BinaryBindStore bbs;
    vector1<bool> isbound(4 * N);
    vector1<int> boundto(4 * N);
    bbs.isbound = isbound;
    bbs.boundto = boundto;
    obj.setbindings(bbs.isbound, bbs.boundto);
    // run_singlebond's random initial binding (Condensate.cpp:478-484), with its argument types
    vector<patchint> opairs;
    vector<int> runs_diff;
    obj.setup_random_binding(opairs, runs_diff, pots, bbs, single, 7);
    matrix<double> F(N, 3), T(N, 3);
    obj.calculate_forces_and_torques3D_onlyone_nonlets(F, T);
    obj.init_forces();
    for (int i = 0; i < runtime; i++) obj.step(1);
    obj.getbindings(bbs.isbound, bbs.boundto);
    obj.getdat(dat);
}

// Condensate::run's own loop body (Condensate.cpp:288-378) with the integrator object swapped for the subclass of
// LangevinNVTR: every call keeps the reference's signature and argument types
void condensate_loop_with_the_subclass(double l, matrix<double> &dat, int runtime, ComboPatch *pots) {
    vector1<bool> pb(3, true);
    cube geo(l, pb, 3);
    mtg_dropin::LangevinNVTRGPU b(geo, *pots);
    b.setdt(0.005);
    b.setkT(1.0);
    b.setgamma(1.0);
    b.setgammar(1.0);
    const int NN = dat.getNsafe();
    matrix<double> mom(NN, 3), ang(NN, 3), orient(NN, 9);
    for (int i = 0; i < NN; i++) orient(i, 0) = orient(i, 4) = orient(i, 8) = 1.0;
    b.initialize(dat, mom, orient, ang);
    int ccc;
    matrix<int> boxes = b.getgeo().generate_boxes_relationships(10, ccc);
    matrix<int> *pairs = b.calculatepairs_parallel(boxes, 3.5);
    HSPotential wsa(3.0, 1.0);
    matrix<double> F(NN, 3), T(NN, 3), RT(NN, 6), zeromatrix(NN, 3);
    F = b.calculateforces(*pairs, wsa);
    b.calculate_forces_and_torques3D(*pairs, *pots, F, T);
    generate_uniform_random_matrix(RT);
    b.create_forces_and_torques_sphere(F, T, RT);
    vector1<double> meas(6);
    for (int i = 0; i < runtime; i++) {
        b.measured_temperature(meas);
        b.advancemom_halfstep(F, T);
        b.advance_pos();
        b.rotate();
        F = b.calculateforces(*pairs, wsa);
        T = zeromatrix;
        b.calculate_forces_and_torques3D(*pairs, *pots, F, T);
        generate_uniform_random_matrix(RT);
        b.create_forces_and_torques_sphere(F, T, RT);
        b.advancemom_halfstep(F, T);
    }
    delete pairs;
    dat = b.getdat();
}

// the reference's own patch objects converted to the C ABI's model, without hand-filled arrays
void patch_models(int N) {
    TetrahedralPatch tp(8.0, 1.2, acos(0.9));
    BivalentPatch bp(8.0, 1.2, acos(0.9));
    vector1<int> ppt(1), npt(1);
    ppt[0] = 4;
    npt[0] = N;
    matrix<double> params(16, 3), orient(4, 3);
    for (int q = 0; q < 16; q++) {
        params(q, 0) = 10.0;
        params(q, 1) = 1.15;
        params(q, 2) = acos(0.92);
    }
    orient(0, 2) = 1.0;
    orient(1, 2) = -1.0;
    orient(2, 0) = 1.0;
    orient(3, 0) = -1.0;
    GeneralPatch gp(ppt, npt, params, orient);
    mtg_patch_model m[3] = {mtg_adapter::model_from_tetrahedral(tp), mtg_adapter::model_from_bivalent(bp),
                            mtg_adapter::model_from_general(gp)};
    (void)m;
    mtg_patch_model d = mtg_dropin::patch_model_of(gp, N);
    (void)d;
}

int main() { return 0; }
