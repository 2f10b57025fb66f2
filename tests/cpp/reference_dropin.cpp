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
    matrix<double> F(N, 3), T(N, 3);
    obj.calculate_forces_and_torques3D_onlyone_nonlets(F, T);
    obj.init_forces();
    for (int i = 0; i < runtime; i++) obj.step(1);
    obj.getbindings(bbs.isbound, bbs.boundto);
    obj.getdat(dat);
}

int main() { return 0; }
