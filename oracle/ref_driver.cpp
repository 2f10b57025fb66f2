// ref_driver.cpp -- thin extern "C" shim over the reference's OWN routines (osmanovicdino/mtcode),
// compiled from the reference sources where they lie (the build recipe oracle/build_ref.sh passes
// -I <reference>/Code).  TEST INFRASTRUCTURE: used only to pin the oracle (oracle.c) and to generate
// the golden fixtures under tests/golden/.  Nothing in the product links it.
//
// Each entry point drives the reference classes exactly the way Condensate::run does
// (Condensate/Condensate.cpp:288-420), on a periodic or reflecting cube built directly
// (the Condensate constructor itself hard-codes a reflecting box, Condensate.cpp:19-20).
// Built WITHOUT -fopenmp: the reference's force/torque scatter is unsynchronised under OpenMP
// (MD.cpp:1754-1758, LangevinR.cpp:1023-1037), so golden values come from the serial build.

#include <stdlib.h>
#include <iostream>
#include <fstream>
#include <stdio.h>
#include <stdarg.h>
#include <vector>
#include <algorithm>
#include <stdexcept>
#include <sstream>
#include <string>
#include <iomanip>
#include <sys/stat.h>
#include <random>
#include <chrono>
#include <unistd.h>
#include <execinfo.h>
#include <signal.h>

typedef int omp_int_t;
inline omp_int_t omp_get_thread_num() { return 0; }
inline omp_int_t omp_get_max_threads() { return 1; }
inline omp_int_t omp_get_num_threads() { return 1; }

using namespace std;
using namespace std::chrono;

#include "Basic/basic.h"
#include "DataStructures/vector1.h"
#include "DataStructures/matrix2.h"
#include "DataStructures/matrix2.cpp"
#include "MDBase/MD.h"
#include "MDBase/Langevin.h"
#include "Condensate/Condensate.h"

namespace {

// model_kind: 0 = TetrahedralPatch(att, dis, thetam), 1 = BivalentPatch(att, dis, thetam),
//             2 = GeneralPatch from (n_types, patches_per_type, num_per_type, orient, params)
struct RefModelDesc {
    int kind;
    double att, dis, thetam;
    int n_types;
    const int *patches_per_type;
    const int *num_per_type;
    const double *orient;   // rows x 3
    const double *params;   // n_pots x 3 (att, dis, thetam)
};

ComboPatch *make_model(const RefModelDesc &d)
{
    if (d.kind == 0) return new TetrahedralPatch(d.att, d.dis, d.thetam);
    if (d.kind == 1) return new BivalentPatch(d.att, d.dis, d.thetam);
    vector1<int> npt(d.n_types), nper(d.n_types);
    int nor = 0, npots = 0;
    for (int k = 0; k < d.n_types; k++) {
        npt[k] = d.patches_per_type[k];
        nper[k] = d.num_per_type[k];
        nor += d.patches_per_type[k];
    }
    for (int a = 0; a < d.n_types; a++)
        for (int b = a; b < d.n_types; b++) npots += d.patches_per_type[a] * d.patches_per_type[b];
    matrix<double> params(npots, 3), orient(nor, 3);
    for (int i = 0; i < npots; i++)
        for (int k = 0; k < 3; k++) params(i, k) = d.params[3 * i + k];
    for (int i = 0; i < nor; i++)
        for (int k = 0; k < 3; k++) orient(i, k) = d.orient[3 * i + k];
    return new GeneralPatch(npt, nper, params, orient);
}

matrix<double> to_mat(const double *a, int n, int c)
{
    matrix<double> m(n, c);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < c; k++) m(i, k) = a[(size_t)c * i + k];
    return m;
}

void from_mat(matrix<double> &m, double *a, int n, int c)
{
    for (int i = 0; i < n; i++)
        for (int k = 0; k < c; k++) a[(size_t)c * i + k] = m(i, k);
}

LangevinNVTR *make_system(int n, double box, int periodic, const double *x, const double *p, const double *Lb,
                          const double *Q, double dt, double kT, double gamma, double gammar)
{
    vector1<bool> pb(3, periodic != 0);
    cube geo(box, pb, 3);
    LangevinNVTR *b = new LangevinNVTR(geo);
    matrix<double> X = to_mat(x, n, 3), Pm = to_mat(p, n, 3), L = to_mat(Lb, n, 3), O = to_mat(Q, n, 9);
    b->initialize(X, Pm, O, L);
    b->setdt(dt);
    b->setgamma(gamma);
    b->setgammar(gammar);
    b->setkT(kT);
    return b;
}

}  // namespace

extern "C" {

// MD::calculatepairs (MD.cpp:1035-1098) with boxes from cube::generate_boxes_relationships(ncell).
long ref_pairs(int n, double box, int periodic, const double *x, int ncell, double rc, int *out, long cap)
{
    vector<double> zeros3(3 * (size_t)n, 0.0), zeros9(9 * (size_t)n, 0.0);
    LangevinNVTR *b = make_system(n, box, periodic, x, zeros3.data(), zeros3.data(), zeros9.data(), 0.005, 1, 1, 1);
    int ccc;
    matrix<int> boxes = b->getgeo().generate_boxes_relationships(ncell, ccc);
    matrix<int> *pairs = b->calculatepairs(boxes, rc);
    long np = pairs->getNsafe();
    for (long i = 0; i < np && i < cap; i++) {
        out[2 * i] = (*pairs)(i, 0);
        out[2 * i + 1] = (*pairs)(i, 1);
    }
    delete pairs;
    delete b;
    return np;
}

// Same pair build through MD::calculatepairs_parallel + SingleHistogramParallel (MD.cpp:1100-1176).
long ref_pairs_parallel(int n, double box, int periodic, const double *x, int ncell, double rc, int *out, long cap)
{
    vector<double> zeros3(3 * (size_t)n, 0.0), zeros9(9 * (size_t)n, 0.0);
    LangevinNVTR *b = make_system(n, box, periodic, x, zeros3.data(), zeros3.data(), zeros9.data(), 0.005, 1, 1, 1);
    int ccc;
    matrix<int> boxes = b->getgeo().generate_boxes_relationships(ncell, ccc);
    matrix<int> *pairs = b->calculatepairs_parallel(boxes, rc);
    long np = pairs->getNsafe();
    for (long i = 0; i < np && i < cap; i++) {
        out[2 * i] = (*pairs)(i, 0);
        out[2 * i + 1] = (*pairs)(i, 1);
    }
    delete pairs;
    delete b;
    return np;
}

// F = MD::calculateforces(pairs, HSPotential(eps, sigma)); T = 0;
// LangevinNVTR::calculate_forces_and_torques3D(pairs, ComboPatch, F, T)   (Condensate.cpp:370-374)
void ref_forces(int n, double box, int periodic, const double *x, const double *Q, int ncell, double rc,
                double hs_eps, double hs_sigma, int kind, double att, double dis, double thetam, int n_types,
                const int *ppt, const int *npt, const double *orient, const double *params, double *F, double *T)
{
    vector<double> zeros3(3 * (size_t)n, 0.0);
    LangevinNVTR *b = make_system(n, box, periodic, x, zeros3.data(), zeros3.data(), Q, 0.005, 1, 1, 1);
    RefModelDesc d = {kind, att, dis, thetam, n_types, ppt, npt, orient, params};
    ComboPatch *pots = make_model(d);
    int ccc;
    matrix<int> boxes = b->getgeo().generate_boxes_relationships(ncell, ccc);
    matrix<int> *pairs = b->calculatepairs(boxes, rc);
    HSPotential wsa(hs_eps, hs_sigma);
    matrix<double> Fm = b->calculateforces(*pairs, wsa);
    matrix<double> Tm(n, 3);
    Tm.reset_parallel(0.0);
    b->calculate_forces_and_torques3D(*pairs, *pots, Fm, Tm);
    from_mat(Fm, F, n, 3);
    from_mat(Tm, T, n, 3);
    delete pairs;
    delete pots;
    delete b;
}

// F = MD::calculateforces(bond list, HarmonicPotential(k, r0))  (MD.cpp:1684-1764, potential.h:265-297),
// the bonded term of the polymer drivers (mainActivePolymer.cpp:390).
void ref_bond_forces(int n, double box, int periodic, const double *x, const int *bonds, long nb, double k, double r0,
                     double *F)
{
    vector<double> zeros3(3 * (size_t)n, 0.0), zeros9(9 * (size_t)n, 0.0);
    LangevinNVTR *b = make_system(n, box, periodic, x, zeros3.data(), zeros3.data(), zeros9.data(), 0.005, 1, 1, 1);
    matrix<int> bp((int)nb, 2);
    for (long i = 0; i < nb; i++) {
        bp(i, 0) = bonds[2 * i];
        bp(i, 1) = bonds[2 * i + 1];
    }
    HarmonicPotential pot(k, r0);
    matrix<double> Fm = b->calculateforces(bp, pot);
    from_mat(Fm, F, n, 3);
    delete b;
}

// The force pass of a bonded patchy system, summed as the polymer drivers do (mainActivePolymer.cpp:
// 390-402): F = calculateforces(bonds, HarmonicPotential(k, r0)); F += calculateforces(pairs,
// HSPotential); T = 0; calculate_forces_and_torques3D(pairs, ComboPatch, F, T).
void ref_forces_bonded(int n, double box, int periodic, const double *x, const double *Q, int ncell, double rc,
                       double hs_eps, double hs_sigma, int n_types, const int *ppt, const int *npt, const double *orient,
                       const double *params, const int *bonds, long nb, double k, double r0, double *F, double *T)
{
    vector<double> zeros3(3 * (size_t)n, 0.0);
    LangevinNVTR *b = make_system(n, box, periodic, x, zeros3.data(), zeros3.data(), Q, 0.005, 1, 1, 1);
    RefModelDesc d = {2, 0.0, 0.0, 0.0, n_types, ppt, npt, orient, params};
    ComboPatch *pots = make_model(d);
    int ccc;
    matrix<int> boxes = b->getgeo().generate_boxes_relationships(ncell, ccc);
    matrix<int> *pairs = b->calculatepairs(boxes, rc);
    matrix<int> bp((int)nb, 2);
    for (long i = 0; i < nb; i++) {
        bp(i, 0) = bonds[2 * i];
        bp(i, 1) = bonds[2 * i + 1];
    }
    HarmonicPotential bond(k, r0);
    HSPotential wsa(hs_eps, hs_sigma);
    matrix<double> Fm = b->calculateforces(bp, bond);
    matrix<double> F2 = b->calculateforces(*pairs, wsa);
    Fm += F2;
    matrix<double> Tm(n, 3);
    Tm.reset_parallel(0.0);
    b->calculate_forces_and_torques3D(*pairs, *pots, Fm, Tm);
    from_mat(Fm, F, n, 3);
    from_mat(Tm, T, n, 3);
    delete pairs;
    delete pots;
    delete b;
}

// The frame writer and reader of Condensate::run: ofstream << = matrix (matrix2.cpp:898-912) and
// importcsv (matrix2.cpp:1597-1640).
void ref_write_csv(const char *path, const double *a, int rows, int cols)
{
    matrix<double> m(rows, cols);
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) m(i, j) = a[(size_t)i * cols + j];
    ofstream f(path);
    f <<= m;
    f.close();
}

long ref_import_csv(const char *path, double *out, long cap, int *cols)
{
    bool err = false;
    matrix<double> m = importcsv(string(path), 0.0, err);
    if (err) return -1;
    long nr = m.getNsafe();
    *cols = m.getncols();
    for (long i = 0; i < nr && (i + 1) * (long)*cols <= cap; i++)
        for (int j = 0; j < *cols; j++) out[i * *cols + j] = m(i, j);
    return nr;
}

// calcg1 (MDBase/Analysis/PairCorrelation.cpp:9-153): returns the bin count, hist receives <= cap bins
long ref_calcg1(int n, double box, int periodic, const double *x, double max, double dx, long *hist, long cap)
{
    vector1<bool> pb(3, periodic != 0);
    cube geo(box, pb, 3);
    matrix<double> X = to_mat(x, n, 3);
    vector1<int> g = calcg1(X, geo, max, dx);
    long m = g.getsize();
    for (long i = 0; i < m && i < cap; i++) hist[i] = g[i];
    return m;
}

// distance_graph (MDBase/Analysis/AnalyzeGrowth.cpp:136-171) on cells of side >= cut, every pair kept
void ref_distance_graph(int n, double box, int periodic, const double *x, double cut, int *labels)
{
    vector1<bool> pb(3, periodic != 0);
    cube geo(box, pb, 3);
    matrix<double> X = to_mat(x, n, 3);
    int ccc;
    int num = (int)floor(box / cut);
    matrix<int> boxes = geo.generate_boxes_relationships(num, ccc);
    index_test all;
    vector1<int> lab = distance_graph(X, boxes, geo, cut, &all);
    for (int i = 0; i < n; i++) labels[i] = lab[i];
}

// Condensate::run loop body (Condensate.cpp:335-378), nsteps times.  Pairs are rebuilt from the
// positions at the start of a step every `rebuild` steps (the driver uses 20 at rc 3.5).
// noise: nsteps x n x 6 values used in place of generate_uniform_random_matrix, or NULL for zeros.
// Ft/Tt are the carried F~ (lab) / T~ (body) in and out.  If init != 0 they are first computed as the
// driver does before its loop (Condensate.cpp:312-334) with noise0 (n x 6, or NULL for zeros).
void ref_run(int n, double box, int periodic, double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt,
             double dt, double kT, double gamma, double gammar, double hs_eps, double hs_sigma, int kind, double att,
             double dis, double thetam, int n_types, const int *ppt, const int *npt, const double *orient,
             const double *params, int ncell, double rc, int rebuild, int nsteps, const double *noise, int init,
             const double *noise0, double *temperature_out)
{
    LangevinNVTR *obj = make_system(n, box, periodic, x, p, Lb, Q, dt, kT, gamma, gammar);
    RefModelDesc d = {kind, att, dis, thetam, n_types, ppt, npt, orient, params};
    ComboPatch *pots = make_model(d);
    int ccc;
    matrix<int> boxes = obj->getgeo().generate_boxes_relationships(ncell, ccc);
    matrix<int> *pairs = obj->calculatepairs(boxes, rc);
    HSPotential wsa(hs_eps, hs_sigma);
    matrix<double> F(n, 3), T(n, 3), RT(n, 6);
    if (init) {
        F = obj->calculateforces(*pairs, wsa);
        obj->calculate_forces_and_torques3D(*pairs, *pots, F, T);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 6; k++) RT(i, k) = noise0 ? noise0[6 * (size_t)i + k] : 0.0;
        obj->create_forces_and_torques_sphere(F, T, RT);
    } else {
        F = to_mat(Ft, n, 3);
        T = to_mat(Tt, n, 3);
    }
    for (int i = 0; i < nsteps; i++) {
        if (temperature_out) {
            vector1<double> meas(6);
            obj->measured_temperature(meas);
            for (int k = 0; k < 6; k++) temperature_out[6 * (size_t)i + k] = meas[k];
        }
        if (i > 0 && (rebuild <= 1 || i % rebuild == 0)) {
            delete pairs;
            pairs = obj->calculatepairs(boxes, rc);
        }
        obj->advancemom_halfstep(F, T);
        obj->advance_pos();
        obj->rotate();
        F = obj->calculateforces(*pairs, wsa);
        T.reset_parallel(0.0);
        obj->calculate_forces_and_torques3D(*pairs, *pots, F, T);
        for (int a = 0; a < n; a++)
            for (int k = 0; k < 6; k++) RT(a, k) = noise ? noise[((size_t)i * n + a) * 6 + k] : 0.0;
        obj->create_forces_and_torques_sphere(F, T, RT);
        obj->advancemom_halfstep(F, T);
    }
    matrix<double> X = obj->getdat(), P = obj->getmom();
    from_mat(X, x, n, 3);
    from_mat(P, p, n, 3);
    from_mat(obj->getangmom(), Lb, n, 3);
    from_mat(obj->getorientation(), Q, n, 9);
    from_mat(F, Ft, n, 3);
    from_mat(T, Tt, n, 3);
    delete pairs;
    delete pots;
    delete obj;
}

// One call of the single-bond force pass as Condensate::run_singlebond makes it (Condensate.cpp:430-470):
// pairs = calculatepairs(boxes, pair_cut), opairs = calculate_patch_list(*pairs, *pots), runs_diff =
// adjacency(opairs), then srand(seed) and calculate_forces_and_torques3D_onlyone_nonlets(opairs, runs_diff,
// *pots, bbs, *bm, F, T) from F = T = 0.  Binding model bm_kind: 0 BindingModelSingle(args[0] on, args[1] off),
// 1 BindingModelBinary(args[0] div) + setup_equilibrium(), 2 BindingModelTernary<SortingFunctionUniform>
// (div1 args[0], div2 args[1]) + setup(args[2..16]), 3 BindingModelTernary<SortingFunctionNonUniform>
// (div1, div2, np = args[0..2]) + setup(args[3..17]).  Outputs: boundto / isbound updated in place, F, T,
// the candidate list (plist, 5 ints per entry, up to plist_cap; the count is returned), the model's rate
// vectors in tables (doubr11, 12, 13, 22, 23, 33 then tripr111 ... 333, zero where the model has none) and
// max_ang / max_check in caps[0..1].
static long singlebond_call(int n, double box, int periodic, const double *x, const double *Q, int ncell,
                            double pair_cut, int kind, double att, double dis, double thetam, int n_types,
                            const int *ppt, const int *npt, const double *orient, const double *params, int bm_kind,
                            const double *args, int *boundto, unsigned char *isbound, unsigned seed, double *F,
                            double *T, int *plist, long plist_cap, double *tables, double *caps, int setup);

long ref_singlebond(int n, double box, int periodic, const double *x, const double *Q, int ncell, double pair_cut,
                    int kind, double att, double dis, double thetam, int n_types, const int *ppt, const int *npt,
                    const double *orient, const double *params, int bm_kind, const double *args, int *boundto,
                    unsigned char *isbound, unsigned seed, double *F, double *T, int *plist, long plist_cap,
                    double *tables, double *caps)
{
    return singlebond_call(n, box, periodic, x, Q, ncell, pair_cut, kind, att, dis, thetam, n_types, ppt, npt, orient,
                           params, bm_kind, args, boundto, isbound, seed, F, T, plist, plist_cap, tables, caps, 0);
}

// LangevinNVTR::setup_random_binding(opairs, runs_diff, *pots, bbs, *bm) (LangevinRforceUtil.cpp:749-1010) on the
// same candidate list as ref_singlebond builds (Condensate.cpp:478-484); its edge order comes from
// std::random_device, so the result is one random draw of the reference's.  boundto / isbound updated in place.
long ref_setup_random_binding(int n, double box, int periodic, const double *x, const double *Q, int ncell,
                              double pair_cut, int kind, double att, double dis, double thetam, int n_types,
                              const int *ppt, const int *npt, const double *orient, const double *params, int bm_kind,
                              const double *args, int *boundto, unsigned char *isbound, int *plist, long plist_cap)
{
    return singlebond_call(n, box, periodic, x, Q, ncell, pair_cut, kind, att, dis, thetam, n_types, ppt, npt, orient,
                           params, bm_kind, args, boundto, isbound, 0u, nullptr, nullptr, plist, plist_cap, nullptr,
                           nullptr, 1);
}

static long singlebond_call(int n, double box, int periodic, const double *x, const double *Q, int ncell,
                            double pair_cut, int kind, double att, double dis, double thetam, int n_types,
                            const int *ppt, const int *npt, const double *orient, const double *params, int bm_kind,
                            const double *args, int *boundto, unsigned char *isbound, unsigned seed, double *F,
                            double *T, int *plist, long plist_cap, double *tables, double *caps, int setup)
{
    vector<double> zeros3(3 * (size_t)n, 0.0);
    LangevinNVTR *b = make_system(n, box, periodic, x, zeros3.data(), zeros3.data(), Q, 0.005, 1, 1, 1);
    RefModelDesc d = {kind, att, dis, thetam, n_types, ppt, npt, orient, params};
    ComboPatch *pots = make_model(d);
    int ccc;
    matrix<int> boxes = b->getgeo().generate_boxes_relationships(ncell, ccc);
    matrix<int> *pairs = b->calculatepairs(boxes, pair_cut);
    vector<patchint> opairs = b->calculate_patch_list(*pairs, *pots);
    vector<int> runs_diff = adjacency(opairs);
    int nh = pots->get_total_patches(n);
    BinaryBindStore bbs;
    vector1<bool> ib(nh);
    vector1<int> bt(nh);
    for (int i = 0; i < nh; i++) {
        ib[i] = isbound[i] != 0;
        bt[i] = boundto[i];
    }
    bbs.isbound = ib;
    bbs.boundto = bt;
    AbstractBindingModel *bm = nullptr;
    vector<const vector1<double> *> dv(6, nullptr), tv(10, nullptr);
    BindingModelBinary *bb = nullptr;
    SortingFunctionUniform fu;
    SortingFunctionNonUniform fn;
    BindingModelTernary<SortingFunctionUniform> *tu = nullptr;
    BindingModelTernary<SortingFunctionNonUniform> *tn = nullptr;
    if (bm_kind == 0) {
        bm = new BindingModelSingle(args[0], args[1]);
    } else if (bm_kind == 1) {
        bb = new BindingModelBinary((int)args[0]);
        bb->setup_equilibrium();
        bm = bb;
        dv[0] = &bb->doubr11; dv[1] = &bb->doubr12; dv[3] = &bb->doubr22;
        tv[0] = &bb->tripr111; tv[1] = &bb->tripr112; tv[3] = &bb->tripr122; tv[6] = &bb->tripr222;
    } else if (bm_kind == 2) {
        fu.div1 = (int)args[0];
        fu.div2 = (int)args[1];
        tu = new BindingModelTernary<SortingFunctionUniform>(fu);
        tu->setup(args[2], args[3], args[4], args[5], args[6], args[7], args[8], args[9], args[10], args[11],
                  args[12], args[13], args[14], args[15], args[16]);
        bm = tu;
    } else {
        fn.div1 = (int)args[0];
        fn.div2 = (int)args[1];
        fn.np = (int)args[2];
        tn = new BindingModelTernary<SortingFunctionNonUniform>(fn);
        tn->setup(args[3], args[4], args[5], args[6], args[7], args[8], args[9], args[10], args[11], args[12],
                  args[13], args[14], args[15], args[16], args[17]);
        bm = tn;
    }
    if (tu || tn) {
        auto fill = [&](auto *t) {
            dv[0] = &t->doubr11; dv[1] = &t->doubr12; dv[2] = &t->doubr13;
            dv[3] = &t->doubr22; dv[4] = &t->doubr23; dv[5] = &t->doubr33;
            tv[0] = &t->tripr111; tv[1] = &t->tripr112; tv[2] = &t->tripr113; tv[3] = &t->tripr122;
            tv[4] = &t->tripr123; tv[5] = &t->tripr133; tv[6] = &t->tripr222; tv[7] = &t->tripr223;
            tv[8] = &t->tripr233; tv[9] = &t->tripr333;
        };
        if (tu) fill(tu);
        else fill(tn);
    }
    if (tables) {
        for (int r = 0; r < 6; r++)
            for (int k = 0; k < 4; k++) tables[4 * r + k] = dv[r] && dv[r]->getsize() > k ? dv[r]->gpcons(k) : 0.0;
        for (int r = 0; r < 10; r++)
            for (int k = 0; k < 16; k++)
                tables[24 + 16 * r + k] = tv[r] && tv[r]->getsize() > k ? tv[r]->gpcons(k) : 0.0;
    }
    if (caps) {
        caps[0] = pots->max_ang;
        caps[1] = pots->max_check;
    }
    long np = (long)opairs.size();
    for (long q = 0; q < np && q < plist_cap; q++) {
        plist[5 * q + 0] = opairs[q].particle_index1;
        plist[5 * q + 1] = opairs[q].particle_index2;
        plist[5 * q + 2] = opairs[q].potn;
        plist[5 * q + 3] = opairs[q].patch_index1;
        plist[5 * q + 4] = opairs[q].patch_index2;
    }
    if (setup) {
        b->setup_random_binding(opairs, runs_diff, *pots, bbs, *bm);
    } else {
        matrix<double> Fm(n, 3), Tm(n, 3);
        Fm.reset_parallel(0.0);
        Tm.reset_parallel(0.0);
        srand(seed);
        b->calculate_forces_and_torques3D_onlyone_nonlets(opairs, runs_diff, *pots, bbs, *bm, Fm, Tm);
        from_mat(Fm, F, n, 3);
        from_mat(Tm, T, n, 3);
    }
    for (int i = 0; i < nh; i++) {
        isbound[i] = bbs.isbound[i] ? 1 : 0;
        boundto[i] = bbs.boundto[i];
    }
    delete bm;
    delete pairs;
    delete pots;
    delete b;
    return np;
}

// LangevinNVTR::genfullmat (LangevinR.cpp:392-461) for a single particle's body angular momentum.
void ref_rotation_matrix(double dt, const double *L, double *R)
{
    vector1<bool> pb(3, true);
    cube geo(10.0, pb, 3);
    LangevinNVTR b(geo);
    matrix<double> X(1, 3), P(1, 3), Lm(1, 3), O(1, 9);
    for (int k = 0; k < 3; k++) Lm(0, k) = L[k];
    O(0, 0) = O(0, 4) = O(0, 8) = 1.0;
    b.initialize(X, P, O, Lm);
    b.setdt(dt);
    vector1<double> up = b.genfullmat(0);
    for (int k = 0; k < 9; k++) R[k] = up[k];
}

}  // extern "C"
