// phases_gpu.cpp -- Condensate::run's loop body (Condensate/Condensate.cpp:288-378) called method by method
// through the C++ adapter include/LangevinNVTRGPU.hpp, with the reference's signatures: calculatepairs_parallel,
// calculateforces, calculate_forces_and_torques3D, create_forces_and_torques_sphere, advancemom_halfstep,
// advance_pos, rotate.  The patch model is converted from a GeneralPatch-shaped object (the members the
// reference's GeneralPatch has), not filled by hand.  Reads n, precision, steps, box, kT, dt, x, Q and the noise
// of every draw (steps + 1 blocks of n x 6); writes the pair count, F~ and T~ after the initial pass, and the
// final state.
#include <cmath>
#include <cstdio>
#include <vector>

#include "LangevinNVTRGPU.hpp"

// minimal row-major matrices with the interface the adapter uses (the reference's matrix<double> and
// matrix<int> offer the same operator()(i, j), (rows, cols) constructor and getnrows())
struct Mat {
    int r = 0, c = 0;
    std::vector<double> v;
    Mat(int rr = 0, int cc = 0) : r(rr), c(cc), v((size_t)rr * cc, 0.0) {}
    double &operator()(int i, int j) { return v[(size_t)c * i + j]; }
    int getnrows() const { return r; }
};
struct IMat {
    int r = 0;
    std::vector<int> v;
    IMat(int rr = 0, int = 2) : r(rr), v((size_t)rr * 2, 0) {}
    int &operator()(int i, int j) { return v[2 * (size_t)i + j]; }
};
// the public members of the reference's GeneralPatch (GeneralPatch.h) that the converter reads
struct GeneralPatchLike {
    int no_types = 1;
    int no_patches_per_type[1] = {4};
    int num_per_type[1] = {0};
    Mat orient{4, 3}, params{16, 3};
};
struct HSLike {};   // the HSPotential argument of calculateforces (the handle holds the core's parameters)

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: phases_gpu in.bin out.bin\n"); return 2; }
    std::FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[3];
    double par[3];
    if (std::fread(hdr, sizeof(int), 3, f) != 3 || std::fread(par, sizeof(double), 3, f) != 3) return 2;
    const int n = hdr[0], precision = hdr[1], steps = hdr[2];
    const double box = par[0], kT = par[1], dt = par[2];
    Mat x(n, 3), p(n, 3), L(n, 3), Q(n, 9), F(n, 3), T(n, 3);
    std::vector<Mat> noise(steps + 1, Mat(n, 6));
    if (std::fread(x.v.data(), sizeof(double), x.v.size(), f) != x.v.size()) return 2;
    if (std::fread(Q.v.data(), sizeof(double), Q.v.size(), f) != Q.v.size()) return 2;
    for (Mat &m : noise)
        if (std::fread(m.v.data(), sizeof(double), m.v.size(), f) != m.v.size()) return 2;
    std::fclose(f);
    try {
        GeneralPatchLike gp;   // the tetrahedral model as a one-type GeneralPatch
        gp.num_per_type[0] = n;
        const double tv[4][3] = {{std::sqrt(8. / 9.), 0., -1. / 3.}, {-std::sqrt(2. / 9.), std::sqrt(2. / 3.), -1. / 3.},
                                 {-std::sqrt(2. / 9.), -std::sqrt(2. / 3.), -1. / 3.}, {0., 0., 1.}};
        for (int i = 0; i < 4; i++)
            for (int c = 0; c < 3; c++) gp.orient(i, c) = tv[i][c];
        for (int q = 0; q < 16; q++) {
            gp.params(q, 0) = 8.0;
            gp.params(q, 1) = 1.2;
            gp.params(q, 2) = std::acos(0.90);
        }
        LangevinNVTRGPU<Mat> obj(box, true, n, mtg_adapter::model_from_general(gp), precision);
        obj.setdt(dt);
        obj.setkT(kT);
        obj.setgamma(1.0);
        obj.setgammar(1.0);
        obj.initialize(x, p, Q, L);
        IMat boxes;
        HSLike wsa;
        IMat *pairs = obj.calculatepairs_parallel(boxes, 3.5);      // Condensate.cpp:308
        F = obj.calculateforces(*pairs, wsa);                        // :322
        obj.calculate_forces_and_torques3D(*pairs, gp, F, T);        // :324
        obj.create_forces_and_torques_sphere(F, T, noise[0]);        // :333
        Mat F0 = F, T0 = T;
        for (int i = 0; i < steps; i++) {                            // :335-378
            obj.advancemom_halfstep(F, T);
            obj.advance_pos();
            obj.rotate();
            F = obj.calculateforces(*pairs, wsa);
            T = Mat(n, 3);
            obj.calculate_forces_and_torques3D(*pairs, gp, F, T);
            obj.create_forces_and_torques_sphere(F, T, noise[i + 1]);
            obj.advancemom_halfstep(F, T);
        }
        obj.getdat(x);
        obj.getmom(p);
        obj.getorientation(Q);
        obj.getangmom(L);
        long np = pairs->r;
        delete pairs;                                                // the caller deletes, Condensate.cpp:348-349
        std::FILE *o = std::fopen(argv[2], "wb");
        std::fwrite(&np, sizeof(long), 1, o);
        for (Mat *m : {&F0, &T0, &x, &p, &Q, &L}) std::fwrite(m->v.data(), sizeof(double), m->v.size(), o);
        std::fclose(o);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
