// condensate_gpu.cpp -- the Condensate::run loop (Condensate/Condensate.cpp:288-420) driven through
// the C++ adapter include/LangevinNVTRGPU.hpp, the way a maintainer of the reference would call it.
// Reads an input file written by the test (n, box, precision, kT, steps, x[n*3], Q[n*9]) and writes
// the forces, torques, per-step temperatures and the final state to an output file.
#include <cmath>
#include <cstdio>
#include <vector>

#include "LangevinNVTRGPU.hpp"

// a minimal row-major matrix with the interface the adapter uses (the reference's matrix<double>
// offers the same operator()(i, j))
struct Mat {
    int r = 0, c = 0;
    std::vector<double> v;
    Mat(int rr = 0, int cc = 0) : r(rr), c(cc), v((size_t)rr * cc, 0.0) {}
    double &operator()(int i, int j) { return v[(size_t)c * i + j]; }
    void resize(long rr, int cc) { r = (int)rr; c = cc; v.assign((size_t)rr * cc, 0.0); }
};
struct IMat {
    long r = 0;
    std::vector<int> v;
    int &operator()(long i, int j) { return v[2 * i + j]; }
    void resize(long rr, int) { r = rr; v.assign(2 * rr, 0); }
};

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: condensate_gpu in.bin out.bin\n"); return 2; }
    std::FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[3];
    double par[3];
    if (std::fread(hdr, sizeof(int), 3, f) != 3 || std::fread(par, sizeof(double), 3, f) != 3) return 2;
    const int n = hdr[0], precision = hdr[1], steps = hdr[2];
    const double box = par[0], kT = par[1], dt = par[2];
    Mat x(n, 3), p(n, 3), L(n, 3), Q(n, 9), F(n, 3), T(n, 3);
    if (std::fread(x.v.data(), sizeof(double), x.v.size(), f) != x.v.size()) return 2;
    if (std::fread(Q.v.data(), sizeof(double), Q.v.size(), f) != Q.v.size()) return 2;
    std::fclose(f);
    try {
        mtg_patch_model model;
        mtg_model_tetrahedral(&model, 8.0, 1.2, std::acos(0.90));    // TetrahedralPatch(8, 1.2, acos .9)
        LangevinNVTRGPU<Mat> obj(box, true, n, model, precision);
        obj.setdt(dt);
        obj.setkT(kT);
        obj.setgamma(1.0);
        obj.setgammar(1.0);
        obj.initialize(x, p, Q, L);
        obj.calculate_forces_and_torques3D(F, T);
        IMat pairs;
        obj.calculatepairs_parallel(1.68, pairs);
        obj.init_forces();
        std::vector<double> temps;
        double meas[6];
        for (int i = 0; i < steps; i++) {                         // Condensate.cpp:335-378
            obj.measured_temperature(meas);
            temps.insert(temps.end(), meas, meas + 6);
            obj.step(1);
        }
        obj.getdat(x);
        obj.getmom(p);
        obj.getorientation(Q);
        obj.getangmom(L);
        std::FILE *o = std::fopen(argv[2], "wb");
        long np = pairs.r;
        std::fwrite(&np, sizeof(long), 1, o);
        std::fwrite(pairs.v.data(), sizeof(int), pairs.v.size(), o);
        for (Mat *m : {&F, &T, &x, &p, &Q, &L}) std::fwrite(m->v.data(), sizeof(double), m->v.size(), o);
        std::fwrite(temps.data(), sizeof(double), temps.size(), o);
        std::fclose(o);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
