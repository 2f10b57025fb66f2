// singlebond_gpu.cpp -- Condensate::run_singlebond's loop (Condensate/Condensate.cpp:422-618) driven through
// the C++ adapter include/LangevinNVTRGPU.hpp: the binding model converted from an object with the
// reference's BindingModelSingle members, one onlyone_nonlets pass, the initial force pass and the steps.
// Reads (n, precision, steps, box, kT, dt, x[n*3], Q[n*9]); writes F, T and the bond state of the first
// pass, then the final x, Q and bond state.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "LangevinNVTRGPU.hpp"

struct Mat {
    int r = 0, c = 0;
    std::vector<double> v;
    Mat(int rr = 0, int cc = 0) : r(rr), c(cc), v((size_t)rr * cc, 0.0) {}
    double &operator()(int i, int j) { return v[(size_t)c * i + j]; }
};

// the public members the adapter reads from a reference BindingModelSingle (BindingModelSingle.h)
struct SingleRates {
    double on_rate, off_rate;
};

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: singlebond_gpu in.bin out.bin\n"); return 2; }
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
        mtg_model_tetrahedral(&model, 8.0, 1.2, std::acos(0.70));
        LangevinNVTRGPU<Mat> obj(box, true, n, model, precision);
        obj.setdt(dt);
        obj.setkT(kT);
        obj.setgamma(1.0);
        obj.setgammar(1.0);
        obj.setsinglebond(mtg_adapter::binding_single_from(SingleRates{0.7, 0.5}));
        obj.initialize(x, p, Q, L);
        const int np = 4 * n;
        std::vector<bool> ib(np, false);
        std::vector<int> bt(np, 0);
        obj.setbindings(ib, bt);
        obj.calculate_forces_and_torques3D_onlyone_nonlets(F, T);   // draw 0
        std::vector<bool> ib1(np);
        std::vector<int> bt1(np);
        obj.getbindings(ib1, bt1);
        obj.init_forces();                                          // draw 1
        for (int i = 0; i < steps; i++) obj.step(1);                // draws 2, 3, ...
        obj.getdat(x);
        obj.getorientation(Q);
        std::vector<bool> ib2(np);
        std::vector<int> bt2(np);
        obj.getbindings(ib2, bt2);
        std::FILE *o = std::fopen(argv[2], "wb");
        for (Mat *m : {&F, &T}) std::fwrite(m->v.data(), sizeof(double), m->v.size(), o);
        for (const std::vector<bool> *b : {&ib1, &ib2}) {
            std::vector<uint8_t> u(b->begin(), b->end());
            std::fwrite(u.data(), 1, u.size(), o);
        }
        for (const std::vector<int> *b : {&bt1, &bt2}) std::fwrite(b->data(), sizeof(int), b->size(), o);
        for (Mat *m : {&x, &Q}) std::fwrite(m->v.data(), sizeof(double), m->v.size(), o);
        std::fclose(o);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
