/*
 * oracle.c -- CPU restatement (FP64) of the mtcode rotational-Langevin step.  TEST INFRASTRUCTURE:
 * the checker for the CUDA path, never part of it (see oracle.h).
 *
 * Each routine cites the reference function it restates.  The arithmetic keeps the reference's
 * operation order and precision (including the long-double angular factors that come from
 * `pi` being a long double, Basic/basic.h:31) so that, compiled with -ffp-contract=off, the results
 * agree bit for bit with the reference's own routines on x86-64 (checked against the reference
 * build in oracle/_ref by tests/test_oracle_golden.py).
 *
 * Build:  gcc -O2 -std=c11 -ffp-contract=off -fPIC -shared oracle.c -lm -o liboracle.so
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Basic/basic.h:31 declares `const long double pi` but initialises it from a DOUBLE literal, so its
 * value is pi rounded to double, carried in long double arithmetic.  The oracle does the same. */
static const long double ORC_PI_L = (long double)3.1415926535897932384626433832795028841971693993751;

#define SQR(x) ((x) * (x))

/* SIGN(a,b) of Basic/basic.h:54 */
static inline double orc_sign(double a, double b) { return b >= 0 ? fabs(a) : -fabs(a); }

/* fasterfloor, Basic/basic.h:58 */
static inline int orc_fasterfloor(double x) { return x > 0 ? (int)x : (int)x - 1; }

/* ---------------------------------------------------------------- cell list */

int orc_assign_box(const double *xrow, int n, double box)
{
    int c = 0, stride = 1;
    for (int k = 0; k < 3; k++) {
        int m = orc_fasterfloor(n * xrow[k] / box);
        if (m < 0) m = 0;
        else if (m > n - 1) m = n - 1;
        c += m * stride;
        stride *= n;
    }
    return c;
}

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

int orc_neighbor_cells(int c, int n, int *out)
{
    int ix = c % n, iy = (c / n) % n, iz = c / (n * n);
    int tmp[27];
    int k = 0;
    for (int t = 0; t < 27; t++) {
        int d[3] = {t % 3 - 1, (t / 3) % 3 - 1, (t / 9) % 3 - 1};
        int cc[3] = {ix + d[0], iy + d[1], iz + d[2]};
        for (int a = 0; a < 3; a++) {
            if (cc[a] < 0) cc[a] += n;
            else if (cc[a] > n - 1) cc[a] -= n;
        }
        tmp[k++] = cc[0] + n * cc[1] + n * n * cc[2];
    }
    qsort(tmp, 27, sizeof(int), cmp_int);
    int m = 0;
    for (int i = 0; i < 27; i++)
        if (m == 0 || tmp[i] != out[m - 1]) out[m++] = tmp[i];
    return m;
}

/* cube::distance_less_than, geometry.h:145-162 */
static int orc_distance_less_than(const orc_params *P, const double *x, int i, int j, double val)
{
    double temp = 0.0;
    for (int k = 0; k < 3; k++) {
        double dx = x[3 * i + k] - x[3 * j + k];
        if (P->periodic) {
            if (fabs(dx) > P->box * 0.5) dx = dx - orc_sign(P->box, dx);
        }
        dx = SQR(dx);
        if (dx > SQR(val)) return 0;
        temp += dx;
    }
    return temp < SQR(val);
}

/* cube::distance_vector, geometry.h:277-294: un = x_i - x_j (minimum image), returns |un|^2 */
static double orc_distance_vector(const orc_params *P, const double *x, int i, int j, double un[3])
{
    double temp = 0.0;
    double l2s = SQR(P->box / 2.);
    for (int k = 0; k < 3; k++) {
        double as = x[3 * i + k] - x[3 * j + k];
        if (P->periodic) {
            if (SQR(as) > l2s) as = as - orc_sign(P->box, as);
        }
        temp += SQR(as);
        un[k] = as;
    }
    return temp;
}

long orc_pairs(const orc_params *P, const double *x, int ncell, double rc, int *pairs, long cap)
{
    int n = ncell;
    int total = n * n * n;
    int N = P->n;
    /* members of each cell in increasing particle order (MD.cpp:1078-1083) */
    int *count = (int *)calloc((size_t)total + 1, sizeof(int));
    int *start = (int *)calloc((size_t)total + 1, sizeof(int));
    int *cellof = (int *)malloc(sizeof(int) * (size_t)(N > 0 ? N : 1));
    int *members = (int *)malloc(sizeof(int) * (size_t)(N > 0 ? N : 1));
    for (int i = 0; i < N; i++) {
        cellof[i] = orc_assign_box(x + 3 * i, n, P->box);
        count[cellof[i]]++;
    }
    for (int c = 0; c < total; c++) start[c + 1] = start[c] + count[c];
    memset(count, 0, sizeof(int) * (size_t)total);
    for (int i = 0; i < N; i++) members[start[cellof[i]] + count[cellof[i]]++] = i;

    long np = 0;
    int nb[27];
    for (int c1 = 0; c1 < total; c1++) {
        int m = orc_neighbor_cells(c1, n, nb);
        for (int s = 0; s < m; s++) {
            int c2 = nb[s];
            int b1s = start[c1 + 1] - start[c1];
            int b2s = start[c2 + 1] - start[c2];
            if (c1 == c2) {
                for (int a = 0; a < b1s; a++)
                    for (int b = a + 1; b < b2s; b++) {
                        int i = members[start[c1] + a], j = members[start[c2] + b];
                        if (orc_distance_less_than(P, x, i, j, rc)) {
                            if (np < cap) { pairs[2 * np] = i; pairs[2 * np + 1] = j; }
                            np++;
                        }
                    }
            } else if (c2 > c1) {
                for (int a = 0; a < b1s; a++)
                    for (int b = 0; b < b2s; b++) {
                        int i = members[start[c1] + a], j = members[start[c2] + b];
                        if (orc_distance_less_than(P, x, i, j, rc)) {
                            if (np < cap) { pairs[2 * np] = i; pairs[2 * np + 1] = j; }
                            np++;
                        }
                    }
            }
        }
    }
    free(count); free(start); free(cellof); free(members);
    return np;
}

/* ---------------------------------------------------------------- central (WCA core) force */

/* HSPotential::force, potential.h:106-118 */
static double orc_hs_force(double eps, double sigma, double r)
{
    double paramlimit = 1.12246 * sigma;
    if (r < paramlimit) {
        double sigma6 = SQR(sigma * sigma * sigma);
        double sigma12 = SQR(sigma6);
        double a = r * r * r;
        a = SQR(a);
        return 4 * eps * (12 * sigma12 / (r * SQR(a)) - 6 * sigma6 / (r * a));
    }
    return 0;
}

void orc_hs_forces(const orc_params *P, const double *x, const int *pairs, long np, double *F)
{
    memset(F, 0, sizeof(double) * 3 * (size_t)P->n);
    for (long q = 0; q < np; q++) {
        int p1 = pairs[2 * q], p2 = pairs[2 * q + 1];
        double un[3];
        double dis = orc_distance_vector(P, x, p1, p2, un);
        double f1 = orc_hs_force(P->hs_eps, P->hs_sigma, sqrt(dis));
        for (int j = 0; j < 3; j++) {
            double fac = f1 * un[j] / sqrt(dis);
            F[3 * p1 + j] += fac;
            F[3 * p2 + j] += -fac;
        }
    }
}

void orc_bond_forces(const orc_params *P, const double *x, const int *bonds, long nb, double k, double r0, double *F)
{
    memset(F, 0, sizeof(double) * 3 * (size_t)P->n);
    for (long q = 0; q < nb; q++) {
        int p1 = bonds[2 * q], p2 = bonds[2 * q + 1];
        double un[3];
        double dis = orc_distance_vector(P, x, p1, p2, un);
        double f1 = -k * (sqrt(dis) - r0);
        for (int j = 0; j < 3; j++) {
            double fac = f1 * un[j] / sqrt(dis);
            F[3 * p1 + j] += fac;
            F[3 * p2 + j] += -fac;
        }
    }
}

void orc_central_forces(const orc_params *P, const double *x, const int *pairs, long np, double *F)
{
    if (P->nbonds <= 0 || !P->bonds) {
        orc_hs_forces(P, x, pairs, np, F);
        return;
    }
    double *F2 = (double *)malloc(sizeof(double) * 3 * (size_t)(P->n > 0 ? P->n : 1));
    orc_bond_forces(P, x, P->bonds, P->nbonds, P->bond_k, P->bond_r0, F);
    orc_hs_forces(P, x, pairs, np, F2);
    for (size_t i = 0; i < 3 * (size_t)P->n; i++) F[i] += F2[i];
    free(F2);
}

/* ---------------------------------------------------------------- patch force (KernFrenkelOnePatch2) */

void orc_kf2_force_torque(const double nb1[3], const double nb2[3], double att, double dis, double thetam,
                          const double un[3], double rij, const double *q, const double *g, double o[9])
{
    for (int k = 0; k < 9; k++) o[k] = 0.0;
    if (rij > 1.4 * dis) return; /* interaction_distance, potentialtheta.h:416 */

    double nx1 = nb1[0] * q[0] + nb1[1] * q[3] + nb1[2] * q[6];
    double ny1 = nb1[0] * q[1] + nb1[1] * q[4] + nb1[2] * q[7];
    double nz1 = nb1[0] * q[2] + nb1[1] * q[5] + nb1[2] * q[8];
    double nx2 = nb2[0] * g[0] + nb2[1] * g[3] + nb2[2] * g[6];
    double ny2 = nb2[0] * g[1] + nb2[1] * g[4] + nb2[2] * g[7];
    double nz2 = nb2[0] * g[2] + nb2[1] * g[5] + nb2[2] * g[8];

    double ci = -(nx1 * un[0] + ny1 * un[1] + nz1 * un[2]);
    double cj = (nx2 * un[0] + ny2 * un[1] + nz2 * un[2]);
    if (!(ci > cos(thetam) && cj > cos(thetam))) return;
    if (ci > 1.) ci = 0.999999;
    if (cj > 1.) cj = 0.999999;

    double thi = acos(ci), thj = acos(cj);
    long double ai = ORC_PI_L * thi / (2. * thetam);
    long double aj = ORC_PI_L * thj / (2. * thetam);
    long double k = ORC_PI_L / (2. * thetam);
    double f = (double)(cosl(ai) * cosl(aj));

    double fac = rij / dis;
    double fac2 = SQR(fac), fac4 = SQR(fac2), fac8 = SQR(fac4), fac10 = fac2 * fac8;
    double ex = exp(-0.5 * fac10);
    double pot = -att * ex;
    double potf = -5. * att * fac8 * (fac / dis) * ex;

    double fx = f * potf * un[0];
    double fy = f * potf * un[1];
    double fz = f * potf * un[2];

    double d1 = (fabs(SQR(ci) - 1) < 1E-5) ? 0.0 : -1. / sqrt(1 - SQR(ci));
    double d2 = (fabs(SQR(cj) - 1) < 1E-5) ? 0.0 : -1. / sqrt(1 - SQR(cj));

    double t1 = (double)(-pot * (k * sinl(ai) * d1 * cosl(aj)));
    double t2 = (double)(-pot * (k * sinl(aj) * d2 * cosl(ai)));

    fx += (t1 / rij) * (nx1 + ci * un[0]);
    fy += (t1 / rij) * (ny1 + ci * un[1]);
    fz += (t1 / rij) * (nz1 + ci * un[2]);
    fx += -(t2 / rij) * (nx2 - cj * un[0]);
    fy += -(t2 / rij) * (ny2 - cj * un[1]);
    fz += -(t2 / rij) * (nz2 - cj * un[2]);

    long double gi = -k * pot * sinl(ai) * d1 * cosl(aj);
    long double gj = -k * pot * sinl(aj) * d2 * cosl(ai);
    o[0] = fx; o[1] = fy; o[2] = fz;
    o[3] = (double)(gi * (un[2] * ny1 - un[1] * nz1));
    o[4] = (double)(gi * (-un[2] * nx1 + un[0] * nz1));
    o[5] = (double)(gi * (un[1] * nx1 - un[0] * ny1));
    o[6] = (double)(gj * (-un[2] * ny2 + un[1] * nz2));
    o[7] = (double)(gj * (un[2] * nx2 - un[0] * nz2));
    o[8] = (double)(gj * (-un[1] * nx2 + un[0] * ny2));
}

static int orc_type_of(const orc_model *M, int i)
{
    for (int k = 0; k < M->n_types; k++)
        if (i < M->num_per_type[k]) return k;
    return M->n_types - 1;
}

/* first potential index of type pair (k1 <= k2), GeneralPatch.cpp:43-61 enumeration */
static int orc_pot_start(const orc_model *M, int k1, int k2)
{
    int s = 0;
    for (int a = 0; a < M->n_types; a++)
        for (int b = a; b < M->n_types; b++) {
            if (a == k1 && b == k2) return s;
            s += M->patches_per_type[a] * M->patches_per_type[b];
        }
    return s;
}

static int orc_orient_start(const orc_model *M, int k)
{
    int s = 0;
    for (int a = 0; a < k; a++) s += M->patches_per_type[a];
    return s;
}

void orc_patch_forces(const orc_params *P, const double *x, const double *Q, const int *pairs, long np,
                      double *F, double *T)
{
    const orc_model *M = P->model;
    for (long q = 0; q < np; q++) {
        int p1 = pairs[2 * q], p2 = pairs[2 * q + 1];
        if (p2 < p1) { int t = p1; p1 = p2; p2 = t; }
        double un[3];
        double dis = orc_distance_vector(P, x, p1, p2, un);
        if (!(dis < P->max_dist2)) continue;
        dis = sqrt(dis);
        un[0] /= dis; un[1] /= dis; un[2] /= dis;
        int k1 = orc_type_of(M, p1), k2 = orc_type_of(M, p2);
        int n1 = M->patches_per_type[k1], n2 = M->patches_per_type[k2];
        int ps = orc_pot_start(M, k1, k2);
        int o1 = orc_orient_start(M, k1), o2 = orc_orient_start(M, k2);
        for (int a = 0; a < n1; a++)
            for (int b = 0; b < n2; b++) {
                int potn = ps + a * n2 + b;
                double o[9];
                orc_kf2_force_torque(M->orient[o1 + a], M->orient[o2 + b], M->att[potn], M->dis[potn],
                                     M->thetam[potn], un, dis, Q + 9 * p1, Q + 9 * p2, o);
                F[3 * p1 + 0] += o[0]; F[3 * p1 + 1] += o[1]; F[3 * p1 + 2] += o[2];
                F[3 * p2 + 0] += -o[0]; F[3 * p2 + 1] += -o[1]; F[3 * p2 + 2] += -o[2];
                T[3 * p1 + 0] += o[3]; T[3 * p1 + 1] += o[4]; T[3 * p1 + 2] += o[5];
                T[3 * p2 + 0] += o[6]; T[3 * p2 + 1] += o[7]; T[3 * p2 + 2] += o[8];
            }
    }
}

/* ---------------------------------------------------------------- integrator */

void orc_langevin_forces(const orc_params *P, const double *p, const double *Lb, const double *Q,
                         const double *noise, double *F, double *T)
{
    double Rt = sqrt(2 * P->gamma * P->kT / P->dt);
    double Rr = sqrt(2 * P->gammar * P->kT / P->dt);
    double m = P->mass, I = P->inertia;
    for (int i = 0; i < P->n; i++) {
        const double *q = Q + 9 * i;
        double plx = p[3 * i], ply = p[3 * i + 1], plz = p[3 * i + 2];
        double llx = Lb[3 * i], lly = Lb[3 * i + 1], llz = Lb[3 * i + 2];
        double pbx = q[0] * plx + q[1] * ply + q[2] * plz;
        double pby = q[3] * plx + q[4] * ply + q[5] * plz;
        double pbz = q[6] * plx + q[7] * ply + q[8] * plz;
        double ffx = (-P->gamma / m) * pbx, ffy = (-P->gamma / m) * pby, ffz = (-P->gamma / m) * pbz;
        double tfx = (-P->gammar / I) * llx, tfy = (-P->gammar / I) * lly, tfz = (-P->gammar / I) * llz;
        const double *r = noise ? noise + 6 * (size_t)i : NULL;
        double frx = Rt * (r ? r[0] : 0.0), fry = Rt * (r ? r[1] : 0.0), frz = Rt * (r ? r[2] : 0.0);
        double trx = Rr * (r ? r[3] : 0.0), try_ = Rr * (r ? r[4] : 0.0), trz = Rr * (r ? r[5] : 0.0);
        double *f = F + 3 * i, *t = T + 3 * i;
        double fx = f[0] + (ffx + frx) * q[0] + (ffy + fry) * q[3] + (ffz + frz) * q[6];
        double fy = f[1] + (ffx + frx) * q[1] + (ffy + fry) * q[4] + (ffz + frz) * q[7];
        double fz = f[2] + (ffx + frx) * q[2] + (ffy + fry) * q[5] + (ffz + frz) * q[8];
        double tbx = tfx + trx + t[0] * q[0] + t[1] * q[1] + t[2] * q[2];
        double tby = tfy + try_ + t[0] * q[3] + t[1] * q[4] + t[2] * q[5];
        double tbz = tfz + trz + t[0] * q[6] + t[1] * q[7] + t[2] * q[8];
        f[0] = fx; f[1] = fy; f[2] = fz;
        t[0] = tbx; t[1] = tby; t[2] = tbz;
    }
}

void orc_halfkick(int n, double dt, double *p, double *Lb, const double *F, const double *T)
{
    for (int i = 0; i < 3 * n; i++) {
        p[i] += (dt / 2.) * F[i];
        Lb[i] += (dt / 2.) * T[i];
    }
}

void orc_drift(const orc_params *P, double *x, double *p)
{
    double c1 = P->dt / P->mass, l = P->box;
    for (int i = 0; i < 3 * P->n; i++) x[i] = x[i] + c1 * p[i];
    for (int i = 0; i < 3 * P->n; i++) {
        if (P->periodic) {
            double temp = x[i];
            if (temp < 0) {
                while (temp < 0) temp += l;
                x[i] = temp;
            } else if (temp > l) {
                while (temp > l) temp -= l;
                x[i] = temp;
            }
        } else {
            if (x[i] < 0) { x[i] = -x[i]; p[i] = -p[i]; }
            else if (x[i] > l) { x[i] = l - (x[i] - l); p[i] = -p[i]; }
        }
    }
}

void orc_rotation_matrix(double dt, double I, const double L[3], double up[9])
{
    double tx = dt * L[0] / I, ty = dt * L[1] / I, tz = dt * L[2] / I;
    double a1 = (1 - SQR(tx / 4.)) / (1 + SQR(tx / 4.));
    double a2 = tx / (2. * (1 + SQR(tx / 4.)));
    double a3 = (1 - SQR(ty / 4.)) / (1 + SQR(ty / 4.));
    double a4 = ty / (2. * (1 + SQR(ty / 4.)));
    double a5 = (1 - SQR(tz / 2.)) / (1 + SQR(tz / 2.));
    double a6 = tz / (1 + SQR(tz / 2.));
    up[0] = -SQR(a4) + SQR(a3) * a5;
    up[1] = a3 * (a2 * a4 * (1 + a5) - a1 * a6);
    up[2] = a3 * (a1 * a4 * (1 + a5) + a2 * a6);
    up[3] = a3 * (a2 * a4 * (1 + a5) + a1 * a6);
    up[4] = SQR(a1) * a5 + SQR(a2) * (-SQR(a3) + SQR(a4) * a5);
    up[5] = -(a1 * a2 * (SQR(a3) + a5 - SQR(a4) * a5)) + (SQR(a1) + SQR(a2)) * a4 * a6;
    up[6] = -(a1 * a3 * a4 * (1 + a5)) + a2 * a3 * a6;
    up[7] = a1 * a2 * (SQR(a3) + a5 - SQR(a4) * a5) + (SQR(a1) + SQR(a2)) * a4 * a6;
    up[8] = -(SQR(a2) * a5) + SQR(a1) * (SQR(a3) - SQR(a4) * a5);
}

void orc_rotate(const orc_params *P, double *Lb, double *Q)
{
    for (int i = 0; i < P->n; i++) {
        double *L = Lb + 3 * i, *q = Q + 9 * i, R[9], nq[9];
        orc_rotation_matrix(P->dt, P->inertia, L, R);
        double j0 = L[0] * R[0] + L[1] * R[1] + L[2] * R[2];
        double j1 = L[0] * R[3] + L[1] * R[4] + L[2] * R[5];
        double j2 = L[0] * R[6] + L[1] * R[7] + L[2] * R[8];
        /* Q <- R^T Q */
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                nq[3 * a + b] = q[b] * R[a] + q[3 + b] * R[3 + a] + q[6 + b] * R[6 + a];
        L[0] = j0; L[1] = j1; L[2] = j2;
        memcpy(q, nq, sizeof(nq));
    }
}

void orc_temperature(const orc_params *P, const double *p, const double *Lb, double out[6])
{
    double mom[3] = {0, 0, 0}, ang[3] = {0, 0, 0};
    for (int i = 0; i < P->n; i++)
        for (int k = 0; k < 3; k++) {
            mom[k] += (p[3 * i + k] * p[3 * i + k]) / (2. * P->mass);
            ang[k] += (Lb[3 * i + k] * Lb[3 * i + k]) / (2. * P->inertia);
        }
    for (int k = 0; k < 3; k++) {
        out[k] = mom[k] / (double)P->n;
        out[3 + k] = ang[k] / (double)P->n;
    }
}

/* ---------------------------------------------------------------- Philox4x32-10 */

static inline void orc_mulhilo(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo)
{
    uint64_t prod = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(prod >> 32);
    *lo = (uint32_t)prod;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        orc_mulhilo(0xD2511F53u, c0, &hi0, &lo0);
        orc_mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_philox_noise(int n, uint64_t seed, uint32_t replica, uint64_t draw, double *noise)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int i = 0; i < n; i++) {
        uint32_t w[8];
        for (int blk = 0; blk < 2; blk++) {
            uint32_t ctr[4] = {(uint32_t)i, (uint32_t)draw, (uint32_t)(draw >> 32), 2u * replica + (uint32_t)blk};
            orc_philox4x32_10(ctr, key, w + 4 * blk);
        }
        for (int k = 0; k < 6; k++) {
            double u = (double)(w[k] >> 8) * (1.0 / 16777216.0);
            noise[6 * (size_t)i + k] = 3.464101615 * u - 1.732050808;
        }
    }
}

/* ---------------------------------------------------------------- observables */

void orc_observables(const orc_params *P, const double *x, const double *Q, const int *pairs, long np,
                     double out[4])
{
    const orc_model *M = P->model;
    double maxcheck = 1.0; /* ComboPatch max_check starts at 1.0 (combopatch.h:15) */
    for (int q = 0; q < M->n_pots; q++)
        if (1.4 * M->dis[q] > maxcheck) maxcheck = 1.4 * M->dis[q];
    double upatch = 0, uwca = 0, vir = 0, bonds = 0;
    double eps = P->hs_eps, sigma = P->hs_sigma;
    for (long q = 0; q < np; q++) {
        int p1 = pairs[2 * q], p2 = pairs[2 * q + 1];
        if (p2 < p1) { int t = p1; p1 = p2; p2 = t; }
        double un[3];
        double d2 = orc_distance_vector(P, x, p1, p2, un);
        double r = sqrt(d2);
        double f[3] = {0, 0, 0};
        double fh = orc_hs_force(eps, sigma, r);
        if (r < 1.12246 * sigma) {
            double s6 = pow(sigma / r, 6);
            uwca += 4 * eps * (s6 * s6 - s6) + eps;
        }
        for (int k = 0; k < 3; k++) f[k] += fh * un[k] / r;
        double u[3] = {un[0] / r, un[1] / r, un[2] / r};
        int k1 = orc_type_of(M, p1), k2 = orc_type_of(M, p2);
        int n1 = M->patches_per_type[k1], n2 = M->patches_per_type[k2];
        int ps = orc_pot_start(M, k1, k2);
        int o1 = orc_orient_start(M, k1), o2 = orc_orient_start(M, k2);
        const double *qi = Q + 9 * p1, *qj = Q + 9 * p2;
        for (int a = 0; a < n1; a++)
            for (int b = 0; b < n2; b++) {
                int potn = ps + a * n2 + b;
                const double *nb1 = M->orient[o1 + a], *nb2 = M->orient[o2 + b];
                double nx1 = nb1[0] * qi[0] + nb1[1] * qi[3] + nb1[2] * qi[6];
                double ny1 = nb1[0] * qi[1] + nb1[1] * qi[4] + nb1[2] * qi[7];
                double nz1 = nb1[0] * qi[2] + nb1[1] * qi[5] + nb1[2] * qi[8];
                double nx2 = nb2[0] * qj[0] + nb2[1] * qj[3] + nb2[2] * qj[6];
                double ny2 = nb2[0] * qj[1] + nb2[1] * qj[4] + nb2[2] * qj[7];
                double nz2 = nb2[0] * qj[2] + nb2[1] * qj[5] + nb2[2] * qj[8];
                double ci = -(nx1 * u[0] + ny1 * u[1] + nz1 * u[2]);
                double cj = nx2 * u[0] + ny2 * u[1] + nz2 * u[2];
                int incone = ci > cos(M->thetam[potn]) && cj > cos(M->thetam[potn]);
                if (r < maxcheck && incone) bonds += 1;
                if (d2 < P->max_dist2) {
                    if (r <= 1.4 * M->dis[potn] && incone) {
                        double cci = ci > 1. ? 0.999999 : ci, ccj = cj > 1. ? 0.999999 : cj;
                        long double ai = ORC_PI_L * acos(cci) / (2. * M->thetam[potn]);
                        long double aj = ORC_PI_L * acos(ccj) / (2. * M->thetam[potn]);
                        double fac = r / M->dis[potn];
                        double fac10 = pow(fac, 10);
                        upatch += -M->att[potn] * exp(-0.5 * fac10) * (double)(cosl(ai) * cosl(aj));
                    }
                    double o[9];
                    orc_kf2_force_torque(nb1, nb2, M->att[potn], M->dis[potn], M->thetam[potn], u, r, qi, qj, o);
                    f[0] += o[0]; f[1] += o[1]; f[2] += o[2];
                }
            }
        vir += un[0] * f[0] + un[1] * f[1] + un[2] * f[2];
    }
    out[0] = upatch; out[1] = uwca; out[2] = vir; out[3] = bonds;
}

/* ---------------------------------------------------------------- drivers */

static long orc_pairs_alloc(const orc_params *P, const double *x, int ncell, double rc, int **out)
{
    long cap = 16L * (P->n > 0 ? P->n : 1) + 64;
    int *pairs = (int *)malloc(sizeof(int) * 2 * (size_t)cap);
    long np = orc_pairs(P, x, ncell, rc, pairs, cap);
    if (np > cap) {
        free(pairs);
        cap = np;
        pairs = (int *)malloc(sizeof(int) * 2 * (size_t)cap);
        np = orc_pairs(P, x, ncell, rc, pairs, cap);
    }
    *out = pairs;
    return np;
}

/* cube::distance (geometry.h:107-121) */
static double orc_distance(const orc_params *P, const double *x, int i, int j)
{
    double temp = 0.0;
    for (int k = 0; k < 3; k++) {
        double dx = x[3 * i + k] - x[3 * j + k];
        if (P->periodic && fabs(dx) > P->box * 0.5) dx = dx - (dx >= 0.0 ? P->box : -P->box);
        temp += dx * dx;
    }
    return sqrt(temp);
}

int orc_gr(const orc_params *P, const double *x, double max, double dx, long *hist, int cap)
{
    int gs = (int)floor(max / dx);
    for (int b = 0; b < gs && b < cap; b++) hist[b] = 0;
    /* every unordered pair once; only distances below gs * dx <= max land in a bin */
    for (int i = 0; i < P->n; i++)
        for (int j = i + 1; j < P->n; j++) {
            int in = (int)floor(orc_distance(P, x, i, j) / dx);
            if (in < gs && in < cap) hist[in] += 1;
        }
    return gs;
}

static int orc_find(int *parent, int a)
{
    while (parent[a] != a) a = parent[a];
    return a;
}

void orc_clusters(const orc_params *P, const double *x, double cut, int *labels)
{
    int *pairs;
    int ncell = (int)floor(P->box / cut);
    if (ncell < 1) ncell = 1;
    long np = orc_pairs_alloc(P, x, ncell, cut, &pairs);
    for (int i = 0; i < P->n; i++) labels[i] = i;
    for (long q = 0; q < np; q++) {  /* union by smaller root: a component's root is its smallest index */
        int a = orc_find(labels, pairs[2 * q]), b = orc_find(labels, pairs[2 * q + 1]);
        if (a < b) labels[b] = a;
        else if (b < a) labels[a] = b;
    }
    for (int i = 0; i < P->n; i++) labels[i] = orc_find(labels, i);
    free(pairs);
}

void orc_forces(const orc_params *P, const double *x, const double *Q, int ncell, double rc, double *F, double *T)
{
    int *pairs;
    long np = orc_pairs_alloc(P, x, ncell, rc, &pairs);
    orc_central_forces(P, x, pairs, np, F);
    memset(T, 0, sizeof(double) * 3 * (size_t)P->n);
    orc_patch_forces(P, x, Q, pairs, np, F, T);
    free(pairs);
}

void orc_init_forces(const orc_params *P, const double *x, const double *p, const double *Lb, const double *Q,
                     int ncell, double rc, const double *noise, double *Ft, double *Tt)
{
    orc_forces(P, x, Q, ncell, rc, Ft, Tt);
    orc_langevin_forces(P, p, Lb, Q, noise, Ft, Tt);
}

/* number of pairs within the force range, from a fresh cell list */
static long orc_count_in_range(const orc_params *P, const double *x, const int *pairs, long np, double r2)
{
    long c = 0;
    for (long q = 0; q < np; q++) {
        double un[3];
        if (orc_distance_vector(P, x, pairs[2 * q], pairs[2 * q + 1], un) < r2) c++;
    }
    return c;
}

int orc_run(const orc_params *P, double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt,
            int nsteps, int ncell, double rc, int rebuild, int noise_mode, const double *noise,
            uint64_t seed, uint32_t replica, uint64_t draw0, int check_skin)
{
    int n = P->n;
    int status = 0;
    int *pairs = NULL;
    long np = 0;
    double *xi = (double *)calloc(6 * (size_t)(n > 0 ? n : 1), sizeof(double));
    double hs = 1.12246 * P->hs_sigma;
    double frange2 = P->max_dist2 > hs * hs ? P->max_dist2 : hs * hs;
    int nfresh = ncell;
    for (int s = 0; s < nsteps; s++) {
        if (rebuild <= 1 || s % rebuild == 0) {
            free(pairs);
            np = orc_pairs_alloc(P, x, ncell, rc, &pairs);
        }
        orc_halfkick(n, P->dt, p, Lb, Ft, Tt);
        orc_drift(P, x, p);
        orc_rotate(P, Lb, Q);
        orc_central_forces(P, x, pairs, np, Ft);
        memset(Tt, 0, sizeof(double) * 3 * (size_t)n);
        orc_patch_forces(P, x, Q, pairs, np, Ft, Tt);
        if (check_skin) {   /* every pair within the force range must be in the list */
            int *fresh;
            long nf = orc_pairs_alloc(P, x, nfresh, rc, &fresh);
            if (orc_count_in_range(P, x, fresh, nf, frange2) != orc_count_in_range(P, x, pairs, np, frange2))
                status = -1;
            free(fresh);
        }
        const double *nz = NULL;
        if (noise_mode == 1) nz = noise + 6 * (size_t)n * (size_t)s;
        else if (noise_mode == 2) { orc_philox_noise(n, seed, replica, draw0 + (uint64_t)s, xi); nz = xi; }
        else nz = xi;
        orc_langevin_forces(P, p, Lb, Q, nz, Ft, Tt);
        orc_halfkick(n, P->dt, p, Lb, Ft, Tt);
    }
    free(pairs);
    free(xi);
    return status;
}
