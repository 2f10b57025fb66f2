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

/* ================================================================ single-bond-per-patch mode
 * Condensate::run_singlebond (Condensate/Condensate.cpp:422-618): every patch holds at most one bond,
 * decided each step by LangevinNVTR::calculate_forces_and_torques3D_onlyone_nonlets
 * (MDBase/Rotational/LangevinRforce.cpp:2874-3500) from a candidate patch-pair list
 * (LangevinNVTR::calculate_patch_list, LangevinR.cpp:1702-1852) and a binding model
 * (MDBase/Bindings/BindingModel{Single,Binary,Ternary}). */

/* ComboPatch::max_check: 1 (combopatch.h:15) raised to every potential's interaction_distance = 1.4 dis
 * (potentialtheta.h:416; GeneralPatch.cpp:97, TetrahedralPatch.cpp:42) */
double orc_max_check(const orc_model *M)
{
    double mc = 1.0;
    for (int q = 0; q < M->n_pots; q++)
        if (1.4 * M->dis[q] > mc) mc = 1.4 * M->dis[q];
    return mc;
}

/* first patch index of type k (GeneralPatch total_patches_per_type, GeneralPatch.cpp:285-295) */
static int orc_patch_base(const orc_model *M, int k)
{
    int s = 0;
    for (int a = 0; a < k; a++) s += M->patches_per_type[a] * (M->num_per_type[a] - (a ? M->num_per_type[a - 1] : 0));
    return s;
}

int orc_total_patches(const orc_model *M, int n)
{
    (void)n;
    return orc_patch_base(M, M->n_types);
}

/* GeneralPatch::which_patch (GeneralPatch.cpp:297-320) for particle i, type k, patch c */
static int orc_patch_index(const orc_model *M, int i, int k, int c)
{
    return orc_patch_base(M, k) + (i - (k ? M->num_per_type[k - 1] : 0)) * M->patches_per_type[k] + c;
}

/* GeneralPatch::which_particle (GeneralPatch.cpp:431-448): particle and its patch number of patch wp */
static void orc_patch_owner(const orc_model *M, int wp, int *particle, int *type, int *patch)
{
    for (int k = 0; k < M->n_types; k++) {
        int b0 = orc_patch_base(M, k), b1 = orc_patch_base(M, k + 1);
        if (wp >= b0 && wp < b1) {
            *type = k;
            *particle = (k ? M->num_per_type[k - 1] : 0) + (wp - b0) / M->patches_per_type[k];
            *patch = (wp - b0) % M->patches_per_type[k];
            return;
        }
    }
    *type = -1; *particle = -1; *patch = -1;
}

/* lab-frame patch vector Q^T n_b in the reference's operation order (LangevinRforce.cpp:2980-2985) */
static void orc_lab_patch(const double nb[3], const double *q, double n[3])
{
    n[0] = nb[0] * q[0] + nb[1] * q[3] + nb[2] * q[6];
    n[1] = nb[0] * q[1] + nb[1] * q[4] + nb[2] * q[7];
    n[2] = nb[0] * q[2] + nb[1] * q[5] + nb[2] * q[8];
}

long orc_patch_list(const orc_params *P, const double *x, const double *Q, const int *pairs, long np,
                    double max_ang, orc_patchint *out, long cap)
{
    const orc_model *M = P->model;
    double max_dis = orc_max_check(M) + 1.;
    long cnt = 0;
    for (long q = 0; q < np; q++) {
        int p1 = pairs[2 * q], p2 = pairs[2 * q + 1];
        if (p2 < p1) { int t = p1; p1 = p2; p2 = t; }
        double un[3];
        double dis = sqrt(orc_distance_vector(P, x, p1, p2, un));
        if (!(dis < max_dis)) continue;
        un[0] /= dis; un[1] /= dis; un[2] /= dis;
        int k1 = orc_type_of(M, p1), k2 = orc_type_of(M, p2);
        int n1 = M->patches_per_type[k1], n2 = M->patches_per_type[k2];
        int ps = orc_pot_start(M, k1, k2), o1 = orc_orient_start(M, k1), o2 = orc_orient_start(M, k2);
        for (int a = 0; a < n1; a++)
            for (int b = 0; b < n2; b++) {
                double m1[3], m2[3];
                orc_lab_patch(M->orient[o1 + a], Q + 9 * p1, m1);
                orc_lab_patch(M->orient[o2 + b], Q + 9 * p2, m2);
                double ai = -(m1[0] * un[0] + m1[1] * un[1] + m1[2] * un[2]);
                double aj = (m2[0] * un[0] + m2[1] * un[1] + m2[2] * un[2]);
                if ((ai - max_ang) + (aj - max_ang) > -0.4) {
                    if (cnt < cap) {
                        orc_patchint *e = out + cnt;
                        e->p1 = p1; e->p2 = p2; e->potn = ps + a * n2 + b;
                        e->wp1 = orc_patch_index(M, p1, k1, a);
                        e->wp2 = orc_patch_index(M, p2, k2, b);
                    }
                    cnt++;
                }
            }
    }
    return cnt;
}

/* species of a patch index: SortingFunctionUniform / SortingFunctionNonUniform
 * (Bindings/BindingModelTernary.h:6-30); BindingModelBinary's `index < div` (BindingModelBinary.cpp);
 * a single species for BindingModelSingle */
static int orc_species(const orc_binding *B, int idx)
{
    switch (B->rule) {
    case 1: return idx < B->div1 ? 1 : 2;
    case 2: return idx < B->div1 ? 1 : (idx < B->div2 ? 2 : 3);
    case 3:
        if (idx < B->div1) return 1;
        if (idx < B->div2) return 2;
        return ((idx - B->div2) % B->np == B->np - 1) ? 3 : 1;
    default: return 1;
    }
}

/* table rows: species pairs 11, 12, 13, 22, 23, 33 and sorted triples 111 ... 333 in lexicographic order
 * (get_drate / get_trate, BindingModelTernary.cpp:489-520, 652-700) */
static int orc_pair_row(int a, int b) { return a == 1 ? b - 1 : (a == 2 ? b + 1 : 5); }
static int orc_triple_row(int a, int b, int c)
{
    static const int base[4] = {0, 0, 6, 9};   /* rows starting with species a */
    if (a == 1) return b == 1 ? c - 1 : (b == 2 ? c + 1 : 5);
    if (a == 2) return base[2] + (b == 2 ? c - 2 : 2);
    return base[3];
}

/* AbstractBindingModel::doublet (BindingModelTernary.cpp:523-560; the Single / Binary forms are the
 * same arithmetic on their own tables) */
static int orc_doublet(const orc_binding *B, int before, int i1, int i2, double ran)
{
    int s1 = orc_species(B, i1), s2 = orc_species(B, i2);
    if (s2 < s1) { int t = s1; s1 = s2; s2 = t; }
    const double *rt = B->drate[orc_pair_row(s1, s2)];
    int st = before ? 1 : 0;
    double r1 = rt[st * 2 + 0], r2 = rt[st * 2 + 1];
    double totalr = r1 + r2;
    double rr = totalr * ran;
    return !(rr < r1);
}

/* sort_triplet_and_save_permutation (Basic/basic.h:166-230): perm ids 0..5 = 123, 132, 312, 213, 231, 321 */
static int orc_sort3(const int t[3], int s[3])
{
    int a = t[0], b = t[1], c = t[2];
    if (a <= b) {
        if (b <= c) { s[0] = a; s[1] = b; s[2] = c; return 0; }
        if (a <= c) { s[0] = a; s[1] = c; s[2] = b; return 1; }
        s[0] = c; s[1] = a; s[2] = b; return 2;
    }
    if (a <= c) { s[0] = b; s[1] = a; s[2] = c; return 3; }
    if (b <= c) { s[0] = b; s[1] = c; s[2] = a; return 4; }
    s[0] = c; s[1] = b; s[2] = a; return 5;
}

/* save_to_type / inverse_save_to_type (Basic/basic.h:373-470) as slot maps over (12, 23, 13):
 * out[k] = in[map[perm][k]] */
static const int ORC_SAVE[6][3] = {{0, 1, 2}, {2, 1, 0}, {1, 2, 0}, {0, 2, 1}, {1, 2, 0}, {1, 0, 2}};
static const int ORC_UNSAVE[6][3] = {{0, 1, 2}, {2, 1, 0}, {1, 2, 0}, {0, 2, 1}, {2, 0, 1}, {1, 0, 2}};

/* AbstractBindingModel::triplet (BindingModelTernary.cpp:791-870) -> out[0..2] = (a12, a23, a13) */
static void orc_triplet(const orc_binding *B, const int b[3], const int c[3], int i1, int i2, int i3, double ran,
                        int out[3])
{
    int sp[3] = {orc_species(B, i1), orc_species(B, i2), orc_species(B, i3)}, st[3];
    int perm = orc_sort3(sp, st);
    int tb[3], tc[3], ta[3];
    for (int k = 0; k < 3; k++) { tb[k] = b[ORC_SAVE[perm][k]]; tc[k] = c[ORC_SAVE[perm][k]]; }
    int state = tb[0] ? 0 : (tb[1] ? 1 : (tb[2] ? 2 : 3));
    const double *rt = B->trate[orc_triple_row(st[0], st[1], st[2])];
    double r1 = tc[0] * rt[state * 4 + 0];
    double r2 = tc[1] * rt[state * 4 + 1];
    double r3 = tc[2] * rt[state * 4 + 2];
    double r4 = rt[state * 4 + 3];
    double totalr = r1 + r2 + r3 + r4;
    double rr = totalr * ran;
    ta[0] = ta[1] = ta[2] = 0;
    if (rr < r1) ta[0] = 1;
    else if (rr >= r1 && rr < r1 + r2) ta[1] = 1;
    else if (rr >= r1 + r2 && rr < r1 + r2 + r3) ta[2] = 1;
    for (int k = 0; k < 3; k++) out[k] = ta[ORC_UNSAVE[perm][k]];
}

/* uniform [0, 1) for a binding decision (Philox stream of the GPU path): cluster root patch, draw, the
 * decision's number inside its cluster */
double orc_bind_uniform(uint64_t seed, uint32_t replica, uint64_t draw, uint32_t root, uint32_t iter)
{
    uint32_t ctr[4] = {root, (uint32_t)draw, (uint32_t)(draw >> 32), replica};
    uint32_t key[2] = {(uint32_t)seed + 0x2545F491u * (iter + 1u), (uint32_t)(seed >> 32) ^ 0x6A09E667u};
    uint32_t o[4];
    orc_philox4x32_10(ctr, key, o);
    uint64_t w = ((uint64_t)o[1] << 32) | o[0];
    return (double)(w >> 11) * (1.0 / 9007199254740992.0);
}

typedef struct { int a, b; double scr; } orc_wedge;

/* one bound pair: KernFrenkelOnePatch2::force_and_torque of the pair's potential
 * (LangevinRforce.cpp:3960-4010) accumulated into F, T */
static void orc_bound_force(const orc_params *P, const double *x, const double *Q, int wp1, int wp2, double *F,
                            double *T)
{
    const orc_model *M = P->model;
    int p1, p2, k1, k2, c1, c2;
    orc_patch_owner(M, wp1, &p1, &k1, &c1);
    orc_patch_owner(M, wp2, &p2, &k2, &c2);
    if (p2 < p1) { int t = p1; p1 = p2; p2 = t; }
    double un[3];
    double dis = sqrt(orc_distance_vector(P, x, p1, p2, un));
    /* GeneralPatch::which_potential (GeneralPatch.cpp:450-462) with the patch numbers of wp1, wp2 */
    int potn = orc_pot_start(M, orc_type_of(M, p1), orc_type_of(M, p2)) + c1 * M->patches_per_type[k2] + c2;
    un[0] /= dis; un[1] /= dis; un[2] /= dis;
    int o1 = orc_orient_start(M, orc_type_of(M, p1)), o2 = orc_orient_start(M, orc_type_of(M, p2));
    double o[9];
    orc_kf2_force_torque(M->orient[o1 + c1], M->orient[o2 + c2], M->att[potn], M->dis[potn], M->thetam[potn], un,
                         dis, Q + 9 * p1, Q + 9 * p2, o);
    F[3 * p1 + 0] += o[0]; F[3 * p1 + 1] += o[1]; F[3 * p1 + 2] += o[2];
    F[3 * p2 + 0] += -o[0]; F[3 * p2 + 1] += -o[1]; F[3 * p2 + 2] += -o[2];
    T[3 * p1 + 0] += o[3]; T[3 * p1 + 1] += o[4]; T[3 * p1 + 2] += o[5];
    T[3 * p2 + 0] += o[6]; T[3 * p2 + 1] += o[7]; T[3 * p2 + 2] += o[8];
}

/* ConnectedComponents (Bindings/GraphAlgorithms.cpp:487-551) of n nodes under edges e[0..ne): the
 * depth-first order from each unvisited node in index order (DFUtilstore), neighbours in edge order.
 * ind <- visit order, dem[0..ncomp] <- component boundaries; returns ncomp. */
static int orc_dfs_components(int n, const orc_wedge *e, int ne, int *ind, int *dem)
{
    int *deg = (int *)calloc((size_t)n + 1, sizeof(int));
    int *adj = (int *)malloc(sizeof(int) * (size_t)(2 * ne + 1));
    int *fill = (int *)calloc((size_t)n + 1, sizeof(int));
    for (int q = 0; q < ne; q++) { deg[e[q].a + 1]++; deg[e[q].b + 1]++; }
    for (int i = 0; i < n; i++) deg[i + 1] += deg[i];
    for (int q = 0; q < ne; q++) {   /* PairHistogram order: a's list gets b, b's list gets a */
        adj[deg[e[q].a] + fill[e[q].a]++] = e[q].b;
        adj[deg[e[q].b] + fill[e[q].b]++] = e[q].a;
    }
    int *seen = (int *)calloc((size_t)n + 1, sizeof(int));
    int *stk = (int *)malloc(sizeof(int) * (size_t)(n + 1)), *pos = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    int it = 0, nc = 0;
    dem[0] = 0;
    for (int s = 0; s < n; s++) {
        if (seen[s]) continue;
        int top = 0;
        stk[0] = s; pos[0] = 0; seen[s] = 1; ind[it++] = s;
        while (top >= 0) {   /* recursive preorder, iteratively */
            int v = stk[top];
            if (pos[top] < deg[v + 1] - deg[v]) {
                int w = adj[deg[v] + pos[top]++];
                if (!seen[w]) { seen[w] = 1; ind[it++] = w; stk[++top] = w; pos[top] = 0; }
            } else {
                top--;
            }
        }
        nc++;
        dem[nc] = it;
    }
    free(deg); free(adj); free(fill); free(seen); free(stk); free(pos);
    return nc;
}

static int orc_first_max(const orc_wedge *e, int ne)
{
    int m = 0;
    for (int q = 1; q < ne; q++)
        if (e[m].scr < e[q].scr) m = q;   /* std::max_element with mdpairwdCompareScore */
    return m;
}

static void orc_push_pair(int **pairs, int *np, int *cap, int a, int b)
{
    if (*np == *cap) {
        *cap = *cap ? 2 * *cap : 64;
        *pairs = (int *)realloc(*pairs, sizeof(int) * 2 * (size_t)*cap);
    }
    (*pairs)[2 * *np] = a;
    (*pairs)[2 * *np + 1] = b;
    (*np)++;
}

/* the triplet's connectivity flags from the adjacency of its lowest member (LangevinRforce.cpp:3230-3280):
 * nb1 = degree of m1, first = its first neighbour; returns 0 or -1 (the reference's error()) */
static int orc_triplet_links(int nb1, int first, int nb2, int m2, int m3, int c[3])
{
    if (nb1 == 1) {
        if (first == m2) { c[0] = 1; c[2] = 0; c[1] = 1; }
        else if (first == m3) { c[2] = 1; c[0] = 0; c[1] = 1; }
        else return -1;
    } else if (nb1 == 2) {
        c[0] = 1; c[2] = 1;
        c[1] = nb2 == 1 ? 0 : 1;
    } else {
        return -1;
    }
    return 0;
}

static void orc_apply_triplet(const int a[3], int i1, int i2, int i3, int *boundto, unsigned char *isbound,
                              int **pairs, int *np, int *cap)
{
    if (a[0]) {
        boundto[i1] = i2; boundto[i2] = i1;
        isbound[i1] = 1; isbound[i2] = 1; isbound[i3] = 0;
        orc_push_pair(pairs, np, cap, i1, i2);
    } else if (a[1]) {
        boundto[i2] = i3; boundto[i3] = i2;
        isbound[i1] = 0; isbound[i2] = 1; isbound[i3] = 1;
        orc_push_pair(pairs, np, cap, i2, i3);
    } else if (a[2]) {
        boundto[i1] = i3; boundto[i3] = i1;
        isbound[i1] = 1; isbound[i2] = 0; isbound[i3] = 1;
        orc_push_pair(pairs, np, cap, i1, i3);
    } else {
        isbound[i1] = 0; isbound[i2] = 0; isbound[i3] = 0;
    }
}

static void orc_apply_doublet(int aft, int i1, int i2, int *boundto, unsigned char *isbound, int **pairs, int *np,
                              int *cap)
{
    if (aft) {
        boundto[i1] = i2; boundto[i2] = i1;
        isbound[i1] = 1; isbound[i2] = 1;
        orc_push_pair(pairs, np, cap, i1, i2);
    } else {
        isbound[i1] = 0; isbound[i2] = 0;
    }
}

static void orc_sort3_plain(int a, int b, int c, int s[3])
{
    int t[3] = {a, b, c};
    orc_sort3(t, s);
}

int orc_bind_update(const orc_params *P, const double *x, const double *Q, const orc_patchint *list, long nl,
                    const orc_binding *B, int rng, uint64_t seed, uint32_t replica, uint64_t draw, int *boundto,
                    unsigned char *isbound, double *F, double *T)
{
    const orc_model *M = P->model;
    const int np = orc_total_patches(M, P->n);
    const double mk = orc_max_check(M);
    int status = 0;

    /* ---- candidate patch pairs -> edges with scores (LangevinRforce.cpp:2900-3090) */
    orc_wedge *edges = (orc_wedge *)malloc(sizeof(orc_wedge) * (size_t)(nl + 1));
    int ne = 0;
    for (long q = 0; q < nl; q++) {
        const orc_patchint *e = list + q;
        double un[3];
        double dis = orc_distance_vector(P, x, e->p1, e->p2, un);
        if (!(dis < SQR(mk))) continue;
        dis = sqrt(dis);
        un[0] /= dis; un[1] /= dis; un[2] /= dis;
        int wp1 = e->wp1, wp2 = e->wp2, potn = e->potn;
        int k1 = orc_type_of(M, e->p1), k2 = orc_type_of(M, e->p2);
        int ps = orc_pot_start(M, k1, k2), n2 = M->patches_per_type[k2];
        int a = (potn - ps) / n2, b = (potn - ps) % n2;
        double m1[3], m2[3];
        orc_lab_patch(M->orient[orc_orient_start(M, k1) + a], Q + 9 * e->p1, m1);
        orc_lab_patch(M->orient[orc_orient_start(M, k2) + b], Q + 9 * e->p2, m2);
        double disp = 1.4 * M->dis[potn], thetam = M->thetam[potn], ctm = cos(thetam);
        double ai = -(m1[0] * un[0] + m1[1] * un[1] + m1[2] * un[2]);
        double aj = (m2[0] * un[0] + m2[1] * un[1] + m2[2] * un[2]);
        int cond1 = boundto[wp1] == wp2 && boundto[wp2] == wp1;
        int b1 = isbound[wp1] != 0, b2 = isbound[wp2] != 0;
        double disp2;
        if (b1 && b2 && cond1) disp2 = disp;
        else if (b1 && b2 && !cond1) disp2 = 0.5 * disp;
        else if (b1 != b2) disp2 = 0.7 * disp;
        else disp2 = disp;
        if (ai > ctm && aj > ctm && dis < disp2) {
            double scr1 = 1 - (ai - cos(thetam));
            double scr2 = 1 - (aj - cos(thetam));
            double scr3 = 2 * (dis / disp2);
            edges[ne].a = wp1; edges[ne].b = wp2; edges[ne].scr = scr1 + scr2 + scr3;
            ne++;
        }
    }

    /* ---- PairHistogramExtended (GraphAlgorithms.cpp:264-330): per patch, partners and scores in edge order */
    int *start = (int *)calloc((size_t)np + 1, sizeof(int));
    int *fill = (int *)calloc((size_t)np + 1, sizeof(int));
    int *nbr = (int *)malloc(sizeof(int) * (size_t)(2 * ne + 1));
    double *nsc = (double *)malloc(sizeof(double) * (size_t)(2 * ne + 1));
    for (int q = 0; q < ne; q++) { start[edges[q].a + 1]++; start[edges[q].b + 1]++; }
    for (int i = 0; i < np; i++) start[i + 1] += start[i];
    for (int q = 0; q < ne; q++) {
        int a = edges[q].a, b = edges[q].b;
        nbr[start[a] + fill[a]] = b; nsc[start[a] + fill[a]++] = edges[q].scr;
        nbr[start[b] + fill[b]] = a; nsc[start[b] + fill[b]++] = edges[q].scr;
    }
#define DEG(i) (start[(i) + 1] - start[(i)])

    /* ---- a bond whose partner is no longer a candidate breaks (LangevinRforce.cpp:3110-3133) */
    for (int i = 0; i < np; i++) {
        if (!isbound[i]) continue;
        int found = 0;
        for (int k = start[i]; k < start[i + 1]; k++)
            if (nbr[k] == boundto[i]) { found = 1; break; }
        if (!found) isbound[i] = 0;
    }

    /* ---- ConnectedComponentsParallel_Old: each patch labelled by the smallest index of its component;
     * SingleHistogram (GraphAlgorithms.cpp:2-48): members per label in increasing order */
    int *lab = (int *)malloc(sizeof(int) * (size_t)(np + 1));
    for (int i = 0; i < np; i++) lab[i] = i;
    for (int q = 0; q < ne; q++) {
        int a = orc_find(lab, edges[q].a), b = orc_find(lab, edges[q].b);
        if (a < b) lab[b] = a;
        else if (b < a) lab[a] = b;
    }
    for (int i = 0; i < np; i++) lab[i] = orc_find(lab, i);
    int *ccs = (int *)calloc((size_t)np + 1, sizeof(int));
    for (int i = 0; i < np; i++) ccs[lab[i]]++;
    int *mstart = (int *)calloc((size_t)np + 1, sizeof(int));
    for (int i = 0; i < np; i++) mstart[i + 1] = mstart[i] + ccs[i];
    int *members = (int *)malloc(sizeof(int) * (size_t)(np + 1));
    int *mfill = (int *)calloc((size_t)np + 1, sizeof(int));
    for (int i = 0; i < np; i++) members[mstart[lab[i]] + mfill[lab[i]]++] = i;

    /* ---- one random number per cluster of two or more (Generate_Random_Numbers_Needed,
     * GraphAlgorithms.cpp:431-438) */
    double *rands = (double *)calloc((size_t)np + 1, sizeof(double));
    int maxc = 0;
    for (int i = 0; i < np; i++) {
        if (ccs[i] > maxc) maxc = ccs[i];
        if (ccs[i] > 1)
            rands[i] = rng == 1 ? (double)rand() / (double)RAND_MAX : orc_bind_uniform(seed, replica, draw, (uint32_t)i, 0);
    }

    int *bpairs = NULL, nbp = 0, bcap = 0;
    int *large = (int *)malloc(sizeof(int) * (size_t)(np + 1));
    int nlarge = 0;
    /* ---- clusters of one, two and three patches (LangevinRforce.cpp:3160-3480) */
    for (int i = 0; i < np && status == 0; i++) {
        int sz = ccs[i];
        const int *mb = members + mstart[i];
        if (sz == 0) continue;
        if (sz == 1) {
            isbound[mb[0]] = 0;
        } else if (sz == 2) {
            int i1 = mb[0] < mb[1] ? mb[0] : mb[1], i2 = mb[0] < mb[1] ? mb[1] : mb[0];
            int already = boundto[i1] == i2 && boundto[i2] == i1 && isbound[i1] && isbound[i2];
            orc_apply_doublet(orc_doublet(B, already, i1, i2, rands[i]), i1, i2, boundto, isbound, &bpairs, &nbp, &bcap);
        } else if (sz == 3) {
            int s[3];
            orc_sort3_plain(mb[0], mb[1], mb[2], s);
            int i1 = s[0], i2 = s[1], i3 = s[2];
            int bb[3] = {boundto[i1] == i2 && boundto[i2] == i1 && isbound[i1] && isbound[i2],
                         boundto[i2] == i3 && boundto[i3] == i2 && isbound[i2] && isbound[i3],
                         boundto[i1] == i3 && boundto[i3] == i1 && isbound[i1] && isbound[i3]};
            int c[3] = {0, 0, 0};
            if (orc_triplet_links(DEG(i1), DEG(i1) > 0 ? nbr[start[i1]] : -1, DEG(i2), i2, i3, c)) { status = -2; break; }
            int a[3];
            orc_triplet(B, bb, c, i1, i2, i3, rands[i], a);
            orc_apply_triplet(a, i1, i2, i3, boundto, isbound, &bpairs, &nbp, &bcap);
        } else {
            large[nlarge++] = i;
        }
    }

    /* ---- larger clusters: drop the highest-scoring edge until no component exceeds three patches,
     * then decide the pieces (LangevinRforce.cpp:3560-3880) */
    int ncols = maxc / 2 + 1;
    double *rl = (double *)malloc(sizeof(double) * (size_t)(nlarge > 0 ? nlarge * ncols : 1));
    if (rng == 1)
        for (int q = 0; q < nlarge * ncols; q++) rl[q] = (double)rand() / (double)RAND_MAX;   /* generate_random_matrix */
    for (int allc = 0; allc < nlarge && status == 0; allc++) {
        int root = large[allc], m = ccs[root];
        const int *u = members + mstart[root];   /* unique_indexes, increasing */
        /* RecapitulateEdges (LangevinRforceUtil.cpp:508-572): local (a < b) edges in member / neighbour order */
        int cap = 1;
        for (int j = 0; j < m; j++) cap += DEG(u[j]);
        orc_wedge *me = (orc_wedge *)malloc(sizeof(orc_wedge) * (size_t)cap);
        int nme = 0;
        for (int j = 0; j < m; j++)
            for (int k = start[u[j]]; k < start[u[j] + 1]; k++) {
                int f2 = 0;
                while (f2 < m && u[f2] != nbr[k]) f2++;
                int a = j < f2 ? j : f2, b = j < f2 ? f2 : j;
                int dup = 0;
                for (int l = 0; l < nme; l++)
                    if (me[l].a == a && me[l].b == b) { dup = 1; break; }
                if (!dup) { me[nme].a = a; me[nme].b = b; me[nme].scr = nsc[k]; nme++; }
            }
        int *ind = (int *)malloc(sizeof(int) * (size_t)m), *dem = (int *)malloc(sizeof(int) * (size_t)(m + 1));
        int mx = orc_first_max(me, nme);
        memmove(me + mx, me + mx + 1, sizeof(orc_wedge) * (size_t)(nme - mx - 1));
        nme--;
        int ncomp = orc_dfs_components(m, me, nme, ind, dem);
        for (;;) {
            int big = 0;
            for (int q = 0; q < ncomp; q++)
                if (dem[q + 1] - dem[q] > big) big = dem[q + 1] - dem[q];
            if (big <= 3) break;
            mx = orc_first_max(me, nme);
            memmove(me + mx, me + mx + 1, sizeof(orc_wedge) * (size_t)(nme - mx - 1));
            nme--;
            ncomp = orc_dfs_components(m, me, nme, ind, dem);
        }
        /* PairHistogram of the remaining edges (degree <= 2 inside a piece) */
        int *lens = (int *)calloc((size_t)m, sizeof(int)), *bx = (int *)malloc(sizeof(int) * 3 * (size_t)m);
        for (int q = 0; q < nme; q++) {
            bx[3 * me[q].a + lens[me[q].a]++] = me[q].b;
            bx[3 * me[q].b + lens[me[q].b]++] = me[q].a;
        }
        for (int k1 = 0; k1 < m; k1++) {
            if (!isbound[u[k1]]) continue;
            int outside = 1;
            for (int k = 0; k < lens[k1]; k++)
                if (boundto[u[k1]] == u[bx[3 * k1 + k]]) { outside = 0; break; }
            if (outside) isbound[u[k1]] = 0;
        }
        int it = 0;
        for (int j = 0; j < ncomp && status == 0; j++) {
            int sz = dem[j + 1] - dem[j];
            double ran = 0;
            if (sz == 2 || sz == 3)
                ran = rng == 1 ? rl[allc * ncols + it] : orc_bind_uniform(seed, replica, draw, (uint32_t)root, (uint32_t)it);
            if (sz == 1) {
                isbound[u[ind[dem[j]]]] = 0;
            } else if (sz == 2) {
                int t1 = u[ind[dem[j]]], t2 = u[ind[dem[j] + 1]];
                int i1 = t1 <= t2 ? t1 : t2, i2 = t1 <= t2 ? t2 : t1;
                int already = boundto[i1] == i2 && boundto[i2] == i1 && isbound[i1] && isbound[i2];
                orc_apply_doublet(orc_doublet(B, already, i1, i2, ran), i1, i2, boundto, isbound, &bpairs, &nbp, &bcap);
                it++;
            } else if (sz == 3) {
                int ni[3], s[3];
                orc_sort3_plain(ind[dem[j]], ind[dem[j] + 1], ind[dem[j] + 2], ni);
                orc_sort3_plain(u[ni[0]], u[ni[1]], u[ni[2]], s);
                int i1 = s[0], i2 = s[1], i3 = s[2];
                int bb[3] = {boundto[i1] == i2 && boundto[i2] == i1 && isbound[i1] && isbound[i2],
                             boundto[i2] == i3 && boundto[i3] == i2 && isbound[i2] && isbound[i3],
                             boundto[i1] == i3 && boundto[i3] == i1 && isbound[i1] && isbound[i3]};
                int c[3] = {0, 0, 0};
                if (orc_triplet_links(lens[ni[0]], lens[ni[0]] > 0 ? bx[3 * ni[0]] : -1, lens[ni[1]], ni[1], ni[2], c)) {
                    status = -2;
                    break;
                }
                int a[3];
                orc_triplet(B, bb, c, i1, i2, i3, ran, a);
                orc_apply_triplet(a, i1, i2, i3, boundto, isbound, &bpairs, &nbp, &bcap);
                it++;
            } else {
                status = -3;
            }
        }
        free(me); free(ind); free(dem); free(lens); free(bx);
    }
#undef DEG

    /* ---- forces of the bound pairs only, in the order they were made (LangevinRforce.cpp:3940-4030) */
    if (status == 0)
        for (int q = 0; q < nbp; q++) orc_bound_force(P, x, Q, bpairs[2 * q], bpairs[2 * q + 1], F, T);

    free(edges); free(start); free(fill); free(nbr); free(nsc); free(lab); free(ccs); free(mstart); free(members);
    free(mfill); free(rands); free(large); free(rl); free(bpairs);
    return status;
}

/* calculate_score(i1, i2, before) of the binding model in table form: BindingModelSingle off_rate if the pair
 * is bound to each other, else on_rate (BindingModelSingle.cpp:25-36; the table holds [0] = [2] = off,
 * [1] = [3] = on); BindingModelBinary doubr11 if both indices are below div, doubr12 if only i1 is, else doubr22,
 * entry [before * 2 + 1] if bound, [before * 2 + 0] if not (BindingModelBinary.cpp:194-230);
 * BindingModelTernary the sorted species pair's [before * 2 + 1] (BindingModelTernary.cpp:596-640) */
static double orc_calculate_score(const orc_binding *B, int i1, int i2, int before)
{
    if (B->rule == 0) return before ? B->drate[0][2] : B->drate[0][1];
    if (B->rule == 1) {
        int row = (i1 < B->div1 && i2 < B->div1) ? 0 : (i1 < B->div1 ? 1 : 3);
        return B->drate[row][before * 2 + (before ? 1 : 0)];
    }
    int s1 = orc_species(B, i1), s2 = orc_species(B, i2);
    if (s2 < s1) { int t = s1; s1 = s2; s2 = t; }
    return B->drate[orc_pair_row(s1, s2)][before * 2 + 1];
}

/* one edge of setup_random_binding: its patches, score and place in the seeded order */
typedef struct { int a, b; double scr; uint32_t prio; int lo, hi; } orc_sedge;

static int orc_sedge_cmp(const void *x, const void *y)
{
    const orc_sedge *e = (const orc_sedge *)x, *f = (const orc_sedge *)y;
    if (e->prio != f->prio) return e->prio < f->prio ? -1 : 1;
    if (e->lo != f->lo) return e->lo < f->lo ? -1 : 1;
    return e->hi < f->hi ? -1 : (e->hi > f->hi ? 1 : 0);
}

uint32_t orc_setup_priority(uint64_t seed, uint32_t replica, uint32_t lo, uint32_t hi)
{
    uint32_t ctr[4] = {lo, hi, replica, 0x53455455u};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    orc_philox4x32_10(ctr, key, o);
    return o[0];
}

/* the edges of setup_random_binding and their scores (LangevinRforceUtil.cpp:781-930): the edge test of the
 * bond update, score scr1 + scr2 + scr3 + scr4; returns the count */
static long orc_setup_edge_list(const orc_params *P, const double *x, const double *Q, const orc_patchint *list,
                                long nl, const orc_binding *B, uint64_t seed, uint32_t replica, const int *boundto,
                                const unsigned char *isbound, orc_sedge *edges)
{
    const orc_model *M = P->model;
    const double mk = orc_max_check(M);
    long ne = 0;
    for (long q = 0; q < nl; q++) {
        const orc_patchint *e = list + q;
        double un[3];
        double dis = orc_distance_vector(P, x, e->p1, e->p2, un);
        if (!(dis < SQR(mk))) continue;
        dis = sqrt(dis);
        un[0] /= dis; un[1] /= dis; un[2] /= dis;
        int wp1 = e->wp1, wp2 = e->wp2, potn = e->potn;
        int k1 = orc_type_of(M, e->p1), k2 = orc_type_of(M, e->p2);
        int ps = orc_pot_start(M, k1, k2), n2 = M->patches_per_type[k2];
        int a = (potn - ps) / n2, b = (potn - ps) % n2;
        double m1[3], m2[3];
        orc_lab_patch(M->orient[orc_orient_start(M, k1) + a], Q + 9 * e->p1, m1);
        orc_lab_patch(M->orient[orc_orient_start(M, k2) + b], Q + 9 * e->p2, m2);
        double disp = 1.4 * M->dis[potn], thetam = M->thetam[potn], ctm = cos(thetam);
        double ai = -(m1[0] * un[0] + m1[1] * un[1] + m1[2] * un[2]);
        double aj = (m2[0] * un[0] + m2[1] * un[1] + m2[2] * un[2]);
        int cond1 = boundto[wp1] == wp2 && boundto[wp2] == wp1;
        int b1 = isbound[wp1] != 0, b2 = isbound[wp2] != 0;
        double disp2;
        if (b1 && b2 && cond1) disp2 = disp;
        else if (b1 && b2 && !cond1) disp2 = 0.5 * disp;
        else if (b1 != b2) disp2 = 0.7 * disp;
        else disp2 = disp;
        if (ai > ctm && aj > ctm && dis < disp2) {
            double scr1 = 1 - (ai - cos(thetam));
            double scr2 = 1 - (aj - cos(thetam));
            double scr3 = 2 * (dis / disp2);
            double scr4 = -log(1E-10 + orc_calculate_score(B, wp1, wp2, b1 && b2 && cond1));
            orc_sedge *s = edges + ne++;
            s->a = wp1; s->b = wp2; s->scr = scr1 + scr2 + scr3 + scr4;
            s->lo = wp1 < wp2 ? wp1 : wp2; s->hi = wp1 < wp2 ? wp2 : wp1;
            s->prio = orc_setup_priority(seed, replica, (uint32_t)s->lo, (uint32_t)s->hi);
        }
    }
    return ne;
}

long orc_setup_edges(const orc_params *P, const double *x, const double *Q, const orc_patchint *list, long nl,
                     const orc_binding *B, const int *boundto, const unsigned char *isbound, int *ab, double *scr)
{
    orc_sedge *edges = (orc_sedge *)malloc(sizeof(orc_sedge) * (size_t)(nl + 1));
    long ne = orc_setup_edge_list(P, x, Q, list, nl, B, 0, 0, boundto, isbound, edges);
    for (long i = 0; i < ne; i++) {
        ab[2 * i] = edges[i].a;
        ab[2 * i + 1] = edges[i].b;
        scr[i] = edges[i].scr;
    }
    free(edges);
    return ne;
}

int orc_setup_random_binding(const orc_params *P, const double *x, const double *Q, const orc_patchint *list, long nl,
                             const orc_binding *B, uint64_t seed, uint32_t replica, int *boundto,
                             unsigned char *isbound)
{
    orc_sedge *edges = (orc_sedge *)malloc(sizeof(orc_sedge) * (size_t)(nl + 1));
    long ne = orc_setup_edge_list(P, x, Q, list, nl, B, seed, replica, boundto, isbound, edges);
    /* the reference's std::shuffle of the edges, here the seeded order; then the greedy walk
     * (LangevinRforceUtil.cpp:985-1005) */
    qsort(edges, (size_t)ne, sizeof(orc_sedge), orc_sedge_cmp);
    for (long i = 0; i < ne; i++) {
        int wp1 = edges[i].a, wp2 = edges[i].b;
        if (!isbound[wp1] && !isbound[wp2] && edges[i].scr < 4.) {
            isbound[wp1] = 1; isbound[wp2] = 1;
            boundto[wp1] = wp2; boundto[wp2] = wp1;
        }
    }
    free(edges);
    return 0;
}

static long orc_patch_list_alloc(const orc_params *P, const double *x, const double *Q, const int *pairs, long np,
                                 double max_ang, orc_patchint **out)
{
    long n = orc_patch_list(P, x, Q, pairs, np, max_ang, NULL, 0);
    *out = (orc_patchint *)malloc(sizeof(orc_patchint) * (size_t)(n > 0 ? n : 1));
    orc_patch_list(P, x, Q, pairs, np, max_ang, *out, n);
    return n;
}

int orc_run_singlebond(const orc_params *P, double *x, double *p, double *Lb, double *Q, double *Ft, double *Tt,
                       int *boundto, unsigned char *isbound, const orc_binding *B, double max_ang, int nsteps, int i0,
                       int ncell, double pair_cut, int pair_every, int patch_every, int init, uint64_t init_draw,
                       int noise_mode, const double *noise, uint64_t seed, uint32_t replica, uint64_t draw0)
{
    int n = P->n, status = 0;
    int *pairs = NULL;
    orc_patchint *plist = NULL;
    double *xi = (double *)calloc(6 * (size_t)(n > 0 ? n : 1), sizeof(double));
    long np = orc_pairs_alloc(P, x, ncell, pair_cut, &pairs);
    long nl = orc_patch_list_alloc(P, x, Q, pairs, np, max_ang, &plist);
    if (init) {
        orc_central_forces(P, x, pairs, np, Ft);
        memset(Tt, 0, sizeof(double) * 3 * (size_t)n);
        status |= orc_bind_update(P, x, Q, plist, nl, B, 0, seed, replica, init_draw, boundto, isbound, Ft, Tt);
        if (noise_mode == 2) orc_philox_noise(n, seed, replica, init_draw, xi);
        orc_langevin_forces(P, p, Lb, Q, xi, Ft, Tt);   /* Philox draw init_draw, or xi = 0 */
    }
    for (int s = 0; s < nsteps; s++) {
        int i = i0 + s;
        if (i > 0 && i % pair_every == 0 && s > 0) {
            free(pairs);
            np = orc_pairs_alloc(P, x, ncell, pair_cut, &pairs);
        }
        if (i > 0 && i % patch_every == 0) {
            free(plist);
            nl = orc_patch_list_alloc(P, x, Q, pairs, np, max_ang, &plist);
        }
        orc_halfkick(n, P->dt, p, Lb, Ft, Tt);
        orc_drift(P, x, p);
        orc_rotate(P, Lb, Q);
        orc_central_forces(P, x, pairs, np, Ft);
        memset(Tt, 0, sizeof(double) * 3 * (size_t)n);
        status |= orc_bind_update(P, x, Q, plist, nl, B, 0, seed, replica, draw0 + (uint64_t)s, boundto, isbound, Ft, Tt);
        const double *nz = xi;
        if (noise_mode == 1) nz = noise + 6 * (size_t)n * (size_t)s;
        else if (noise_mode == 2) orc_philox_noise(n, seed, replica, draw0 + (uint64_t)s, xi);
        else memset(xi, 0, sizeof(double) * 6 * (size_t)n);
        orc_langevin_forces(P, p, Lb, Q, nz, Ft, Tt);
        orc_halfkick(n, P->dt, p, Lb, Ft, Tt);
    }
    free(pairs);
    free(plist);
    free(xi);
    return status;
}

/* ---------------------------------------------------------------- seeded synthetic inputs */

/* splitmix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014) */
static uint64_t orc_splitmix(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* [0, 1) from the top 53 bits */
static double orc_unit(uint64_t *s) { return (double)(orc_splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

/* accepted particles hashed by cell: head per cell, next per particle */
typedef struct {
    int nc;
    double scale;
    int *head, *next;
} orc_hash;

static int orc_hash_init(orc_hash *h, double box, double min_dist, int cap_nc, long n)
{
    int nc = min_dist > 0 ? (int)floor(box / min_dist) : 1;
    if (nc < 1) nc = 1;
    if (nc > cap_nc) nc = cap_nc;
    h->nc = nc;
    h->scale = nc / box;
    size_t ncell = (size_t)nc * nc * nc;
    h->head = (int *)malloc(sizeof(int) * ncell);
    h->next = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!h->head || !h->next) return -1;
    for (size_t c = 0; c < ncell; c++) h->head[c] = -1;
    for (long i = 0; i < (n > 0 ? n : 1); i++) h->next[i] = -1;
    return 0;
}

static void orc_hash_free(orc_hash *h)
{
    free(h->head);
    free(h->next);
}

static int orc_hash_cell(const orc_hash *h, const double c[3], int clamp_low)
{
    int ci[3];
    for (int k = 0; k < 3; k++) {
        ci[k] = (int)(c[k] * h->scale);
        if (ci[k] >= h->nc) ci[k] = h->nc - 1;
        if (clamp_low && ci[k] < 0) ci[k] = 0;
    }
    return ci[0] + h->nc * (ci[1] + h->nc * ci[2]);
}

/* 1 if no accepted particle of the 27 surrounding cells is closer than sqrt(md2) (minimum image) */
static int orc_hash_free_at(const orc_hash *h, const double *x, const double c[3], int cell, double box, int periodic,
                            double md2)
{
    const int nc = h->nc;
    const int ci[3] = {cell % nc, (cell / nc) % nc, cell / (nc * nc)};
    const int lo = nc >= 3 ? -1 : 0, hi = nc >= 2 ? 1 : 0;
    for (int dz = lo; dz <= hi; dz++)
        for (int dy = lo; dy <= hi; dy++)
            for (int dx = lo; dx <= hi; dx++) {
                int a = ci[0] + dx, b = ci[1] + dy, e = ci[2] + dz;
                if (!periodic && (a < 0 || a >= nc || b < 0 || b >= nc || e < 0 || e >= nc)) continue;
                a = (a + nc) % nc;
                b = (b + nc) % nc;
                e = (e + nc) % nc;
                for (int j = h->head[(size_t)a + nc * ((size_t)b + (size_t)nc * e)]; j >= 0; j = h->next[j]) {
                    double d2 = 0;
                    for (int k = 0; k < 3; k++) {
                        double d = c[k] - x[3 * (size_t)j + k];
                        if (periodic) d -= box * nearbyint(d / box);
                        d2 += d * d;
                    }
                    if (d2 < md2) return 0;
                }
            }
    return 1;
}

int orc_random_positions(int n, double box, int periodic, double min_dist, uint64_t seed, double *x)
{
    if (n < 0 || box <= 0 || min_dist < 0 || !x) return -1;
    uint64_t s = seed ^ 0x5DEECE66Dull;
    orc_hash h;
    if (orc_hash_init(&h, box, min_dist, 512, n) != 0) {
        orc_hash_free(&h);
        return -1;
    }
    const double md2 = min_dist * min_dist;
    long long attempts = 0, limit = 1000LL * (long long)(n > 0 ? n : 1);
    int placed = 0;
    while (placed < n) {
        if (++attempts > limit) {
            orc_hash_free(&h);
            return -1;
        }
        double c[3];
        c[0] = orc_unit(&s) * box;   /* one statement each: the draws are taken x, y, z */
        c[1] = orc_unit(&s) * box;
        c[2] = orc_unit(&s) * box;
        const int cell = orc_hash_cell(&h, c, 0);
        if (!orc_hash_free_at(&h, x, c, cell, box, periodic, md2)) continue;
        for (int k = 0; k < 3; k++) x[3 * (size_t)placed + k] = c[k];
        h.next[placed] = h.head[cell];
        h.head[cell] = placed;
        placed++;
    }
    orc_hash_free(&h);
    return 0;
}

void orc_random_rotations(int n, uint64_t seed, double *Q)
{
    uint64_t s = seed ^ 0xA0761D6478BD642Full;
    const double two_pi = 6.283185307179586476925286766559;
    for (int i = 0; i < n; i++) {
        double x1 = orc_unit(&s);
        double x2 = orc_unit(&s);
        double x3 = orc_unit(&s);
        /* v uniform on the sphere's upper half from (x2, x3), a Householder reflection of a rotation about
         * z by 2 pi x1: the construction of LangevinR.cpp:239-267 */
        double v[3] = {cos(two_pi * x2) * sqrt(x3), sin(two_pi * x2) * sqrt(x3), sqrt(1. - x3)};
        double c = cos(two_pi * x1), sn = sin(two_pi * x1);
        double Rz[3][3] = {{c, sn, 0}, {-sn, c, 0}, {0, 0, 1}};
        double *q = Q + 9 * (size_t)i;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double acc = 0;
                for (int k = 0; k < 3; k++) acc += (2 * v[a] * v[k] - (a == k ? 1.0 : 0.0)) * Rz[k][b];
                q[3 * a + b] = acc;
            }
    }
}

int orc_random_chains(int n_chains, int beads, double box, int periodic, double step, double min_dist,
                      uint64_t seed, double *x)
{
    if (n_chains < 0 || beads < 1 || box <= 0 || step <= 0 || min_dist < 0 || min_dist >= step || !x) return -1;
    const long long n = (long long)n_chains * beads;
    if (n > 2147483647LL) return -1;
    uint64_t s = seed ^ 0x2545F4914F6CDD1Dull;
    orc_hash h;
    int *cell_of = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!cell_of || orc_hash_init(&h, box, min_dist, 1024, (long)n) != 0) {
        free(cell_of);
        return -1;
    }
    const double md2 = min_dist * min_dist;
    int status = 0;
    for (int ch = 0; ch < n_chains && status == 0; ch++) {
        const int i0 = ch * beads;
        int done = 0;
        for (int restart = 0; restart < 1000 && !done; restart++) {
            int placed = 0;
            for (int tries = 0; tries < 10000 && placed == 0; tries++) {
                double c[3];
                c[0] = orc_unit(&s) * box;
                c[1] = orc_unit(&s) * box;
                c[2] = orc_unit(&s) * box;
                const int cell = orc_hash_cell(&h, c, 1);
                if (orc_hash_free_at(&h, x, c, cell, box, periodic, md2)) {
                    for (int k = 0; k < 3; k++) x[3 * (size_t)i0 + k] = c[k];
                    cell_of[i0] = cell;
                    h.next[i0] = h.head[cell];
                    h.head[cell] = i0;
                    placed = 1;
                }
            }
            if (!placed) {
                status = -1;
                break;
            }
            while (placed < beads) {
                int ok = 0;
                for (int tries = 0; tries < 200 && !ok; tries++) {
                    double v[3], r2 = 0;
                    do {
                        r2 = 0;
                        for (int k = 0; k < 3; k++) {
                            v[k] = 2.0 * orc_unit(&s) - 1.0;
                            r2 += v[k] * v[k];
                        }
                    } while (r2 > 1.0 || r2 < 1e-6);
                    const double inv = step / sqrt(r2);
                    double c[3];
                    int inside = 1;
                    for (int k = 0; k < 3; k++) {
                        c[k] = x[3 * (size_t)(i0 + placed - 1) + k] + v[k] * inv;
                        if (periodic) {
                            if (c[k] < 0) c[k] += box;
                            else if (c[k] >= box) c[k] -= box;
                        } else if (c[k] < 0 || c[k] >= box) {
                            inside = 0;
                        }
                    }
                    if (!inside) continue;
                    const int cell = orc_hash_cell(&h, c, 1);
                    if (orc_hash_free_at(&h, x, c, cell, box, periodic, md2)) {
                        const int i = i0 + placed;
                        for (int k = 0; k < 3; k++) x[3 * (size_t)i + k] = c[k];
                        cell_of[i] = cell;
                        h.next[i] = h.head[cell];
                        h.head[cell] = i;
                        ok = 1;
                    }
                }
                if (!ok) break;
                placed++;
            }
            if (placed == beads) {
                done = 1;
            } else {
                /* stuck: unlink this chain's beads (the most recent insertions head their cells) */
                for (int i = i0 + placed - 1; i >= i0; i--) h.head[cell_of[i]] = h.next[i];
            }
        }
        if (!done && status == 0) status = -1;
    }
    orc_hash_free(&h);
    free(cell_of);
    return status;
}
