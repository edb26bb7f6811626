/* Test infrastructure, not product code.
 *
 * CPU oracle: plain-C restatement of the reference fdm algorithms on the
 * Poisson / NSCube path (declarations and the list of what each function
 * restates: fdm_oracle.h).  The tests, the smoke check and the CPU-baseline
 * leg of bench.py are its only users; the product never links it.
 *
 * Arithmetic follows the reference expression by expression so that the
 * results agree to round-off; the code itself is written independently.
 */
#include "fdm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static int g_threads = 0;

void orc_set_threads(int n) { g_threads = n; }

int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

static double sqd(double x) { return x * x; } /* asp::sq, src/asp_misc.h:295 */

static int log2_exact(int N) {
    int q = 0;
    if (N < 2) return -1;
    while ((1 << q) < N) q++;
    return (1 << q) == N ? q : -1;
}

/* ------------------------------------------------------------------ */
/* DST-I (Samarskii-Nikolaev real recursion)                           */
/* ------------------------------------------------------------------ */

/* Table of 1/(2 cos(pi (2k-1) / 2^(l+2))), l = -1..q-1, k = 1..2^(l+1);
 * entry (k,l) at [(l+1)*N + k-1].  Restates FFTTable::init's ffiCOS,
 * src/fft.cpp:60-95. */
typedef struct {
    int N, q;
    double* icos;
} sn_table;

static int sn_table_init(sn_table* t, int N) {
    t->N = N;
    t->q = log2_exact(N);
    if (t->q < 0) return -1;
    t->icos = (double*)calloc((size_t)(t->q + 1) * N, sizeof(double));
    for (int l = -1; l <= t->q - 1; l++)
        for (int k = 1; k <= (1 << (l + 1)); k++) {
            double x = 2. * cos(M_PI * (2 * k - 1) / (1 << (l + 2)));
            t->icos[(l + 1) * N + (k - 1)] = 1. / x;
        }
    return 0;
}

static void sn_table_free(sn_table* t) { free(t->icos); }

/* One sine transform; work arrays b, bn of N entries.  Restates
 * FFT<T>::sFFT(S,s,dx,N,n), src/fft.cpp:294-359: for each level l the
 * input is folded (sadvance, :26-33), the b-recursion (36) builds the
 * reduced rows, the z-recursion (37) applies the 1/(2cos) factors, and the
 * outputs S[2^(q-l-1)(2k-1)] are read off.  S[N/2] comes last. */
static void sn_sine(const sn_table* t, double* S, double* a, double dx, double* b, double* bn) {
    const int N = t->N, q = t->q;
    for (int l = q - 1; l >= 1; l--) {
        const int half = 1 << l;
        for (int j = 1; j <= half - 1; j++) {
            double lo = a[j], hi = a[2 * half - j];
            a[j] = lo - hi;
            a[2 * half - j] = lo + hi;
        }
        for (int j = 1; j <= half; j++) b[j - 1] = a[2 * half - j];
        int m;
        for (m = 1; m <= l - 1; m++) {
            const int W = 1 << m, Wp = W >> 1, rows = 1 << (l - m);
            for (int j = 1; j <= rows - 1; j++)
                for (int s = 1; s <= Wp; s++) {
                    bn[(j - 1) * W + 2 * s - 2] = b[(2 * j - 2) * Wp + s - 1] + b[(2 * j) * Wp + s - 1];
                    bn[(j - 1) * W + 2 * s - 1] = b[(2 * j - 1) * Wp + s - 1];
                }
            for (int s = 1; s <= Wp; s++) {
                bn[(rows - 1) * W + 2 * s - 2] = b[(2 * rows - 2) * Wp + s - 1];
                bn[(rows - 1) * W + 2 * s - 1] = b[(2 * rows - 1) * Wp + s - 1];
            }
            double* tmp = b; b = bn; bn = tmp;
        }
        {   /* m == l: interleave the two remaining rows */
            const int Wp = 1 << (l - 1);
            for (int s = 1; s <= Wp; s++) {
                bn[2 * s - 1] = b[Wp + s - 1];
                bn[2 * s - 2] = b[s - 1];
            }
            double* tmp = b; b = bn; bn = tmp;
        }
        for (m = l; m >= 1; m--) {
            const int W = 1 << m, Wh = W >> 1, rows = 1 << (l - m);
            const double* ic = t->icos + (size_t)(l - m + 1) * N;
            for (int k = 1; k <= rows; k++) {
                const double c = ic[k - 1];
                for (int s = 1; s <= Wh; s++) {
                    double even = b[(k - 1) * W + 2 * s - 1];
                    double odd = b[(k - 1) * W + 2 * s - 2];
                    bn[(k - 1) * Wh + s - 1] = even + c * odd;
                    bn[(2 * rows - k) * Wh + s - 1] = -even + c * odd;
                }
            }
            double* tmp = b; b = bn; bn = tmp;
        }
        for (int k = 1; k <= half; k++) S[(1 << (q - l - 1)) * (2 * k - 1)] = dx * b[k - 1];
    }
    S[1 << (q - 1)] = dx * a[1];
}

int orc_sfft(double* S, double* s, double dx, int N) {
    sn_table t;
    if (sn_table_init(&t, N)) return -1;
    double* b = (double*)calloc(N, sizeof(double));
    double* bn = (double*)calloc(N, sizeof(double));
    sn_sine(&t, S, s, dx, b, bn);
    free(b);
    free(bn);
    sn_table_free(&t);
    return 0;
}

void orc_sft_naive(double* S, const double* s, double dx, int N) {
    for (int k = 1; k <= N - 1; ++k) {
        double sum = 0.0;
        for (int j = 1; j <= N - 1; ++j) sum += s[j] * sin(k * M_PI * j / ((double)N));
        S[k] = dx * sum;
    }
}

/* ------------------------------------------------------------------ */
/* LaplCube (Dirichlet)                                                */
/* ------------------------------------------------------------------ */

/* Dirichlet eigenvalues 4/h^2 sin^2(j pi / (2(n+1))), j=1..n, at [j];
 * src/lapl_cube.cpp:145-172. */
static double* dirichlet_lm(int n, double h) {
    double* lm = (double*)calloc(n + 1, sizeof(double));
    const double h2 = h * h;
    for (int j = 1; j <= n; j++) lm[j] = 4. / h2 * sqd(sin(j * M_PI * 0.5 / (n + 1)));
    return lm;
}

/* Applies the DST along one axis of an nz*ny*nx array for every line.
 * axis 0 = x (stride 1), 1 = y (stride nx), 2 = z (stride nx*ny).
 * Restates one of the six line loops of src/lapl_cube.cpp:13-141: gather the
 * line into s[1..n], transform, scatter S[1..n]. */
static void dst_axis(const sn_table* t, int nx, int ny, int nz, int axis, double scale,
                     const double* in, double* out) {
    const int n = axis == 0 ? nx : axis == 1 ? ny : nz;
    const long stride = axis == 0 ? 1 : axis == 1 ? nx : (long)nx * ny;
    const long lines = (long)nx * ny * nz / n;
    const int N = t->N;
#pragma omp parallel num_threads(orc_get_threads())
    {
        double* s = (double*)calloc(N + 1, sizeof(double));
        double* S = (double*)calloc(N + 1, sizeof(double));
        double* b = (double*)calloc(N, sizeof(double));
        double* bn = (double*)calloc(N, sizeof(double));
#pragma omp for schedule(static)
        for (long L = 0; L < lines; L++) {
            long base;
            if (axis == 0) base = L * nx;
            else if (axis == 1) base = (L / nx) * (long)nx * ny + (L % nx);
            else base = L;
            for (int i = 1; i <= n; i++) s[i] = in[base + (i - 1) * stride];
            sn_sine(t, S, s, scale, b, bn);
            for (int i = 1; i <= n; i++) out[base + (i - 1) * stride] = S[i];
        }
        free(s); free(S); free(b); free(bn);
    }
}

int orc_lapl_cube_solve(int nx, int ny, int nz, double dx, double dy, double dz,
                        double lx, double ly, double lz, double* ans, const double* rhs) {
    sn_table tx, ty, tz;
    if (log2_exact(nx + 1) < 0 || log2_exact(ny + 1) < 0 || log2_exact(nz + 1) < 0) return -1;
    sn_table_init(&tx, nx + 1);
    sn_table_init(&ty, ny + 1);
    sn_table_init(&tz, nz + 1);
    const double slx = sqrt(2. / lx), sly = sqrt(2. / ly), slz = sqrt(2. / lz);
    /* The reference shares lm_y for x (resp. z) whenever the point counts are
     * equal, whatever the spacings (src/lapl_cube.cpp:165, :171). */
    double* lmy = dirichlet_lm(ny, dy);
    double* lmx_own = dirichlet_lm(nx, dx);
    double* lmz_own = dirichlet_lm(nz, dz);
    const double* lmx = (nx == ny) ? lmy : lmx_own;
    const double* lmz = (nz == ny) ? lmy : lmz_own;
    const long total = (long)nx * ny * nz;
    double* w = (double*)malloc(sizeof(double) * total);

    dst_axis(&tz, nx, ny, nz, 2, dz * slz, rhs, w);
    dst_axis(&ty, nx, ny, nz, 1, dy * sly, w, w);
    dst_axis(&tx, nx, ny, nz, 0, dx * slx, w, w);
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
    for (int i = 1; i <= nz; i++)
        for (int k = 1; k <= ny; k++)
            for (int j = 1; j <= nx; j++) {
                double k2 = lmz[i] + lmy[k] + lmx[j];
                w[((long)(i - 1) * ny + (k - 1)) * nx + (j - 1)] /= -k2;
            }
    dst_axis(&tx, nx, ny, nz, 0, slx, w, ans);
    dst_axis(&ty, nx, ny, nz, 1, sly, ans, ans);
    dst_axis(&tz, nx, ny, nz, 2, slz, ans, ans);

    free(w);
    free(lmy); free(lmx_own); free(lmz_own);
    sn_table_free(&tx); sn_table_free(&ty); sn_table_free(&tz);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Tridiagonal solvers                                                 */
/* ------------------------------------------------------------------ */

void orc_thomas(double* B, double* A1, double* A2, double* A3, int n) {
    for (int j = 0; j < n - 1; j++) {
        double a = A1[j] / A2[j];
        A1[j] = 0;
        A2[j + 1] -= A3[j] * a;
        B[j + 1] -= B[j] * a;
    }
    for (int j = n - 1; j > 0; j--) {
        double a = A3[j - 1] / A2[j];
        B[j - 1] -= B[j] * a;
    }
    for (int i = 0; i < n; i++) B[i] *= 1 / (A2[i]);
}

void orc_cyclic_reduction(double* d, double* e, double* f, double* b, int q, int n, int general) {
    int l, j, s, h;
    double alpha, gamma;
    if (!general) {
        for (l = 1; l < q; l++) {
            s = 1 << l;
            h = 1 << (l - 1);
            for (j = s - 1; j < n - h; j += s) {
                alpha = -e[j] / d[j - h];
                gamma = -f[j] / d[j + h];
                d[j] += alpha * f[j - h] + gamma * e[j + h];
                b[j] += alpha * b[j - h] + gamma * b[j + h];
                e[j] = alpha * e[j - h];
                f[j] = gamma * f[j + h];
            }
        }
        j = (1 << (q - 1)) - 1;
        b[j] = b[j] / d[j];
        for (l = q - 1; l > 0; l--) {
            s = 1 << l;
            h = 1 << (l - 1);
            j = h - 1;
            b[j] = (b[j] - f[j] * b[j + h]) / d[j];
            for (j = h + s - 1; j < n - h; j += s) b[j] = (b[j] - e[j] * b[j - h] - f[j] * b[j + h]) / d[j];
            b[j] = (b[j] - e[j] * b[j - h]) / d[j];
        }
        return;
    }
    for (l = 1; l < q; l++) {
        s = 1 << l;
        h = 1 << (l - 1);
        for (j = s - 1; j + h < n; j += s) {
            alpha = -e[j] / d[j - h];
            gamma = -f[j] / d[j + h];
            d[j] += alpha * f[j - h] + gamma * e[j + h];
            b[j] += alpha * b[j - h] + gamma * b[j + h];
            e[j] = alpha * e[j - h];
            f[j] = gamma * f[j + h];
        }
        for (; j < n; j += s) {
            alpha = -e[j] / d[j - h];
            d[j] += alpha * f[j - h];
            b[j] += alpha * b[j - h];
            e[j] = alpha * e[j - h];
        }
    }
    j = (1 << (q - 1)) - 1;
    if (j > n - 1) j = n - 1;
    b[j] /= d[j];
    for (l = q - 1; l > 0; l--) {
        s = 1 << l;
        h = 1 << (l - 1);
        for (j = h - 1; j - h < 0; j += s) b[j] = (b[j] - f[j] * b[j + h]) / d[j];
        for (; j + h < n; j += s) b[j] = (b[j] - e[j] * b[j - h] - f[j] * b[j + h]) / d[j];
        for (; j < n; j += s) b[j] = (b[j] - e[j] * b[j - h]) / d[j];
    }
}

/* ------------------------------------------------------------------ */
/* LaplRect / LaplRectFFT2 (Dirichlet)                                 */
/* ------------------------------------------------------------------ */

/* Column DST of an ny*nx array (x fastest) for every x, as the loops of
 * src/lapl_rect.cpp:68-83 / :94-109. */
static void rect_dst_y(const sn_table* t, int nx, int ny, double scale, const double* in, double* out) {
    dst_axis(t, nx, ny, 1, 1, scale, in, out);
}

int orc_lapl_rect_solve(int nx, int ny, double dx, double dy, double lx, double ly,
                        double* ans, const double* rhs) {
    sn_table ty;
    (void)lx;
    if (log2_exact(ny + 1) < 0) return -1;
    sn_table_init(&ty, ny + 1);
    const double sly = sqrt(2. / ly), dx2 = dx * dx;
    double* lmy = dirichlet_lm(ny, dy);
    double* w = (double*)malloc(sizeof(double) * (long)nx * ny);
    rect_dst_y(&ty, nx, ny, dy * sly, rhs, w);
    /* per y-mode: tridiagonal along x, L=U=1/dx^2, D=-2/dx^2-lm_y[k]
     * (src/lapl_rect.cpp:44-61, :85-92); LAPACK gtsv equals the no-pivot
     * Thomas solve on these diagonally dominant matrices. */
#pragma omp parallel num_threads(orc_get_threads())
    {
        double* L = (double*)malloc(sizeof(double) * nx);
        double* D = (double*)malloc(sizeof(double) * nx);
        double* U = (double*)malloc(sizeof(double) * nx);
#pragma omp for schedule(static)
        for (int k = 1; k <= ny; k++) {
            for (int j = 1; j <= nx; j++) {
                D[j - 1] = -2 / dx2 - lmy[k] * 1.0;
                if (j < nx) { L[j - 1] = 1.0 / dx2; U[j - 1] = 1.0 / dx2; }
            }
            orc_thomas(&w[(long)(k - 1) * nx], L, D, U, nx);
        }
        free(L); free(D); free(U);
    }
    rect_dst_y(&ty, nx, ny, sly, w, ans);
    free(w);
    free(lmy);
    sn_table_free(&ty);
    return 0;
}

int orc_lapl_rect_fft2_solve(int nx, int ny, double dx, double dy, double lx, double ly,
                             double* ans, const double* rhs) {
    sn_table tx, ty;
    if (log2_exact(ny + 1) < 0 || log2_exact(nx + 1) < 0) return -1;
    sn_table_init(&tx, nx + 1);
    sn_table_init(&ty, ny + 1);
    const double slx = sqrt(2. / lx), sly = sqrt(2. / ly);
    double* lmy = dirichlet_lm(ny, dy);
    double* lmx_own = dirichlet_lm(nx, dx);
    const double* lmx = (nx == ny) ? lmy : lmx_own; /* src/lapl_rect.cpp:40 */
    double* w = (double*)malloc(sizeof(double) * (long)nx * ny);
    rect_dst_y(&ty, nx, ny, dy * sly, rhs, w);
    dst_axis(&tx, nx, ny, 1, 0, dx * slx, w, w);
    for (int k = 1; k <= ny; k++)
        for (int j = 1; j <= nx; j++) w[(long)(k - 1) * nx + (j - 1)] /= -lmy[k] * 1.0 - lmx[j];
    dst_axis(&tx, nx, ny, 1, 0, slx, w, ans);
    rect_dst_y(&ty, nx, ny, sly, ans, ans);
    free(w);
    free(lmy); free(lmx_own);
    sn_table_free(&tx); sn_table_free(&ty);
    return 0;
}

/* ------------------------------------------------------------------ */
/* NSCube                                                              */
/* ------------------------------------------------------------------ */

/* A reference tensor: inclusive index ranges per axis, row-major, x
 * fastest (src/tensor.h:192-219). */
typedef struct {
    int z1, z2, y1, y2, x1, x2;
    long sy, sz, size;
    double* v;
} t3;

static void t3_init(t3* t, int z1, int z2, int y1, int y2, int x1, int x2) {
    t->z1 = z1; t->z2 = z2; t->y1 = y1; t->y2 = y2; t->x1 = x1; t->x2 = x2;
    t->sy = x2 - x1 + 1;
    t->sz = t->sy * (y2 - y1 + 1);
    t->size = t->sz * (z2 - z1 + 1);
    t->v = (double*)calloc(t->size, sizeof(double));
}

#define AT(t, i, k, j) ((t).v[((long)(i) - (t).z1) * (t).sz + ((long)(k) - (t).y1) * (t).sy + ((j) - (t).x1)])

struct orc_nscube {
    double x1, y1, z1, x2, y2, z2, U0, Re, dt;
    int nx, ny, nz;
    double dx, dy, dz, dx2, dy2, dz2;
    t3 u, v, w, p, x, F, G, H, RHS;
    int time_index;
};

orc_nscube* orc_ns_create(int nx, int nz, double Re, double dt, double u0,
                          double x1, double y1, double z1, double x2, double y2, double z2) {
    if (log2_exact(nx + 1) < 0 || log2_exact(nz + 1) < 0) return NULL;
    orc_nscube* s = (orc_nscube*)calloc(1, sizeof(orc_nscube));
    s->x1 = x1; s->y1 = y1; s->z1 = z1; s->x2 = x2; s->y2 = y2; s->z2 = z2;
    s->U0 = u0; s->Re = Re; s->dt = dt;
    s->nx = nx; s->ny = nx; s->nz = nz;
    s->dx = (x2 - x1) / s->nx; s->dy = (y2 - y1) / s->ny; s->dz = (z2 - z1) / s->nz;
    s->dx2 = s->dx * s->dx; s->dy2 = s->dy * s->dy; s->dz2 = s->dz * s->dz;
    const int NX = s->nx, NY = s->ny, NZ = s->nz;
    t3_init(&s->u, 0, NZ + 1, 0, NY + 1, -1, NX + 1);
    t3_init(&s->v, 0, NZ + 1, -1, NY + 1, 0, NX + 1);
    t3_init(&s->w, -1, NZ + 1, 0, NY + 1, 0, NX + 1);
    t3_init(&s->p, 0, NZ + 1, 0, NY + 1, 0, NX + 1);
    t3_init(&s->x, 1, NZ, 1, NY, 1, NX);
    t3_init(&s->F, 1, NZ, 1, NY, 0, NX);
    t3_init(&s->G, 1, NZ, 0, NY, 1, NX);
    t3_init(&s->H, 0, NZ, 1, NY, 1, NX);
    t3_init(&s->RHS, 1, NZ, 1, NY, 1, NX);
    return s;
}

/* src/ns_cube.cpp:65-122 */
static void ns_init_bound(orc_nscube* s) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const double U0 = s->U0, Re = s->Re, dx = s->dx, dy = s->dy, dz = s->dz;
    for (int k = 0; k <= ny + 1; k++)
        for (int j = -1; j <= nz + 1; j++) AT(s->u, nz + 1, k, j) = 2 * U0 - AT(s->u, nz, k, j);
    for (int i = 0; i <= nz + 1; i++)
        for (int k = 0; k <= ny + 1; k++) {
            AT(s->u, i, k, -1) = AT(s->u, i, k, 1);
            AT(s->u, i, k, nx + 1) = AT(s->u, i, k, nx - 1);
        }
    for (int i = 0; i <= nz + 1; i++)
        for (int j = 0; j <= nx + 1; j++) {
            AT(s->v, i, -1, j) = AT(s->v, i, 1, j);
            AT(s->v, i, ny + 1, j) = AT(s->v, i, ny - 1, j);
        }
    for (int k = 0; k <= ny + 1; k++)
        for (int j = 0; j <= nx + 1; j++) {
            AT(s->w, -1, k, j) = AT(s->w, 1, k, j);
            AT(s->w, nz + 1, k, j) = AT(s->w, nz - 1, k, j);
        }
    for (int i = 1; i <= nz; i++)
        for (int k = 1; k <= ny; k++) {
            AT(s->p, i, k, 0) = AT(s->p, i, k, 1) -
                (AT(s->u, i, k, 1) - 2 * AT(s->u, i, k, 0) + AT(s->u, i, k, -1)) / Re / dx;
            AT(s->p, i, k, nx + 1) = AT(s->p, i, k, nx) -
                (AT(s->u, i, k, nx + 1) - 2 * AT(s->u, i, k, nx) + AT(s->u, i, k, nx - 1)) / Re / dx;
        }
    for (int i = 1; i <= nz; i++)
        for (int j = 1; j <= nx; j++) {
            AT(s->p, i, 0, j) = AT(s->p, i, 1, j) -
                (AT(s->v, i, 1, j) - 2 * AT(s->v, i, 0, j) + AT(s->v, i, -1, j)) / Re / dy;
            AT(s->p, i, ny + 1, j) = AT(s->p, i, ny, j) -
                (AT(s->v, i, ny + 1, j) - 2 * AT(s->v, i, ny, j) + AT(s->v, i, ny - 1, j)) / Re / dy;
        }
    for (int k = 1; k <= ny; k++)
        for (int j = 1; j <= nx; j++) {
            AT(s->p, 0, k, j) = AT(s->p, 1, k, j) -
                (AT(s->w, 1, k, j) - 2 * AT(s->w, 0, k, j) + AT(s->w, -1, k, j)) / Re / dz;
            AT(s->p, nz + 1, k, j) = AT(s->p, nz, k, j) -
                (AT(s->w, nz + 1, k, j) - 2 * AT(s->w, nz, k, j) + AT(s->w, nz - 1, k, j)) / Re / dz;
        }
}

/* src/ns_cube.cpp:126-200 (Fletcher eqs 17.9 / 17.11) */
static void ns_fgh(orc_nscube* s) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const double Re = s->Re, dt = s->dt, dx = s->dx, dy = s->dy, dz = s->dz;
    const double dx2 = s->dx2, dy2 = s->dy2, dz2 = s->dz2;
    t3 u = s->u, v = s->v, w = s->w;
#pragma omp parallel num_threads(orc_get_threads())
    {
#pragma omp for collapse(2) schedule(static)
        for (int i = 1; i <= nz; i++)
            for (int k = 1; k <= ny; k++)
                for (int j = 0; j <= nx; j++) {
                    AT(s->F, i, k, j) = AT(u, i, k, j) + dt * (
                        (AT(u, i, k, j + 1) - 2 * AT(u, i, k, j) + AT(u, i, k, j - 1)) / Re / dx2 +
                        (AT(u, i, k + 1, j) - 2 * AT(u, i, k, j) + AT(u, i, k - 1, j)) / Re / dy2 +
                        (AT(u, i + 1, k, j) - 2 * AT(u, i, k, j) + AT(u, i - 1, k, j)) / Re / dz2 -
                        (sqd(0.5 * (AT(u, i, k, j) + AT(u, i, k, j + 1))) - sqd(0.5 * (AT(u, i, k, j - 1) + AT(u, i, k, j)))) / dx -
                        0.25 * ((AT(u, i, k, j) + AT(u, i, k + 1, j)) * (AT(v, i, k, j + 1) + AT(v, i, k, j)) -
                                (AT(u, i, k - 1, j) + AT(u, i, k, j)) * (AT(v, i, k - 1, j + 1) + AT(v, i, k - 1, j))) / dy -
                        0.25 * ((AT(u, i, k, j) + AT(u, i + 1, k, j)) * (AT(w, i, k, j + 1) + AT(w, i, k, j)) -
                                (AT(u, i - 1, k, j) + AT(u, i, k, j)) * (AT(w, i - 1, k, j + 1) + AT(w, i - 1, k, j))) / dz);
                }
#pragma omp for collapse(2) schedule(static)
        for (int i = 1; i <= nz; i++)
            for (int k = 0; k <= ny; k++)
                for (int j = 1; j <= nx; j++) {
                    AT(s->G, i, k, j) = AT(v, i, k, j) + dt * (
                        (AT(v, i, k, j + 1) - 2 * AT(v, i, k, j) + AT(v, i, k, j - 1)) / Re / dx2 +
                        (AT(v, i, k + 1, j) - 2 * AT(v, i, k, j) + AT(v, i, k - 1, j)) / Re / dy2 +
                        (AT(v, i + 1, k, j) - 2 * AT(v, i, k, j) + AT(v, i - 1, k, j)) / Re / dz2 -
                        (sqd(0.5 * (AT(v, i, k, j) + AT(v, i, k + 1, j))) - sqd(0.5 * (AT(v, i, k - 1, j) + AT(v, i, k, j)))) / dy -
                        0.25 * ((AT(u, i, k, j) + AT(u, i, k + 1, j)) * (AT(v, i, k, j + 1) + AT(v, i, k, j)) -
                                (AT(u, i, k, j - 1) + AT(u, i, k + 1, j - 1)) * (AT(v, i, k, j) + AT(v, i, k, j - 1))) / dx -
                        0.25 * ((AT(w, i, k, j) + AT(w, i, k + 1, j)) * (AT(v, i, k, j) + AT(v, i + 1, k, j)) -
                                (AT(w, i - 1, k, j) + AT(w, i - 1, k + 1, j)) * (AT(v, i - 1, k, j) + AT(v, i, k, j))) / dz);
                }
#pragma omp for collapse(2) schedule(static)
        for (int i = 0; i <= nz; i++)
            for (int k = 1; k <= ny; k++)
                for (int j = 1; j <= nx; j++) {
                    AT(s->H, i, k, j) = AT(w, i, k, j) + dt * (
                        (AT(w, i, k, j + 1) - 2 * AT(w, i, k, j) + AT(w, i, k, j - 1)) / Re / dx2 +
                        (AT(w, i, k + 1, j) - 2 * AT(w, i, k, j) + AT(w, i, k - 1, j)) / Re / dy2 +
                        (AT(w, i + 1, k, j) - 2 * AT(w, i, k, j) + AT(w, i - 1, k, j)) / Re / dz2 -
                        (sqd(0.5 * (AT(w, i + 1, k, j) + AT(w, i, k, j))) - sqd(0.5 * (AT(w, i - 1, k, j) + AT(w, i, k, j)))) / dz -
                        0.25 * ((AT(u, i + 1, k, j) + AT(u, i, k, j)) * (AT(w, i, k, j + 1) + AT(w, i, k, j)) -
                                (AT(u, i + 1, k, j - 1) + AT(u, i, k, j - 1)) * (AT(w, i, k, j) + AT(w, i, k, j - 1))) / dx -
                        0.25 * ((AT(w, i, k, j) + AT(w, i, k + 1, j)) * (AT(v, i, k, j) + AT(v, i + 1, k, j)) -
                                (AT(w, i, k - 1, j) + AT(w, i, k, j)) * (AT(v, i, k - 1, j) + AT(v, i + 1, k - 1, j))) / dy);
                }
    }
}

/* src/ns_cube.cpp:204-238 */
static void ns_poisson(orc_nscube* s) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const double dt = s->dt, dx = s->dx, dy = s->dy, dz = s->dz;
    const double dx2 = s->dx2, dy2 = s->dy2, dz2 = s->dz2;
#pragma omp parallel for collapse(2) num_threads(orc_get_threads())
    for (int i = 1; i <= nz; i++)
        for (int k = 1; k <= ny; k++)
            for (int j = 1; j <= nx; j++) {
                double r = ((AT(s->F, i, k, j) - AT(s->F, i, k, j - 1)) / dx +
                            (AT(s->G, i, k, j) - AT(s->G, i, k - 1, j)) / dy +
                            (AT(s->H, i, k, j) - AT(s->H, i - 1, k, j)) / dz) / dt;
                if (i <= 1) r -= AT(s->p, i - 1, k, j) / dz2;
                if (k <= 1) r -= AT(s->p, i, k - 1, j) / dy2;
                if (j <= 1) r -= AT(s->p, i, k, j - 1) / dx2;
                if (j >= nx) r -= AT(s->p, i, k, j + 1) / dx2;
                if (k >= ny) r -= AT(s->p, i, k + 1, j) / dy2;
                if (i >= nz) r -= AT(s->p, i + 1, k, j) / dz2;
                AT(s->RHS, i, k, j) = r;
            }
    orc_lapl_cube_solve(nx, ny, nz, dx, dy, dz, s->x2 - s->x1 + dx, s->y2 - s->y1 + dy,
                        s->z2 - s->z1 + dz, s->x.v, s->RHS.v);
}

/* src/ns_cube.cpp:241-277 */
static void ns_update(orc_nscube* s) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const double dt = s->dt, dx = s->dx, dy = s->dy, dz = s->dz;
#pragma omp parallel num_threads(orc_get_threads())
    {
#pragma omp for collapse(2) schedule(static)
        for (int i = 1; i <= nz; i++)
            for (int k = 1; k <= ny; k++)
                for (int j = 1; j < nx; j++)
                    AT(s->u, i, k, j) = AT(s->F, i, k, j) - dt / dx * (AT(s->x, i, k, j + 1) - AT(s->x, i, k, j));
#pragma omp for collapse(2) schedule(static)
        for (int i = 1; i <= nz; i++)
            for (int k = 1; k < ny; k++)
                for (int j = 1; j <= nx; j++)
                    AT(s->v, i, k, j) = AT(s->G, i, k, j) - dt / dy * (AT(s->x, i, k + 1, j) - AT(s->x, i, k, j));
#pragma omp for collapse(2) schedule(static)
        for (int i = 1; i < nz; i++)
            for (int k = 1; k <= ny; k++)
                for (int j = 1; j <= nx; j++)
                    AT(s->w, i, k, j) = AT(s->H, i, k, j) - dt / dz * (AT(s->x, i + 1, k, j) - AT(s->x, i, k, j));
    }
    /* p = x over the overlapping index range (src/tensor.h:280-283) */
    for (int i = 1; i <= nz; i++)
        for (int k = 1; k <= ny; k++)
            for (int j = 1; j <= nx; j++) AT(s->p, i, k, j) = AT(s->x, i, k, j);
}

void orc_ns_step(orc_nscube* s, int k) {
    for (int it = 0; it < k; it++) {
        ns_init_bound(s);
        ns_fgh(s);
        ns_poisson(s);
        ns_update(s);
        s->time_index++;
    }
}

static t3* ns_field(const orc_nscube* s, int f) {
    orc_nscube* m = (orc_nscube*)s;
    switch (f) {
        case 0: return &m->u;
        case 1: return &m->v;
        case 2: return &m->w;
        case 3: return &m->p;
        case 4: return &m->x;
        case 5: return &m->F;
        case 6: return &m->G;
        case 7: return &m->H;
        case 8: return &m->RHS;
        default: return NULL;
    }
}

long orc_ns_get(const orc_nscube* s, int field, double* out) {
    t3* t = ns_field(s, field);
    if (!t) return -1;
    if (out) memcpy(out, t->v, sizeof(double) * t->size);
    return t->size;
}

int orc_ns_set(orc_nscube* s, int field, const double* in) {
    t3* t = ns_field(s, field);
    if (!t) return -1;
    memcpy(t->v, in, sizeof(double) * t->size);
    return 0;
}

void orc_ns_destroy(orc_nscube* s) {
    if (!s) return;
    t3* f[] = {&s->u, &s->v, &s->w, &s->p, &s->x, &s->F, &s->G, &s->H, &s->RHS};
    for (int i = 0; i < 9; i++) free(f[i]->v);
    free(s);
}
