// Test infrastructure, not product code.
//
// C-ABI harness around the reference fdm library's own CPU classes, compiled
// together with the reference sources (see oracle/Makefile) into
// oracle/_ref/libfdm_ref.so.  Only the tests, the golden-fixture generator and
// bench.py's CPU-baseline leg load it, and only as the checker or the timed
// CPU baseline.
//
// Wrapped reference interfaces:
//   fdm::LaplCube<T,false,F>::solve      src/lapl_cube.h:58-102, src/lapl_cube.cpp:9-142
//   fdm::LaplRect<T,false>::solve        src/lapl_rect.h:40-68,  src/lapl_rect.cpp:63-110
//   fdm::LaplRectFFT2<T,false>::solve    src/lapl_rect.h:89-105, src/lapl_rect.cpp:113-207
//   fdm::FFT<T>::sFFT                    src/fft.h:45-98,        src/fft.cpp:294-365
//   fdm::cyclic_reduction(_general)      src/cyclic_reduction.h:20-107
//   solve_tdiag_linear_my                src/asp_gauss.cpp:185-207
//   fdm::NSCube<T,false>                 src/ns_cube.h:14-92,    src/ns_cube.cpp:27-277
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lapl_cube.h"
#include "lapl_rect.h"
#include "ns_cube.h"
#include "lapl_cyl.h"
#include "ns_cyl.h"
#include "cyclic_reduction.h"
#include "asp_gauss.h"
#include "config.h"

using namespace fdm;

// LAPACK ?gtsv_ is referenced by LaplRect::solve (src/blas.h:14,72-75) but no
// LAPACK exists in this build.  The matrices LaplRect builds are strictly
// diagonally dominant (|D| = 2/dx^2 + lambda > 2/dx^2 = |L|+|U|), so partial
// pivoting never swaps rows and elimination without pivoting gives the same
// factorisation.  The adapter therefore calls the reference's own no-pivot
// Thomas solver, solve_tdiag_linear_my (src/asp_gauss.cpp:185-207), whose
// argument convention (sub, diag, super) equals LAPACK's (DL, D, DU).
extern "C" void dgtsv_(int* n, int* nrhs, double* dl, double* d, double* du,
                       double* b, int* ldb, int* info) {
    *info = 0;
    if (*nrhs != 1) { *info = -2; return; }
    solve_tdiag_linear_my(b, dl, d, du, *n);
}
extern "C" void sgtsv_(int* n, int* nrhs, float* dl, float* d, float* du,
                       float* b, int* ldb, int* info) {
    *info = 0;
    if (*nrhs != 1) { *info = -2; return; }
    solve_tdiag_linearf_my(b, dl, d, du, *n);
}

// LAPACK ?gttrf_ / ?gttrs_ (LU of a tridiagonal matrix, then solves) are
// referenced by LaplCyl3FFT2 (src/lapl_cyl.cpp:75-82, 150-166;
// src/blas.h:17-22).  Its radial matrices are diagonally dominant
// (|D| = 2/dr^2 + lm_phi/r^2 + lm_z >= |L| + |U| = 2/dr^2 in the interior,
// strictly in the first and last rows), so LAPACK's partial pivoting, which
// swaps only when |dl(i)| > |d(i)|, never swaps; the adapters perform that
// no-swap elimination: multipliers in dl, updated pivots in d, du2 = 0,
// ipiv(i) = i.
template <typename T>
static void gttrf_noswap(int n, T* dl, T* d, T* du, T* du2, int* ipiv) {
    for (int i = 0; i < n; i++) ipiv[i] = i + 1;
    for (int i = 0; i + 2 < n; i++) du2[i] = 0;
    for (int i = 0; i + 1 < n; i++) {
        const T fact = dl[i] / d[i];
        dl[i] = fact;
        d[i + 1] -= fact * du[i];
    }
}
template <typename T>
static void gttrs_noswap(int n, const T* dl, const T* d, const T* du, T* b) {
    for (int i = 0; i + 1 < n; i++) b[i + 1] -= dl[i] * b[i];
    b[n - 1] /= d[n - 1];
    if (n > 1) b[n - 2] = (b[n - 2] - du[n - 2] * b[n - 1]) / d[n - 2];
    for (int i = n - 3; i >= 0; i--) b[i] = (b[i] - du[i] * b[i + 1]) / d[i];
}
extern "C" void dgttrf_(int* n, double* dl, double* d, double* du, double* du2, int* ipiv, int* info) {
    *info = 0;
    gttrf_noswap(*n, dl, d, du, du2, ipiv);
}
extern "C" void sgttrf_(int* n, float* dl, float* d, float* du, float* du2, int* ipiv, int* info) {
    *info = 0;
    gttrf_noswap(*n, dl, d, du, du2, ipiv);
}
extern "C" void dgttrs_(const char*, int* n, int* nrhs, double* dl, double* d, double* du, double*, int*,
                        double* b, int*, int* info) {
    *info = *nrhs == 1 ? 0 : -3;
    if (!*info) gttrs_noswap(*n, dl, d, du, b);
}
extern "C" void sgttrs_(const char*, int* n, int* nrhs, float* dl, float* d, float* du, float*, int*,
                        float* b, int*, int* info) {
    *info = *nrhs == 1 ? 0 : -3;
    if (!*info) gttrs_noswap(*n, dl, d, du, b);
}

namespace {
using periodic3 = tensor_flags<tensor_flag::periodic, tensor_flag::periodic, tensor_flag::periodic>;

template <typename T, typename F>
void cube_solve(int nx, int ny, int nz, double dx, double dy, double dz,
                double lx, double ly, double lz, T* ans, const T* rhs, int reps) {
    LaplCube<T, false, F> lapl(dx, dy, dz, lx, ly, lz, nx, ny, nz);
    std::vector<T> r(rhs, rhs + (size_t)nx * ny * nz);
    for (int i = 0; i < reps; i++) lapl.solve(ans, r.data());
}
}  // namespace

extern "C" {

int ref_lapl_cube_solve_d(int nx, int ny, int nz, double dx, double dy, double dz,
                          double lx, double ly, double lz, int periodic,
                          double* ans, const double* rhs, int reps) {
    if (periodic) cube_solve<double, periodic3>(nx, ny, nz, dx, dy, dz, lx, ly, lz, ans, rhs, reps);
    else cube_solve<double, tensor_flags<>>(nx, ny, nz, dx, dy, dz, lx, ly, lz, ans, rhs, reps);
    return 0;
}

int ref_lapl_cube_solve_f(int nx, int ny, int nz, double dx, double dy, double dz,
                          double lx, double ly, double lz, int periodic,
                          float* ans, const float* rhs, int reps) {
    if (periodic) cube_solve<float, periodic3>(nx, ny, nz, dx, dy, dz, lx, ly, lz, ans, rhs, reps);
    else cube_solve<float, tensor_flags<>>(nx, ny, nz, dx, dy, dz, lx, ly, lz, ans, rhs, reps);
    return 0;
}

int ref_lapl_rect_solve_d(int nx, int ny, double dx, double dy, double lx, double ly,
                          int fft2, double* ans, const double* rhs) {
    std::vector<double> r(rhs, rhs + (size_t)nx * ny);
    if (fft2) {
        LaplRectFFT2<double, false> l(dx, dy, lx, ly, nx, ny);
        l.solve(ans, r.data());
    } else {
        LaplRect<double, false> l(dx, dy, lx, ly, nx, ny);
        l.solve(ans, r.data());
    }
    return 0;
}

// LaplRect / LaplRectFFT2 with periodic flags (src/lapl_rect.cpp:209-238):
// flags bit 1 = y periodic (F::head), bit 0 = x periodic (F::tail::head);
// the instantiated sets are 2 (y) and 3 (y and x).  Arrays are the
// {y1..yn, x1..xn} ranges: ny rows for periodic y, nx columns for periodic x.
}  // extern "C"

template <typename F>
static void rect_flags(int nx, int ny, double dx, double dy, double lx, double ly, int fft2, double* ans,
                       const double* rhs) {
    std::vector<double> r(rhs, rhs + (size_t)nx * ny);
    if (fft2) {
        LaplRectFFT2<double, false, F> l(dx, dy, lx, ly, nx, ny);
        l.solve(ans, r.data());
    } else {
        LaplRect<double, false, F> l(dx, dy, lx, ly, nx, ny);
        l.solve(ans, r.data());
    }
}

extern "C" {

int ref_lapl_rect_flags_d(int nx, int ny, double dx, double dy, double lx, double ly, int fft2, int flags,
                          double* ans, const double* rhs) {
    using P1 = tensor_flags<tensor_flag::periodic>;
    using P2 = tensor_flags<tensor_flag::periodic, tensor_flag::periodic>;
    if (flags == 2) rect_flags<P1>(nx, ny, dx, dy, lx, ly, fft2, ans, rhs);
    else if (flags == 3) rect_flags<P2>(nx, ny, dx, dy, lx, ly, fft2, ans, rhs);
    else return -1;
    return 0;
}

// S[1..N-1] = dx * sum_{j=1}^{N-1} s[j] sin(pi j k / N); s is overwritten.
int ref_sfft_d(double* S, double* s, double dx, int N) {
    FFTTable<double> t(N);
    FFT<double> ft(t, N);
    ft.sFFT(S, s, dx);
    return 0;
}
int ref_sfft_f(float* S, float* s, float dx, int N) {
    FFTTable<float> t(N);
    FFT<float> ft(t, N);
    ft.sFFT(S, s, dx);
    return 0;
}

// Periodic real transforms of the reference: values -> coefficients
// (FFT<T>::pFFT_1, src/fft.cpp:108-194) and back (FFT<T>::pFFT,
// src/fft.cpp:195-212).  Both overwrite their input.
int ref_pfft1_d(double* S, double* s, double dx, int N) {
    FFTTable<double> t(N);
    FFT<double> ft(t, N);
    ft.pFFT_1(S, s, dx);
    return 0;
}
int ref_pfft_d(double* S, double* s, double dx, int N) {
    FFTTable<double> t(N);
    FFT<double> ft(t, N);
    ft.pFFT(S, s, dx);
    return 0;
}
// FFT<double>::pFFT_1_3d / pFFT_3d (src/fft.cpp:214-292) of an N^3 cube
int ref_pfft3d_d(double* S, double* s, double dx, int N, int inverse) {
    FFTTable<double> t(N);
    FFT<double> ft(t, N);
    if (inverse) ft.pFFT_3d(S, s, dx);
    else ft.pFFT_1_3d(S, s, dx);
    return 0;
}

// Periodic LaplCube<double,false,periodic^3> (src/lapl_cube.h:9-106 with
// F = tensor_flags<periodic,periodic,periodic>): rhs/ans hold n_z*n_y*n_x
// points, x fastest, as the reference's periodic test passes them
// (ut/ut_lapl_cube.cpp:156-243: &RHS[0][0][0] of a {0..n-1}^3 tensor).
int ref_lapl_cube_periodic_d(int nx, int ny, int nz, double dx, double dy, double dz, double lx, double ly,
                             double lz, double* ans, double* rhs) {
    using F = tensor_flags<tensor_flag::periodic, tensor_flag::periodic, tensor_flag::periodic>;
    LaplCube<double, false, F> lapl(dx, dy, dz, lx, ly, lz, nx, ny, nz);
    lapl.solve(ans, rhs);
    return 0;
}

// LaplCyl3FFT2<double,false,zflag> (src/lapl_cyl.h:178-262,
// src/lapl_cyl.cpp:10-166): arrays of nphi x nz' x nr points (r fastest;
// nz' = nz Dirichlet, nz periodic), as the tensor {0..nphi-1, z1..zn, 1..nr}.
int ref_lapl_cyl_d(int periodic_z, int nr, int nz, int nphi, double dr, double dz, double r0, double lr,
                   double lz, double* ans, double* rhs) {
    if (periodic_z) {
        LaplCyl3FFT2<double, false, tensor_flag::periodic> lapl(dr, dz, r0, lr, lz, nr, nz, nphi);
        lapl.solve(ans, rhs);
    } else {
        LaplCyl3FFT2<double, false, tensor_flag::none> lapl(dr, dz, r0, lr, lz, nr, nz, nphi);
        lapl.solve(ans, rhs);
    }
    return 0;
}

// NSCyl<double,false,zflag> (src/ns_cyl.h:18-134) from ns:{R,r,h1,h2,u0,Re,dt,
// nr,nz,nphi}; fields copied out whole (ghosts included), layout of the
// reference tensor (phi, z, r), r fastest.
struct RefNSCyl {
    Config cfg;
    NSCyl<double, false, tensor_flag::none>* d = nullptr;
    NSCyl<double, false, tensor_flag::periodic>* p = nullptr;
};

// ns:vrandom=1 when vrandom != 0 (the constructor's random v perturbation,
// src/ns_cyl.h:99-109)
void* ref_nscyl_create_v(int periodic_z, double R, double r0, double h1, double h2, double u0, double Re, double dt,
                         int nr, int nz, int nphi, int vrandom) {
    auto* h = new RefNSCyl();
    char buf[16][96];
    const char* keys[] = {"nr", "nz", "nphi", "R", "r", "h1", "h2", "u0", "Re", "dt"};
    double vals[] = {(double)nr, (double)nz, (double)nphi, R, r0, h1, h2, u0, Re, dt};
    char* argv[16];
    argv[0] = (char*)"ref";
    for (int i = 0; i < 10; i++) {
        if (i < 3) snprintf(buf[i], sizeof(buf[i]), "--ns:%s=%d", keys[i], (int)vals[i]);
        else snprintf(buf[i], sizeof(buf[i]), "--ns:%s=%.17g", keys[i], vals[i]);
        argv[i + 1] = buf[i];
    }
    int argc = 11;
    if (vrandom) argv[argc++] = (char*)"--ns:vrandom=1";
    h->cfg.rewrite(argc, argv);
    if (periodic_z) h->p = new NSCyl<double, false, tensor_flag::periodic>(h->cfg);
    else h->d = new NSCyl<double, false, tensor_flag::none>(h->cfg);
    return h;
}

void* ref_nscyl_create(int periodic_z, double R, double r0, double h1, double h2, double u0, double Re, double dt,
                       int nr, int nz, int nphi) {
    return ref_nscyl_create_v(periodic_z, R, r0, h1, h2, u0, Re, dt, nr, nz, nphi, 0);
}

int ref_nscyl_step(void* hp, int k) {
    auto* h = (RefNSCyl*)hp;
    for (int i = 0; i < k; i++) {
        if (h->d) h->d->step();
        else h->p->step();
    }
    return 0;
}

// NSCyl::L_step (src/ns_cyl.cpp:65-77): the step linearised about u0, v0, w0
int ref_nscyl_l_step(void* hp, int k) {
    auto* h = (RefNSCyl*)hp;
    for (int i = 0; i < k; i++) {
        if (h->d) h->d->L_step();
        else h->p->L_step();
    }
    return 0;
}

}  // extern "C"

// fields 0..8: u v w p x F G H RHS; 9..11: the linearisation point u0 v0 w0
template <typename NS>
static typename NS::tensor* nscyl_field(NS* ns, int field) {
    switch (field) {
        case 0: return &ns->u;
        case 1: return &ns->v;
        case 2: return &ns->w;
        case 3: return &ns->p;
        case 4: return &ns->x;
        case 5: return &ns->F;
        case 6: return &ns->G;
        case 7: return &ns->H;
        case 8: return &ns->RHS;
        case 9: return &ns->u0;
        case 10: return &ns->v0;
        default: return &ns->w0;
    }
}

template <typename NS>
static long nscyl_get(NS* ns, int field, double* out) {
    auto* t = nscyl_field(ns, field);
    long n = t->size;
    if (out) memcpy(out, t->vec, sizeof(double) * n);
    return n;
}

template <typename NS>
static long nscyl_set(NS* ns, int field, const double* in) {
    auto* t = nscyl_field(ns, field);
    memcpy(t->vec, in, sizeof(double) * t->size);
    return t->size;
}

extern "C" {

long ref_nscyl_get(void* hp, int field, double* out) {
    auto* h = (RefNSCyl*)hp;
    if (field < 0 || field > 11) return -1;
    return h->d ? nscyl_get(h->d, field, out) : nscyl_get(h->p, field, out);
}

long ref_nscyl_set(void* hp, int field, const double* in) {
    auto* h = (RefNSCyl*)hp;
    if (field < 0 || field > 11) return -1;
    return h->d ? nscyl_set(h->d, field, in) : nscyl_set(h->p, field, in);
}

void ref_nscyl_destroy(void* hp) {
    auto* h = (RefNSCyl*)hp;
    delete h->d;
    delete h->p;
    delete h;
}

int ref_cyclic_reduction_d(double* d, double* e, double* f, double* b, int q, int n, int general) {
    if (general) cyclic_reduction_general(d, e, f, b, q, n);
    else cyclic_reduction(d, e, f, b, q, n);
    return 0;
}

int ref_thomas_d(double* b, double* lower, double* diag, double* upper, int n) {
    solve_tdiag_linear_my(b, lower, diag, upper, n);
    return 0;
}

// Config (src/config.cpp:78-150, 255-297): load `path`, apply the argv
// overrides, then read section:key with a default of the given kind
// (0 double, 1 int, 2 string).  Checker for the Python Config mirror.
extern "C" int ref_config_get(const char* path, int argc, const char** argv, const char* section, const char* key,
                              int kind, const char* def, double* out_d, int* out_i, char* out_s, int out_len) {
    Config c;
    c.open(path);
    std::vector<char*> av;
    av.push_back((char*)"ref");
    for (int i = 0; i < argc; i++) av.push_back((char*)argv[i]);
    c.rewrite((int)av.size(), av.data());
    if (kind == 0) {
        *out_d = c.get(section, key, atof(def));
    } else if (kind == 1) {
        *out_i = c.get(section, key, atoi(def));
    } else {
        const std::string v = c.get(section, key, std::string(def));
        snprintf(out_s, (size_t)out_len, "%s", v.c_str());
    }
    return 0;
}

struct RefNS {
    Config cfg;
    NSCube<double, false>* ns = nullptr;
};

void* ref_nscube_create(int nx, int nz, double Re, double dt, double u0,
                        double x1, double y1, double z1, double x2, double y2, double z2) {
    auto* h = new RefNS();
    char buf[16][96];
    const char* keys[] = {"nx", "nz", "Re", "dt", "u0", "x1", "y1", "z1", "x2", "y2", "z2"};
    double vals[] = {(double)nx, (double)nz, Re, dt, u0, x1, y1, z1, x2, y2, z2};
    char* argv[16];
    argv[0] = (char*)"ref";
    for (int i = 0; i < 11; i++) {
        if (i < 2) snprintf(buf[i], sizeof(buf[i]), "--ns:%s=%d", keys[i], (int)vals[i]);
        else snprintf(buf[i], sizeof(buf[i]), "--ns:%s=%.17g", keys[i], vals[i]);
        argv[i + 1] = buf[i];
    }
    h->cfg.rewrite(12, argv);
    h->ns = new NSCube<double, false>(h->cfg);
    return h;
}

int ref_nscube_step(void* hp, int k) {
    auto* h = (RefNS*)hp;
    for (int i = 0; i < k; i++) h->ns->step();
    return 0;
}

// Copies a field's whole storage (ghost layers included, layout of the
// reference tensor: row-major over its inclusive index ranges, x fastest).
// field: 0=u 1=v 2=w 3=p 4=x 5=F 6=G 7=H 8=RHS.  Returns the element count,
// or -1 for a bad field id.  out may be NULL to query the size.
long ref_nscube_get(void* hp, int field, double* out) {
    auto* h = (RefNS*)hp;
    auto* ns = h->ns;
    tensor<double, 3, false>* t[] = {&ns->u, &ns->v, &ns->w, &ns->p, &ns->x,
                                     &ns->F, &ns->G, &ns->H, &ns->RHS};
    if (field < 0 || field > 8) return -1;
    long n = t[field]->size;
    if (out) memcpy(out, t[field]->vec, sizeof(double) * n);
    return n;
}

int ref_nscube_set(void* hp, int field, const double* in) {
    auto* h = (RefNS*)hp;
    auto* ns = h->ns;
    tensor<double, 3, false>* t[] = {&ns->u, &ns->v, &ns->w, &ns->p, &ns->x,
                                     &ns->F, &ns->G, &ns->H, &ns->RHS};
    if (field < 0 || field > 8) return -1;
    memcpy(t[field]->vec, in, sizeof(double) * t[field]->size);
    return 0;
}

void ref_nscube_destroy(void* hp) {
    auto* h = (RefNS*)hp;
    delete h->ns;
    delete h;
}

// The float instantiation, NSCube<float,false> (src/ns_cube.cpp:281-282),
// same keys; fields are copied out widened to double.
struct RefNSf {
    Config cfg;
    NSCube<float, false>* ns = nullptr;
};

void* ref_nscubef_create(int nx, int nz, double Re, double dt, double u0,
                         double x1, double y1, double z1, double x2, double y2, double z2) {
    auto* h = new RefNSf();
    char buf[16][96];
    const char* keys[] = {"nx", "nz", "Re", "dt", "u0", "x1", "y1", "z1", "x2", "y2", "z2"};
    double vals[] = {(double)nx, (double)nz, Re, dt, u0, x1, y1, z1, x2, y2, z2};
    char* argv[16];
    argv[0] = (char*)"ref";
    for (int i = 0; i < 11; i++) {
        if (i < 2) snprintf(buf[i], sizeof(buf[i]), "--ns:%s=%d", keys[i], (int)vals[i]);
        else snprintf(buf[i], sizeof(buf[i]), "--ns:%s=%.17g", keys[i], vals[i]);
        argv[i + 1] = buf[i];
    }
    h->cfg.rewrite(12, argv);
    h->ns = new NSCube<float, false>(h->cfg);
    return h;
}

int ref_nscubef_step(void* hp, int k) {
    auto* h = (RefNSf*)hp;
    for (int i = 0; i < k; i++) h->ns->step();
    return 0;
}

long ref_nscubef_get(void* hp, int field, double* out) {
    auto* h = (RefNSf*)hp;
    auto* ns = h->ns;
    tensor<float, 3, false>* t[] = {&ns->u, &ns->v, &ns->w, &ns->p, &ns->x,
                                    &ns->F, &ns->G, &ns->H, &ns->RHS};
    if (field < 0 || field > 8) return -1;
    long n = t[field]->size;
    if (out)
        for (long i = 0; i < n; i++) out[i] = (double)t[field]->vec[i];
    return n;
}

void ref_nscubef_destroy(void* hp) {
    auto* h = (RefNSf*)hp;
    delete h->ns;
    delete h;
}

}  // extern "C"
