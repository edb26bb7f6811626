// Test infrastructure: a C wrapper around the reference's particle-mesh
// N-body driver (class NBody in test/nbody.cpp), compiled from the read-only
// reference tree into oracle/_ref/libfdm_ref.so.  Never part of the product.
//
// test/nbody.cpp is a program: its main() is renamed below and never called.
// Its plotting thread runs (it only waits on a queue; the drawing is compiled
// out in the reference).  BLAS's ?dot is supplied here as the plain
// left-to-right sum of a reference BLAS.
#include <cstring>
#include <vector>

#define main fdm_ref_nbody_program_main
#include "nbody.cpp"
#undef main

extern "C" double cblas_ddot(int n, const double* x, int incx, const double* y, int incy) {
    double s = 0;
    for (int i = 0; i < n; i++) s += x[i * incx] * y[i * incy];
    return s;
}
extern "C" float cblas_sdot(int n, const float* x, int incx, const float* y, int incy) {
    float s = 0;
    for (int i = 0; i < n; i++) s += x[i * incx] * y[i * incy];
    return s;
}

namespace {

struct RefNBody {
    int is_float;
    void* p;
};

template <typename T>
using NB = NBody<T, false>;

template <typename T>
void get_bodies(NB<T>* b, double* x, double* v, double* a, double* aprev, double* mass, double* F) {
    for (int i = 0; i < b->N; i++) {
        const auto& B = b->bodies[i];
        for (int m = 0; m < 3; m++) {
            if (x) x[3 * i + m] = B.x[m];
            if (v) v[3 * i + m] = B.v[m];
            if (a) a[3 * i + m] = B.a[m];
            if (aprev) aprev[3 * i + m] = B.aprev[m];
            if (F) F[3 * i + m] = B.F[m];
        }
        if (mass) mass[i] = B.mass;
    }
}

// Overwrites the bodies and rebuilds what the constructor derives from them:
// the total mass (summed in index order) and the cell lists of both grids,
// filled in index order with the cell formulas of NBody::move.
template <typename T>
void set_bodies(NB<T>* b, const double* x, const double* v, const double* a, const double* aprev, const double* mass) {
    b->mass = 0;
    for (int i = 0; i < b->N; i++) {
        auto& B = b->bodies[i];
        for (int m = 0; m < 3; m++) {
            B.x[m] = (T)x[3 * i + m];
            B.v[m] = (T)v[3 * i + m];
            B.a[m] = a ? (T)a[3 * i + m] : T(0);
            B.aprev[m] = aprev ? (T)aprev[3 * i + m] : T(0);
            B.F[m] = 0;
        }
        B.mass = (T)mass[i];
        b->mass += B.mass;
    }
    for (int i = 0; i < b->n; i++)
        for (int k = 0; k < b->n; k++)
            for (int j = 0; j < b->n; j++) b->cells[i][k][j].bodies.clear();
    for (int i = 0; i < b->npp; i++)
        for (int k = 0; k < b->npp; k++)
            for (int j = 0; j < b->npp; j++) b->cellspp[i][k][j].bodies.clear();
    for (int index = 0; index < b->N; index++) {
        auto& B = b->bodies[index];
        B.j = floor((B.x[0] - b->origin[0]) / b->h);
        B.k = floor((B.x[1] - b->origin[1]) / b->h);
        B.i = floor((B.x[2] - b->origin[2]) / b->h);
        B.jpp = floor((B.x[0] - b->origin[0]) / b->hpp);
        B.kpp = floor((B.x[1] - b->origin[1]) / b->hpp);
        B.ipp = floor((B.x[2] - b->origin[2]) / b->hpp);
        b->cells[B.i][B.k][B.j].bodies.push_back(index);
        b->cellspp[B.ipp][B.kpp][B.jpp].bodies.push_back(index);
    }
}

template <typename T>
void get_fields(NB<T>* b, double* f, double* rhs, double* psi, double* E) {
    const int n = b->n;
    size_t e = 0;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < n; k++)
            for (int j = 0; j < n; j++, e++) {
                if (f) f[e] = b->f[i][k][j];
                if (rhs) rhs[e] = b->rhs[i][k][j];
                if (psi) psi[e] = b->psi[i][k][j];
                if (E)
                    for (int m = 0; m < 3; m++) E[3 * e + m] = b->E[i][k][j][m];
            }
}

}  // namespace

extern "C" {

// NBody<T,false>(x0, y0, z0, l, n, npp, N, dt, G, vel, sgn, local, solar,
// crit, debug=0) of test/nbody.cpp:97-127; the constructor draws the bodies
// (init_points, test/nbody.cpp:515-590).
void* ref_nbody_create(int is_float, double x0, double y0, double z0, double l, int n, int npp, int N, double dt,
                       double G, double vel, int sgn, int local, int solar, double crit) {
    auto* r = new RefNBody{is_float, nullptr};
    if (is_float)
        r->p = new NB<float>((float)x0, (float)y0, (float)z0, l, n, npp, N, dt, G, vel, sgn, local, solar,
                             (float)crit, 0);
    else
        r->p = new NB<double>(x0, y0, z0, l, n, npp, N, dt, G, vel, sgn, local, solar, crit, 0);
    return r;
}

void ref_nbody_destroy(void* h) {
    auto* r = (RefNBody*)h;
    if (r->is_float) delete (NB<float>*)r->p;
    else delete (NB<double>*)r->p;
    delete r;
}

int ref_nbody_count(void* h) {
    auto* r = (RefNBody*)h;
    return r->is_float ? ((NB<float>*)r->p)->N : ((NB<double>*)r->p)->N;
}

double ref_nbody_total_mass(void* h) {
    auto* r = (RefNBody*)h;
    return r->is_float ? ((NB<float>*)r->p)->mass : ((NB<double>*)r->p)->mass;
}

void ref_nbody_get_bodies(void* h, double* x, double* v, double* a, double* aprev, double* mass, double* F) {
    auto* r = (RefNBody*)h;
    if (r->is_float) get_bodies((NB<float>*)r->p, x, v, a, aprev, mass, F);
    else get_bodies((NB<double>*)r->p, x, v, a, aprev, mass, F);
}

void ref_nbody_set_bodies(void* h, const double* x, const double* v, const double* a, const double* aprev,
                          const double* mass) {
    auto* r = (RefNBody*)h;
    if (r->is_float) set_bodies((NB<float>*)r->p, x, v, a, aprev, mass);
    else set_bodies((NB<double>*)r->p, x, v, a, aprev, mass);
}

// NBody::step (test/nbody.cpp:134-143): calc_a_pm, then move
void ref_nbody_step(void* h, int steps) {
    auto* r = (RefNBody*)h;
    for (int s = 0; s < steps; s++) {
        if (r->is_float) ((NB<float>*)r->p)->step();
        else ((NB<double>*)r->p)->step();
    }
}

// density f, right-hand side, potential psi (n^3 each, x fastest) and the
// field E (n^3 x 3) as left by the last step
void ref_nbody_get_fields(void* h, double* f, double* rhs, double* psi, double* E) {
    auto* r = (RefNBody*)h;
    if (r->is_float) get_fields((NB<float>*)r->p, f, rhs, psi, E);
    else get_fields((NB<double>*)r->p, f, rhs, psi, E);
}

}  // extern "C"
