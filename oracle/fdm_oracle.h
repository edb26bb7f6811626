/* Test infrastructure, not product code.
 *
 * CPU oracle: a plain-C restatement of the reference fdm algorithms on the
 * Poisson / NSCube path.  Only the tests, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it, and only as the checker or as the
 * timed CPU baseline.  The product (libfdmgpu.so) never links or calls it.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef FDM_ORACLE_H
#define FDM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Number of OpenMP threads the oracle uses (0 = runtime default). */
void orc_set_threads(int nthreads);
int orc_get_threads(void);

/* DST-I after Samarskii-Nikolaev, src/fft.cpp:294-365 (FFT<T>::sFFT).
 * S[k] = dx * sum_{j=1}^{N-1} s[j] sin(pi j k / N), k = 1..N-1, N = 2^q.
 * Arrays have N entries, index 0 unused.  s is overwritten (as in the
 * reference).  Returns 0, or -1 if N is not a power of two >= 2. */
int orc_sfft(double* S, double* s, double dx, int N);

/* O(N^2) sine sum, src/asp_fft.cpp:308-318 (sFT).  Same indexing. */
void orc_sft_naive(double* S, const double* s, double dx, int N);

/* LaplCube<double>::solve, Dirichlet, src/lapl_cube.cpp:9-142 with the
 * eigenvalues of :145-172 and the constructor of src/lapl_cube.h:58-100.
 * ans/rhs: nz*ny*nx doubles, x fastest.  Returns -1 on a size whose n+1 is
 * not a power of two (the reference aborts there, src/fft.cpp:67). */
int orc_lapl_cube_solve(int nx, int ny, int nz, double dx, double dy, double dz,
                        double lx, double ly, double lz, double* ans, const double* rhs);

/* LaplRect<double>::solve, src/lapl_rect.cpp:63-110 (DST-y, tridiagonal
 * solve along x per y-mode, inverse DST-y).  ans/rhs: ny*nx, x fastest. */
int orc_lapl_rect_solve(int nx, int ny, double dx, double dy, double lx, double ly,
                        double* ans, const double* rhs);

/* LaplRectFFT2<double>::solve, src/lapl_rect.cpp:113-207 (DST on both axes). */
int orc_lapl_rect_fft2_solve(int nx, int ny, double dx, double dy, double lx, double ly,
                             double* ans, const double* rhs);

/* cyclic_reduction / cyclic_reduction_general, src/cyclic_reduction.h:20-107.
 * d diagonal, e lower (e[0]=0), f upper, b rhs -> solution (in place). */
void orc_cyclic_reduction(double* d, double* e, double* f, double* b, int q, int n, int general);

/* solve_tdiag_linear_my, src/asp_gauss.cpp:185-207 (Thomas, no pivoting).
 * lower[j] = A(j+1,j), upper[j] = A(j,j+1); b -> solution. */
void orc_thomas(double* b, double* lower, double* diag, double* upper, int n);

/* NSCube<double>, src/ns_cube.h:14-92 and src/ns_cube.cpp:27-277.
 * ny equals nx (the reference reads ny from key "nx", src/ns_cube.h:57-59). */
typedef struct orc_nscube orc_nscube;
orc_nscube* orc_ns_create(int nx, int nz, double Re, double dt, double u0,
                          double x1, double y1, double z1, double x2, double y2, double z2);
void orc_ns_step(orc_nscube* ns, int k);
/* field: 0=u 1=v 2=w 3=p 4=x 5=F 6=G 7=H 8=RHS.  Copies the whole storage
 * (ghost layers included) in the reference tensor layout; returns the element
 * count (out may be NULL), or -1 for a bad field id. */
long orc_ns_get(const orc_nscube* ns, int field, double* out);
int orc_ns_set(orc_nscube* ns, int field, const double* in);
void orc_ns_destroy(orc_nscube* ns);

#ifdef __cplusplus
}
#endif
#endif
