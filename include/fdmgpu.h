/*
 * fdmgpu — GB300 (sm_103a) fast Poisson solver and NSCube projection step.
 *
 * C ABI of libfdmgpu.so: plain pointers, sizes and status codes, no C++ or
 * CUDA types.  `stream` arguments are a cudaStream_t passed as void* (NULL =
 * the legacy default stream).  Host-pointer entry points are synchronous and
 * keep the reference's semantics; *_device entry points take device pointers
 * and are asynchronous on `stream`.
 *
 * Each entry point names the reference interface it replaces (paths are
 * within the reference project resetius/fdm).  The reference has no C ABI:
 * its interface is the C++ templates listed here, which the header-only shims
 * in include/fdm_gb300/ recreate on top of this ABI.
 *
 * Every function returns FDMGPU_OK (0) or a status code; the message of the
 * calling thread's last error is available from fdmgpu_last_error().  The
 * reference aborts through verify() where these functions return an error
 * (src/verify.h:10-36, src/fft.cpp:67); the C++ shims restore that.
 *
 * Thread safety: a handle is used by one thread at a time (the reference's
 * LaplCube::solve is not re-entrant per instance either, src/lapl_cube.h:55-56).
 * Distinct handles may be used concurrently.
 */
#ifndef FDMGPU_H
#define FDMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    FDMGPU_OK = 0,
    FDMGPU_EINVAL = 1,    /* bad argument (null handle/pointer, bad enum)      */
    FDMGPU_ESIZE = 2,     /* unsupported size: n+1 not a power of two, n < 1,
                             or n above FDMGPU_MAX_N (reference: verify abort,
                             src/fft.cpp:67)                                    */
    FDMGPU_ENOMEM = 3,    /* device or host allocation failed                   */
    FDMGPU_ECUDA = 4,     /* a CUDA runtime call failed                         */
    FDMGPU_ETIMEOUT = 5,  /* a bounded device-side wait gave up                 */
    FDMGPU_ENOTSUP = 6,   /* combination not supported (e.g. periodic flags)    */
    FDMGPU_EBUDGET = 7,   /* request exceeds the configured memory budget      */
    FDMGPU_EBUSY = 8      /* serving loop: queue full, or the request waited
                             past its queue deadline and was shed               */
};

/* element type of user arrays */
enum { FDMGPU_F64 = 0, FDMGPU_F32 = 1 };

/* solve precision */
enum {
    FDMGPU_PLAIN = 0, /* every stage in the element type (FP64 for F64)       */
    FDMGPU_MIXED = 1  /* F64 arrays only: FP32 DST/tridiagonal inner solves,
                         accurate residual, iterative refinement             */
};

/* boundary flags per axis (bit 0 = x, 1 = y, 2 = z, set = periodic).  The
 * reference instantiates all-Dirichlet and all-periodic LaplCube
 * (src/lapl_cube.cpp:174-182); mixed flags return FDMGPU_ENOTSUP.  Periodic:
 * n = nx, ny, nz points per axis, each a power of two <= 512, arrays of
 * nz*ny*nx points as the reference's periodic callers pass them
 * (ut/ut_lapl_cube.cpp:156-243); plain precision only; the zero mode of
 * the answer is set to 0 (src/lapl_cube.cpp:82-84). */
enum { FDMGPU_DIRICHLET = 0, FDMGPU_PERIODIC = 7 };

#define FDMGPU_MAX_N 1023 /* largest interior size per axis */

const char* fdmgpu_last_error(void);
int fdmgpu_version(void);

/* ---- launch accounting and timing (no reference counterpart: the reference
 * times its phases with std::chrono, src/ns_cube.cpp:27-62) ---------------
 * fdmgpu_launch_count: kernels launched by this library since load.
 * fdmgpu_profile_enable(1): bracket every later launch with CUDA events on
 * its stream; fdmgpu_profile_collect resolves them into per-kernel totals
 * (synchronises those events) and reports the number of kernel names;
 * fdmgpu_profile_entry reads total i. */
unsigned long long fdmgpu_launch_count(void);
int fdmgpu_profile_enable(int on);
int fdmgpu_profile_collect(int* nnames);
int fdmgpu_profile_entry(int i, char* name, int namelen, long long* count, double* total_ms);
int fdmgpu_profile_reset(void);

/* ---- LaplCube: 3-D Dirichlet Poisson --------------------------------------
 * Replaces fdm::LaplCube<T,check,F> (src/lapl_cube.h:9-106):
 *   ctor LaplCube(dx,dy,dz, lx,ly,lz, nx,ny,nz)   src/lapl_cube.h:58-100
 *   void solve(T* ans, T* rhs)                    src/lapl_cube.cpp:9-142
 * Arrays are the interior nz*ny*nx points, x fastest (the tensor view
 * {1,nz,1,ny,1,nx}, src/lapl_cube.h:80).  The result equals the reference's
 * DST_z DST_y DST_x / (-lambda) inverse transforms, including its scale
 * convention (forward h*sqrt(2/l), inverse sqrt(2/l) per axis) and its use of
 * lm_y for x and z when the point counts match (src/lapl_cube.cpp:165,171). */
typedef struct fdmgpu_lapl_cube fdmgpu_lapl_cube;

int fdmgpu_lapl_cube_create(fdmgpu_lapl_cube** h, int dtype, int bc_flags,
                            double dx, double dy, double dz,
                            double lx, double ly, double lz,
                            int nx, int ny, int nz);
/* FDMGPU_MIXED needs dtype F64.  tol: target relative error (<= 0 selects
 * 1e-10); max_sweeps: refinement sweeps cap (< 0 selects 3).  Sweeps run by
 * the tolerance: none for tol >= 1e-5, one down to 1e-11, two below.  Plans
 * whose operator is too ill-conditioned for FP32 inner solves (the ratio of
 * the largest to the smallest eigenvalue, summed over the axes, above 3e4:
 * 255^3 is 2.7e4, an axis of 511 or more points exceeds it) solve in FP64
 * instead; last_info then reports sweeps = -1. */
int fdmgpu_lapl_cube_set_precision(fdmgpu_lapl_cube* h, int precision, double tol, int max_sweeps);
/* host pointers, synchronous (LaplCube::solve, src/lapl_cube.cpp:9) */
int fdmgpu_lapl_cube_solve(fdmgpu_lapl_cube* h, void* ans, const void* rhs);
/* host pointers, nrhs volumes back to back, synchronous.  The volumes are
 * pipelined one at a time through a ring of three device slots: the copy-in
 * of one volume, the solve of the previous one and the copy-out of the one
 * before overlap on three streams (page-locked host memory is needed for the
 * copies to overlap).  last_info afterwards reports the last volume. */
int fdmgpu_lapl_cube_solve_host_batch(fdmgpu_lapl_cube* h, void* ans, const void* rhs, int nrhs);
/* device pointers; nrhs volumes back to back (stride nz*ny*nx elements);
 * asynchronous on stream */
int fdmgpu_lapl_cube_solve_device(fdmgpu_lapl_cube* h, void* d_ans, const void* d_rhs,
                                  int nrhs, void* stream);
/* Mixed-precision solve that allocates nothing (no counterpart in the
 * reference, whose LaplCube owns its scratch as member vectors).  For
 * callers that must not allocate device memory while they solve: programs
 * whose device memory belongs to their own pool or to another framework's
 * allocator, loops that must not wait on the allocator after start-up, and
 * hosts that forbid device allocation once initialised.  Same arguments as a
 * handle created with these sizes and set to FDMGPU_MIXED with `tol`, called
 * through fdmgpu_lapl_cube_solve_device (FP64 device arrays, nrhs volumes
 * back to back, asynchronous on stream), but no handle.  It runs the
 * handle's kernels in the five-pass order with FFT DST passes (a handle may
 * instead take the fused plane pass, or the tensor cores for 32-point axes;
 * the answers agree to the mixed tolerance), sweeps chosen by tol, the
 * per-mode z factor table when the z line splits into blocks.  Its tables are computed on the
 * device in FP64 (a handle builds them on the host), so an FP32 table entry
 * can differ in its last bit and the answer agrees with the handle's to
 * round-off of the refined solve, not bit for bit.  The tables, FP32 work
 * volumes and norms live in one array of FDMGPU_NOALLOC_SCRATCH_BYTES that
 * the library holds on every device it is loaded on, until the process
 * exits.  Limit: 4*nx*ny*nz*nrhs bytes per FP32 volume, 1 volume for
 * tol >= 1e-5 (no sweep), 2 for 1e-11 <= tol < 1e-5 (one sweep), 3 below
 * (two sweeps), plus the z table, 4*(2m + 2(P-1)) bytes per (x,y) mode (m =
 * min(nz,15) rows per block, P = (nz+1)/(m+1) blocks; 2.8 MB at 127x127,
 * 15.6 MB at 255x255), plus a few KB: about 8.3M, 4.1M and 2.7M points
 * less the table.  Larger requests return FDMGPU_EBUDGET with the byte
 * counts in the message, and sizes beyond the mixed solve's conditioning
 * limit (see fdmgpu_lapl_cube_set_precision) return FDMGPU_ENOTSUP.  The
 * first call on a device looks up the array's device address (and loads the
 * module there) and keeps it: make that first call before any stream
 * capture, and do not call the library again on a device after
 * cudaDeviceReset (the kept address would be stale).  All calls on a device
 * share the array: calls that overlap on the GPU (other streams, other host
 * threads) race on it, so serialise them.  No cudaMalloc, cudaFree or other
 * allocating routine is called (with fdmgpu_profile_enable(1) the library
 * creates timing events for every launch, this entry point's included). */
#define FDMGPU_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int fdmgpu_lapl_cube_solve_mixed_noalloc(double dx, double dy, double dz, double lx, double ly, double lz,
                                         int nx, int ny, int nz, double tol, void* d_ans, const void* d_rhs,
                                         int nrhs, void* stream);
/* refinement report of the last solve: sweeps done (-1: a mixed plan that
 * solved in FP64) and, per RHS, the estimated relative L2 error left in the
 * answer (-1 when no sweep ran).  Sweep k measures e_k = ||c_k||/||u||, the
 * size of its correction; the estimate after the last sweep is rho e_k with
 * the observed contraction rho = e_k/e_{k-1}, or rho = 100 e_1 after a single
 * sweep (a margin over the FP32 inner solve's contraction measured on GB300),
 * and never below 3e-16 times the operator's eigenvalue ratio (the floor of
 * the float-float residual).
 * est may be NULL; it receives nrhs values.  Synchronises the handle's last
 * stream.  (No reference counterpart: the reference solves exactly in T.) */
int fdmgpu_lapl_cube_last_info(fdmgpu_lapl_cube* h, int* sweeps, double* est, int nrhs);
/* adaptive = 1: after the sweeps that tol asks for, the mixed solve checks
 * every right-hand side's estimate (as last_info reports it) and runs
 * further sweeps, up to max_sweeps, while one exceeds tol; each check
 * synchronises the solve's stream, so the call returns after the device
 * finished.  0 (default): the sweep count follows tol alone and the solve
 * stays asynchronous.  No reference counterpart. */
int fdmgpu_lapl_cube_set_refinement(fdmgpu_lapl_cube* h, int adaptive);
/* bytes of device scratch the handle holds */
int fdmgpu_lapl_cube_scratch_bytes(fdmgpu_lapl_cube* h, size_t* bytes);
/* schedule of the mixed form: ztable = 1 uses the per-mode z factor table
 * (default), 0 computes the factors per solve; dst_tc bit 0 / bit 1 runs the
 * plain FP32 DST passes along x / y on the tensor cores when that axis has
 * 32, 64 or 128 points.  Until this is called, a mixed plan puts 32-point x
 * axes on the tensor cores, and 32-point y axes when it runs the five-pass
 * pipeline (the faster schedules measured on GB300); every other axis runs
 * FFTs. */
int fdmgpu_lapl_cube_set_schedule(fdmgpu_lapl_cube* h, int ztable, int dst_tc);
/* Times every schedule of the mixed form (pipeline, z-solve variant,
 * tensor-core axes) on nrhs right-hand sides at d_rhs (answers to d_ans)
 * and keeps the fastest whose accuracy is assured: with a refinement sweep,
 * a variant without the z factor table or with tensor-core passes must show,
 * from its measured first-sweep correction e, that 10 e^(sweeps+1) <= tol;
 * without a sweep, variants without the table are not kept.  Synchronous on
 * stream; *ms (may be NULL) receives the kept schedule's time per call.  A
 * plain or FP64-fallback plan is left as it is.  No reference counterpart. */
int fdmgpu_lapl_cube_tune(fdmgpu_lapl_cube* h, void* d_ans, const void* d_rhs, int nrhs, void* stream, double* ms);
/* the mixed form's schedule: the pipeline asked for (FDMGPU_PIPE_*;
 * fdmgpu_lapl_cube_pipeline_in_use reports the one a solve runs), ztable and
 * the tensor-core axes (dst_tc bits) */
int fdmgpu_lapl_cube_get_schedule(fdmgpu_lapl_cube* h, int* pipeline, int* ztable, int* dst_tc);
/* pass structure of the mixed form (no counterpart in the reference, which
 * transforms x, y and z in turn, src/lapl_cube.cpp:13-141).
 * FDMGPU_PIPE_PLANES (default): per sweep the DST along y, one fused pass per
 * y-mode plane (DST along x, tridiagonal z solve, inverse DST along x; a
 * cluster of CTAs per plane) and the inverse DST along y: three passes over
 * the volume instead of five.  It applies when the x line has 64, 128 or
 * 256 points, nz + 1 is 1, 2, 4 or 8 times the plane pass's rows per CTA (32
 * at 128 and 256 points, 64 at 64 points), the z factor table is in use and
 * the x DST is not on the tensor cores; otherwise, and with
 * FDMGPU_PIPE_FIVE_PASS, the solve runs DST x, DST y, z solve, inverse DST
 * y, inverse DST x.  Both give the same answer to the mixed tolerance.
 * fdmgpu_lapl_cube_pipeline_in_use reports which one a solve would run. */
enum { FDMGPU_PIPE_FIVE_PASS = 0, FDMGPU_PIPE_PLANES = 1 };
int fdmgpu_lapl_cube_set_pipeline(fdmgpu_lapl_cube* h, int pipeline);
int fdmgpu_lapl_cube_pipeline_in_use(fdmgpu_lapl_cube* h, int* pipeline);
/* 1 in *failed if a tensor-core pass of this handle gave up waiting for its
 * MMAs (synchronises the device) */
int fdmgpu_lapl_cube_device_status(fdmgpu_lapl_cube* h, int* failed);
int fdmgpu_lapl_cube_destroy(fdmgpu_lapl_cube* h);

/* ---- Batched solves of uneven sizes (no counterpart in the reference,
 * which solves one LaplCube at a time) -------------------------------------
 * count right-hand sides, right-hand side i with sizes n3[3i..3i+2]
 * (nx,ny,nz), spacings h3[3i..] and lengths l3[3i..] as in
 * fdmgpu_lapl_cube_create.  Right-hand sides of equal geometry form a group
 * with one plan.  d_ans / d_rhs are host arrays of count device pointers
 * (FP64 volumes).  fdmgpu_batch_tune times each group's schedule candidates
 * (right-hand sides per pipeline launch, z-solve variant) on the given data
 * and keeps the fastest.  The first fdmgpu_batch_solve after creation or
 * tuning captures all groups, on concurrent streams, into one CUDA graph;
 * every solve is then one graph launch, ordered after prior work on
 * `stream` and before later work on it.  Volume pointers may change
 * between solves. */
typedef struct fdmgpu_batch fdmgpu_batch;
int fdmgpu_batch_create(fdmgpu_batch** h, int count, const int* n3, const double* h3, const double* l3,
                        int precision, double tol);
int fdmgpu_batch_tune(fdmgpu_batch* h, void* const* d_ans, const void* const* d_rhs);
int fdmgpu_batch_solve(fdmgpu_batch* h, void* const* d_ans, const void* const* d_rhs, void* stream);
/* groups formed and kernel launches one graph launch replays */
int fdmgpu_batch_info(fdmgpu_batch* h, int* groups, int* launches_per_solve);
/* schedule of one group: sizes, members, chunk, 1 = table-driven z-solve,
 * the tensor-core axes (bit 0 x, bit 1 y), and its tuned time in ms (0
 * before tuning) */
int fdmgpu_batch_schedule(fdmgpu_batch* h, int group, int* n3, int* members, int* chunk, int* ztable,
                          int* dst_tc, double* tuned_ms);
int fdmgpu_batch_destroy(fdmgpu_batch* h);

/* ---- LaplCyl3FFT2: Poisson in a cylindrical annulus ----------------------
 * Replaces fdm::LaplCyl3FFT2<T,check,zflag> (src/lapl_cyl.h:178-262,
 * src/lapl_cyl.cpp:10-166): ctor (dr, dz, r0, lr, lz, nr, nz, nphi), arrays of
 * nphi x nz x nr points, r fastest (the tensor {0..nphi-1, z1..zn, 1..nr}).
 * phi periodic (nphi a power of two <= 512); z Dirichlet (nz+1 a power of
 * two) or periodic (periodic_z, nz a power of two <= 512). */
typedef struct fdmgpu_lapl_cyl fdmgpu_lapl_cyl;
int fdmgpu_lapl_cyl_create(fdmgpu_lapl_cyl** h, int dtype, int periodic_z, double dr, double dz, double r0,
                           double lr, double lz, int nr, int nz, int nphi);
int fdmgpu_lapl_cyl_solve(fdmgpu_lapl_cyl* h, void* ans, const void* rhs);
int fdmgpu_lapl_cyl_solve_device(fdmgpu_lapl_cyl* h, void* d_ans, const void* d_rhs, int nrhs, void* stream);
int fdmgpu_lapl_cyl_destroy(fdmgpu_lapl_cyl* h);

/* ---- LaplRect / LaplRectFFT2: 2-D Dirichlet Poisson ----------------------
 * Replaces fdm::LaplRect<T,check,F> (src/lapl_rect.h:11-73, solve
 * src/lapl_rect.cpp:63-110: DST-y, tridiagonal solve along x per y-mode,
 * inverse DST-y) and fdm::LaplRectFFT2 (src/lapl_rect.h:75-105, solve
 * src/lapl_rect.cpp:113-207: DST on both axes).  ctor (dx,dy,lx,ly,nx,ny);
 * arrays ny*nx, x fastest.  LaplRect needs ny+1 a power of two (any nx >= 1);
 * LaplRectFFT2 needs both. */
enum { FDMGPU_RECT_TRIDIAG = 0, FDMGPU_RECT_FFT2 = 1 };
typedef struct fdmgpu_lapl_rect fdmgpu_lapl_rect;

int fdmgpu_lapl_rect_create(fdmgpu_lapl_rect** h, int dtype, int method,
                            double dx, double dy, double lx, double ly, int nx, int ny);
/* The same with the reference's periodic flags (LaplRect(FFT2)<T,check,F>,
 * src/lapl_rect.cpp:209-238): flags bit 1 = y periodic (F::head), bit 0 = x
 * periodic (F::tail::head).  0, 2 (y) and 3 (y and x) are instantiated; other
 * values return FDMGPU_ENOTSUP.  A periodic axis has n points, a power of two
 * (pFFT_1 / pFFT along it, lm = 4/h^2 sin^2(k pi/n)); arrays are the
 * reference's {y1..yn, x1..xn} ranges, ny x nx.  LaplRect solves x as
 * tridiagonal systems whatever bit 0 says (as the reference does); with both
 * axes periodic LaplRectFFT2 sets the (0, 0) mode to 1 as the reference's
 * "hack for double-period" does (src/lapl_rect.cpp:169-172). */
int fdmgpu_lapl_rect_create_flags(fdmgpu_lapl_rect** h, int dtype, int method, int flags,
                                  double dx, double dy, double lx, double ly, int nx, int ny);
int fdmgpu_lapl_rect_solve(fdmgpu_lapl_rect* h, void* ans, const void* rhs);
int fdmgpu_lapl_rect_solve_device(fdmgpu_lapl_rect* h, void* d_ans, const void* d_rhs,
                                  int nrhs, void* stream);
int fdmgpu_lapl_rect_destroy(fdmgpu_lapl_rect* h);

/* ---- 1-D building blocks (test / integration surface) --------------------
 * fdmgpu_sine_device: S[k] = scale * sum_j s[j] sin(pi j k / N) for nlines
 * contiguous lines of n = N-1 values (FFT<T>::sFFT, src/fft.cpp:294-365, on
 * the 1..N-1 part of its arrays).
 * fdmgpu_tridiag_device: nsys independent tridiagonal systems stored
 * system-interleaved (element i of system s at [i*nsys + s]):
 * lower[i]*x[i-1] + diag[i]*x[i] + upper[i]*x[i+1] = b[i], solved in place
 * in b (the solve of cyclic_reduction / solve_tdiag_linear_my,
 * src/cyclic_reduction.h:20-107, src/asp_gauss.cpp:185-207). */
int fdmgpu_sine_device(int dtype, int N, int nlines, double scale,
                       void* d_out, const void* d_in, void* stream);
/* FFT<T>::pFFT_1_3d (inverse = 0) / pFFT_3d (inverse = 1) of
 * src/fft.cpp:214-292: the periodic real transform in the reference's
 * coefficient layout along x (fastest), then y, then z of an n^3 cube
 * (n a power of two, 2..512), scale dx on every pass.  The _device form
 * takes `count` cubes back to back and is asynchronous on stream; the host
 * form is synchronous. */
int fdmgpu_pfft3d_device(int dtype, int n, int inverse, double dx, void* d_out, const void* d_in, int count,
                         void* stream);
int fdmgpu_pfft3d(int dtype, int n, int inverse, double dx, void* out, const void* in);
/* FFT<T>::pFFT_1 (inverse = 0) / pFFT (inverse = 1), src/fft.cpp:108-212, of
 * nlines contiguous lines of N values (N a power of two, 2..512), scale dx;
 * asynchronous on stream */
int fdmgpu_pfft_device(int dtype, int N, int inverse, int nlines, double dx, void* d_out, const void* d_in,
                       void* stream);
/* DST-I of FP32 lines of N-1 points (N = 32, 64 or 128) as a dense contraction
 * with the sine matrix on the tensor cores (split TF32, FP32 accumulation;
 * no counterpart in the reference).  axis 0: `count` contiguous lines;
 * axis 1: `count` planes of (N-1) rows x nx, transformed along the rows.
 * Synchronous; FDMGPU_ETIMEOUT if the kernel's bounded wait for its MMAs
 * gave up. */
int fdmgpu_sine_tc_device(int N, int axis, int nx, long long count, double scale, void* d_out,
                          const void* d_in, void* stream);
/* Diagnostic of the bounded mbarrier wait of the tensor-core kernels: waits
 * `spins` tries on an mbarrier that nothing arrives at and returns
 * FDMGPU_ETIMEOUT when the wait gives up, as it must (no fault, no hang; the
 * context stays usable).  spins in [1, 2^20]. */
int fdmgpu_check_bounded_wait(unsigned spins);
int fdmgpu_tridiag_device(int dtype, int n, int nsys, const void* d_lower, const void* d_diag,
                          const void* d_upper, void* d_b, void* stream);

/* ---- NSCube: lid-driven cavity projection step ---------------------------
 * Replaces fdm::NSCube<T,check> (src/ns_cube.h:14-92): ctor from Config keys
 * ns:{x1,y1,z1,x2,y2,z2,u0,Re,dt,nx,nz} (ny is read from key nx, as in the
 * reference, src/ns_cube.h:57-59), step() (src/ns_cube.cpp:27-62) and the
 * public tensors u,v,w,p,x,F,G,H,RHS in the reference layouts (inclusive
 * index ranges, x fastest).  State lives on the device.  dtype FDMGPU_F64
 * is NSCube<double>; FDMGPU_F32 is NSCube<float> (src/ns_cube.cpp:281-282):
 * fields in float, each expression evaluated with the reference's C++
 * promotions (float where only fields meet, double once a double parameter
 * enters), the pressure solve by the FP32 LaplCube.  Host buffers of the
 * field copies hold the handle's element type. */
typedef struct fdmgpu_nscube fdmgpu_nscube;
enum {
    FDMGPU_NS_U = 0, FDMGPU_NS_V, FDMGPU_NS_W, FDMGPU_NS_P, FDMGPU_NS_X,
    FDMGPU_NS_F, FDMGPU_NS_G, FDMGPU_NS_H, FDMGPU_NS_RHS
};

int fdmgpu_nscube_create(fdmgpu_nscube** h, int dtype, int nx, int nz,
                         double x1, double y1, double z1, double x2, double y2, double z2,
                         double u0, double Re, double dt);
/* k steps; asynchronous on the handle's stream */
int fdmgpu_nscube_step(fdmgpu_nscube* h, int k);
/* steps[i] steps of each of n distinct FP64 cavities of one geometry (grid,
 * spacing, box extents, quotient form; Re, dt and u0 may differ): step r of
 * every cavity with more than r steps to go is one launch per kernel, the
 * cavity read from a table by the grid's y index.  The fields are bit for
 * bit those of fdmgpu_nscube_step on each handle.  Asynchronous on the
 * first handle's stream, ordered after the work queued on every handle's
 * stream and before what is queued there later.  FDMGPU_EINVAL for a
 * repeated handle or different geometries, FDMGPU_ENOTSUP for FP32.  No
 * reference counterpart: the reference steps one NSCube per call
 * (src/ns_cube.cpp:27-62). */
int fdmgpu_nscube_step_many(fdmgpu_nscube* const* hs, const int* steps, int n);
/* exact = 1: every quotient by a run constant (Re, dx, dx^2, dt, ...) in
 * the boundary ghosts, F/G/H and the divergence is correctly rounded, as the
 * reference's a / b is (five FP64 operations each).  exact = 0 (default):
 * products with reciprocals computed once on the host, about half the FP64
 * operations of F/G/H; the fields then differ from the exact form's in the
 * last bits (about 1e-15 relative after 20 steps of the 15^3 cavity).  No
 * reference counterpart: the reference divides. */
int fdmgpu_nscube_set_exact(fdmgpu_nscube* h, int exact);
int fdmgpu_nscube_set_stream(fdmgpu_nscube* h, void* stream);
/* element count of a field's storage (ghost layers included) and its index
 * ranges {z1,z2,y1,y2,x1,x2} */
int fdmgpu_nscube_field_info(fdmgpu_nscube* h, int field, size_t* count, int* ranges6);
/* copies between a field and host memory (synchronous) */
int fdmgpu_nscube_get_field(fdmgpu_nscube* h, int field, void* host, size_t count);
int fdmgpu_nscube_set_field(fdmgpu_nscube* h, int field, const void* host, size_t count);
/* device pointer of a field's storage */
int fdmgpu_nscube_field_device(fdmgpu_nscube* h, int field, void** dptr);
int fdmgpu_nscube_time_index(fdmgpu_nscube* h, int* t);
int fdmgpu_nscube_dtype(fdmgpu_nscube* h, int* dtype);
/* ASCII VTK snapshot of the cell-centred velocity, as the reference's
 * velocity_plotter::vtk_out writes it for a cube (src/velocity_plot.cpp:
 * 113-119, 200-217): STRUCTURED_POINTS header, one "%f %f %f" line per
 * interior cell, x fastest.  Synchronous. */
int fdmgpu_nscube_vtk_out(fdmgpu_nscube* h, const char* path);
int fdmgpu_nscube_destroy(fdmgpu_nscube* h);
/* Diagnostic of the NSCube stencils' division by run constants (h, h^2, Re,
 * dt): writes the IEEE quotient a/b and the library's constant-divisor
 * quotient (precomputed reciprocal plus remainder corrections) for n device
 * pairs, so a test can check they agree bit for bit. */
int fdmgpu_check_const_division(long long n, const double* d_a, const double* d_b, double* d_q_ieee,
                                double* d_q_const, void* stream);
/* Diagnostic: for n FP64 values x, the mixed path's integer conversions
 * beside the hardware's -- f32 = its nearest float (ties away from zero in
 * the normal float range, the hardware's ties-to-even outside it), f32_hw the
 * hardware conversion, (split_hi, split_lo) its float pair -- and for n float
 * pairs (hi, lo) the pair's FP64 value by integer assembly (f64) beside the
 * hardware sum (f64_hw).  Device arrays; asynchronous on stream. */
int fdmgpu_check_dd_conversions(long long n, const double* d_x, const float* d_hi, const float* d_lo, float* d_f32,
                                float* d_f32_hw, float* d_split_hi, float* d_split_lo, double* d_f64, double* d_f64_hw,
                                void* stream);

/* ---- Serving loop (no counterpart in the reference, which runs one
 * solve or one NSCube on the caller's thread) ------------------------------
 * Requests are Poisson solves (host buffers, FP64, page-locked) and
 * k-step advances of resident NSCube sessions.  One scheduler thread admits
 * them first come first served while their device memory fits under
 * budget_bytes (staging of requests in flight + pooled solver plans +
 * session state), runs up to `lanes` launches concurrently on separate CUDA
 * streams, and merges waiting solves of the same geometry and refinement
 * class into one launch of up to max_batch right-hand sides (continuous
 * batching).  A solve's answer does not depend on the company it keeps.
 * Latency is submit to completion on the device, copies included.
 * Solve tolerance: tol <= 0 selects the plain FP64 form; otherwise the
 * mixed form with the refinement sweeps tol asks for. */
typedef struct fdmgpu_server fdmgpu_server;
enum { FDMGPU_REQ_SOLVE = 0, FDMGPU_REQ_ADVANCE = 1 };
enum {
    FDMGPU_REQ_QUEUED = 0, FDMGPU_REQ_RUNNING = 1, FDMGPU_REQ_DONE = 2,
    FDMGPU_REQ_FAILED = 3, FDMGPU_REQ_CANCELLED = 4
};
typedef struct {
    unsigned long long submitted, completed, failed, cancelled, rejected;
    int queued, running;
    unsigned long long batches, batched_requests; /* solve launches, solves they carried */
    double used_bytes, peak_bytes, budget_bytes, plan_bytes, session_bytes;
    double p50_ms, p99_ms, p50_solve_ms, p99_solve_ms, p50_advance_ms, p99_advance_ms;
    double mean_queue_ms;
    unsigned long long shed; /* refused at a full queue or dropped at the queue deadline (FDMGPU_EBUSY) */
} fdmgpu_server_stats_t;

int fdmgpu_server_create(fdmgpu_server** h, double budget_bytes, int lanes, int max_batch);
/* n3 = (nx,ny,nz), h3 = (dx,dy,dz), l3 = (lx,ly,lz) as fdmgpu_lapl_cube_create;
 * FDMGPU_EBUDGET when the request alone can never fit */
int fdmgpu_server_submit_solve(fdmgpu_server* h, unsigned long long* id, const int* n3, const double* h3,
                               const double* l3, double tol, const double* rhs, double* ans);
/* a resident lid-driven cavity (parameters of fdmgpu_nscube_create, FP64) */
int fdmgpu_server_session_create(fdmgpu_server* h, int* session, int nx, int nz, double x1, double y1,
                                 double z1, double x2, double y2, double z2, double u0, double Re, double dt);
/* advances run in submission order per session; waiting advances of
 * sessions whose cavities have one geometry (grid, spacing, box extents) run
 * their steps as shared launches (up to max_batch sessions), with results
 * bit for bit those of steps run alone */
int fdmgpu_server_submit_advance(fdmgpu_server* h, unsigned long long* id, int session, int steps);
/* state of a request; a finished (done, failed, cancelled) request is
 * reported once and then forgotten.  latency_ms: submit to completion
 * (-1 while unfinished); queue_ms: submit to launch; batch: requests in its
 * launch; err_est (may be NULL): for a finished mixed-precision solve the
 * estimated relative L2 error of its answer (the model of
 * fdmgpu_lapl_cube_last_info), 0 for an FP64 solve, -1 otherwise.  A failed
 * request's message is left in fdmgpu_last_error(). */
int fdmgpu_server_poll(fdmgpu_server* h, unsigned long long id, int* state, int* status, double* latency_ms,
                       double* queue_ms, int* batch, double* err_est);
/* as poll, blocking until the request finishes or timeout_ms passes
 * (FDMGPU_ETIMEOUT) */
int fdmgpu_server_wait(fdmgpu_server* h, unsigned long long id, double timeout_ms, int* state, int* status,
                       double* latency_ms, double* queue_ms, int* batch, double* err_est);
/* the next finished request (any), reported as poll does; FDMGPU_ETIMEOUT
 * when none finishes within timeout_ms */
int fdmgpu_server_next_done(fdmgpu_server* h, double timeout_ms, unsigned long long* id, int* state,
                            int* status, double* latency_ms, double* queue_ms, int* batch, double* err_est);
/* cancels a queued request (FDMGPU_EINVAL once it has started) */
int fdmgpu_server_cancel(fdmgpu_server* h, unsigned long long id);
/* copies a session field (FDMGPU_NS_*) once its queued advances are done */
int fdmgpu_server_session_get_field(fdmgpu_server* h, int session, int field, double* out, size_t count,
                                    long long* steps_done, double timeout_ms);
int fdmgpu_server_session_close(fdmgpu_server* h, int session, double timeout_ms);
int fdmgpu_server_stats(fdmgpu_server* h, fdmgpu_server_stats_t* out);
int fdmgpu_server_stats_reset(fdmgpu_server* h);
/* load shedding (both off by default): with max_queued > 0 a submit finds
 * the queue holding max_queued requests and returns FDMGPU_EBUSY (nothing is
 * queued); with max_wait_ms > 0 a request that has not started max_wait_ms
 * after its submission finishes as FDMGPU_REQ_FAILED with status
 * FDMGPU_EBUSY (a skipped advance leaves its session where it was; later
 * advances of the session still run in order).  Both count in stats.shed. */
int fdmgpu_server_set_admission(fdmgpu_server* h, int max_queued, double max_wait_ms);
/* cancels queued requests, waits for running ones, frees everything */
int fdmgpu_server_destroy(fdmgpu_server* h);

/* ---- NSCyl: flow between coaxial cylinders -------------------------------
 * Replaces fdm::NSCyl<T,check,zflag> (src/ns_cyl.h:18-134,
 * src/ns_cyl.cpp:22-485): Config keys ns:{R, r, h1, h2, u0, Re, dt, nr, nz,
 * nphi}, step(), public tensors u (r), v (z), w (phi), p, x, F, G, H, RHS
 * (field ids FDMGPU_NS_*) in the reference layouts (phi, z, r), r fastest,
 * ranges {0..nphi-1, z-range, r-range}.  The pressure solve is
 * LaplCyl3FFT2.  Dirichlet z needs nz <= nr (the reference's axial ghost loop
 * runs r over the z bounds, src/ns_cyl.cpp:106-111). */
typedef struct fdmgpu_nscyl fdmgpu_nscyl;
int fdmgpu_nscyl_create(fdmgpu_nscyl** h, int dtype, int periodic_z, double R, double r0, double h1, double h2,
                        double u0, double Re, double dt, int nr, int nz, int nphi);
int fdmgpu_nscyl_step(fdmgpu_nscyl* h, int k);
int fdmgpu_nscyl_field_info(fdmgpu_nscyl* h, int field, size_t* count, int* ranges6);
int fdmgpu_nscyl_get_field(fdmgpu_nscyl* h, int field, void* host, size_t count);
/* Fields 9, 10, 11 are u0, v0, w0, the state L_step linearises about
 * (src/ns_cyl.h:40-41, zero until set; layouts of u, v, w).  set_field
 * overwrites a whole field, ghosts included. */
int fdmgpu_nscyl_set_field(fdmgpu_nscyl* h, int field, const void* host, size_t count);
/* NSCyl::L_step (src/ns_cyl.cpp:65-77): init_bound, L_FGH (:279-404),
 * poisson, update; k steps, captured into its own CUDA graph */
int fdmgpu_nscyl_l_step(fdmgpu_nscyl* h, int k);
/* the constructor's ns:vrandom=1 option (src/ns_cyl.h:99-109): call right
 * after fdmgpu_nscyl_create */
int fdmgpu_nscyl_vrandom(fdmgpu_nscyl* h);
int fdmgpu_nscyl_time_index(fdmgpu_nscyl* h, int* t);
int fdmgpu_nscyl_destroy(fdmgpu_nscyl* h);

/* ---- NBody: particle-mesh gravity around the periodic LaplCube ------------
 * Replaces NBody<T,check,CIC3<T>> of test/nbody.cpp:25-511: the constructor
 * NBody(x0, y0, z0, l, n, npp, N, dt, G, vel, sgn, local, solar, crit, debug)
 * (:97-127, Config keys nbody:{x0, y0, z0, l, n, npp, N, dt, G, vel, sign,
 * local, solar, rcrit}), which draws the bodies (init_points, :515-590);
 * step() = calc_a_pm + move (:134-143); calc_error's pair sum (:145-183).
 * dtype selects T (solver:datatype).  n is the periodic mass grid (a power
 * of two), npp the particle-particle grid, rcrit = (l / npp) * crit.
 * Body arrays are host arrays in T, N x 3 for x, v, a, aprev, F (the
 * reference's Body::x[3] layout) and N for mass. */
typedef struct fdmgpu_nbody fdmgpu_nbody;
enum { FDMGPU_NBODY_DENSITY = 0, FDMGPU_NBODY_RHS = 1, FDMGPU_NBODY_PSI = 2, FDMGPU_NBODY_E = 3 };
int fdmgpu_nbody_create(fdmgpu_nbody** h, int dtype, double x0, double y0, double z0, double l, int n, int npp,
                        int nbodies, double dt, double G, double vel, int sgn, int local, int solar, double crit);
/* body count (10 for the solar set), G (2.96e-6 for the solar set), total
 * mass (double sum in index order) and steps taken; NULL skips */
int fdmgpu_nbody_info(fdmgpu_nbody* h, int* nbodies, double* G, double* total_mass, long long* steps_done);
/* replaces every body; a / aprev may be NULL (zero).  The total mass is
 * re-summed and the cell lists hold the new bodies. */
int fdmgpu_nbody_set_bodies(fdmgpu_nbody* h, const void* x, const void* v, const void* a, const void* aprev,
                            const void* mass);
int fdmgpu_nbody_get_bodies(fdmgpu_nbody* h, void* x, void* v, void* a, void* aprev, void* mass, void* F);
/* steps x (calc_a_pm + move); synchronous.  The _async form only enqueues
 * (one CUDA graph launch per step after the first); fdmgpu_nbody_sync waits. */
int fdmgpu_nbody_step(fdmgpu_nbody* h, int steps);
int fdmgpu_nbody_step_async(fdmgpu_nbody* h, int steps);
int fdmgpu_nbody_sync(fdmgpu_nbody* h);
/* calc_a_pm alone: a = F + PM field.  As in the reference it empties the
 * cell lists, so the next step deposits no mass. */
int fdmgpu_nbody_calc_forces(fdmgpu_nbody* h);
/* calc_error's exact sum F_i = sum_{j != i} sgn m_j G (x_i - x_j) / R^3,
 * R = |x_i - x_j| + 1e-5, into F (N x 3, T) */
int fdmgpu_nbody_direct_forces(fdmgpu_nbody* h, void* F);
/* the grids of the last calc_a_pm: density f, rhs, psi (n^3, x fastest) or
 * E (n^3 x 3) */
int fdmgpu_nbody_get_field(fdmgpu_nbody* h, int field, void* out, size_t count);
int fdmgpu_nbody_destroy(fdmgpu_nbody* h);

#ifdef __cplusplus
}
#endif
#endif /* FDMGPU_H */
