// Internal interface of the Poisson plans, shared with the NSCube step.
#pragma once

#include <cuda_runtime.h>

#include "../../include/fdmgpu.h"

namespace fdmgpu {

// Solves on device pointers with a plain FP64 LaplCube plan owned by `h`
// (created through fdmgpu_lapl_cube_create).  Throws fdmgpu::Error.
void cube_solve_device(fdmgpu_lapl_cube* h, void* ans, const void* rhs, int nrhs, cudaStream_t st);

// Plain FP64 solve of nvol volumes addressed through device arrays of
// pointers (d_in[i] -> d_out[i]) with the plan of `h`; scratch: nvol FP64
// work volumes on the device, or null for the plan's own (which then grows
// to nvol volumes).  Throws fdmgpu::Error.
void cube_solve_ptrs(fdmgpu_lapl_cube* h, const void* const* d_in, void* const* d_out, int nvol, double* scratch,
                     cudaStream_t st);

// The line transforms of the plan choose their CTA size as if a solve had
// `vols` volumes (0: its own count), so that results do not depend on how
// many volumes share a launch.
void cube_set_rule_volumes(fdmgpu_lapl_cube* h, int vols);

// Queues on st a copy of the refinement norms of the plan's last solve of
// nrhs right-hand sides into host memory (2 * nrhs * sweeps doubles, page
// locked for the copy to be asynchronous); returns the sweeps of that solve
// (0: none, -1: solved in FP64; nothing is copied then).
int cube_norms_async(fdmgpu_lapl_cube* h, double* host, int nrhs, cudaStream_t st);

// The estimated remaining relative error of each of the nrhs right-hand
// sides from such a copy (fdmgpu_lapl_cube_last_info's model; -1 when no
// sweep ran).  Host arithmetic only.
void cube_estimates(const fdmgpu_lapl_cube* h, const double* norms_host, int sweeps, int nrhs, double* est);

// Resident NSCube cavities (fdmgpu_nscube_create, FP64) stepped together:
// nscube_mergeable says whether two can share launches (the same grid, box
// and form of the quotients); nscube_step_many advances cavity i by
// steps[i] steps on st, all of them in shared launches (round r steps those
// with more than r steps left), with the kernels and transform CTA sizes of
// a single cavity's step, so every field comes out as it would alone.  The
// caller orders st after each cavity's earlier work.  Throws fdmgpu::Error.
bool nscube_mergeable(const fdmgpu_nscube* a, const fdmgpu_nscube* b);
// pool: where the tables and work volumes of the shared steps come from
// (stream-ordered; null = the device's default pool)
void nscube_step_many(fdmgpu_nscube* const* hs, const int* steps, int n, cudaStream_t st,
                      cudaMemPool_t pool = nullptr);

// The same for a LaplCyl3FFT2 plan (fdmgpu_lapl_cyl_create), used by NSCyl.
void cyl_solve_device(fdmgpu_lapl_cyl* h, void* ans, const void* rhs, int nrhs, cudaStream_t st);

}  // namespace fdmgpu
