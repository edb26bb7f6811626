// Internal interface of the Poisson plans, shared with the NSCube step.
#pragma once

#include <cuda_runtime.h>

#include "../../include/fdmgpu.h"

namespace fdmgpu {

// Solves on device pointers with a plain FP64 LaplCube plan owned by `h`
// (created through fdmgpu_lapl_cube_create).  Throws fdmgpu::Error.
void cube_solve_device(fdmgpu_lapl_cube* h, void* ans, const void* rhs, int nrhs, cudaStream_t st);

// Queues on st a copy of the refinement norms of the plan's last solve of
// nrhs right-hand sides into host memory (2 * nrhs * sweeps doubles, page
// locked for the copy to be asynchronous); returns the sweeps of that solve
// (0: none, -1: solved in FP64; nothing is copied then).
int cube_norms_async(fdmgpu_lapl_cube* h, double* host, int nrhs, cudaStream_t st);

// The estimated remaining relative error of each of the nrhs right-hand
// sides from such a copy (fdmgpu_lapl_cube_last_info's model; -1 when no
// sweep ran).  Host arithmetic only.
void cube_estimates(const fdmgpu_lapl_cube* h, const double* norms_host, int sweeps, int nrhs, double* est);

// The same for a LaplCyl3FFT2 plan (fdmgpu_lapl_cyl_create), used by NSCyl.
void cyl_solve_device(fdmgpu_lapl_cyl* h, void* ans, const void* rhs, int nrhs, cudaStream_t st);

}  // namespace fdmgpu
