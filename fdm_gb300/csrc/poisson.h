// Internal interface of the Poisson plans, shared with the NSCube step.
#pragma once

#include <cuda_runtime.h>

#include "../../include/fdmgpu.h"

namespace fdmgpu {

// Solves on device pointers with a plain FP64 LaplCube plan owned by `h`
// (created through fdmgpu_lapl_cube_create).  Throws fdmgpu::Error.
void cube_solve_device(fdmgpu_lapl_cube* h, void* ans, const void* rhs, int nrhs, cudaStream_t st);

// The same for a LaplCyl3FFT2 plan (fdmgpu_lapl_cyl_create), used by NSCyl.
void cyl_solve_device(fdmgpu_lapl_cyl* h, void* ans, const void* rhs, int nrhs, cudaStream_t st);

}  // namespace fdmgpu
