"""fdm_gb300 — GB300 (sm_103a) fast Poisson solver and NSCube projection step.

A drop-in for resetius/fdm's LaplCube / LaplRect / LaplRectFFT2 solve() and
NSCube::step(): the same constructors, array layouts and results, computed by
hand-written CUDA kernels in libfdmgpu.so (C ABI: include/fdmgpu.h).
"""
from ._native import FdmError, load as load_library, LIB_PATH, MAX_N  # noqa: F401
from .config import Config  # noqa: F401
from .lapl import (BatchSolver, LaplCube, LaplCyl3FFT2, LaplRect, LaplRectFFT2, pfft3d_device, pfft_1_3d,  # noqa: F401
                   pfft_3d, pfft_device, sine_transform_device, sine_transform_tc_device, tridiag_device)  # noqa: F401
from .nbody import NBody  # noqa: F401
from .ns_cube import NSCube, NSCyl, Tensor3  # noqa: F401
from .serve import Server  # noqa: F401
