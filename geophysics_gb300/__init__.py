"""GB300-native finite-difference hot path of liaman/Geophysics.

The compute lives in libgeofd.so (CUDA kernels for sm_103a behind a C ABI,
include/geofd.h).  This package is the host-side mirror of the reference's
entry points:

  GPU_vti2dfd, CPU_vti2dfd, GPU_vti3dfd   file-based drop-ins (same arguments)
  fd2d_shot, FD3DPlan, fd3d_shot          array-level forward modelling
  tti2d_shot                              2D TTI forward modelling
  rtm2d_batch                             batched 2D RTM (MPI-program semantics)
  rtm3d                                   3D RTM: boundary-saving, snapshot or learned-codec
  Codec                                   learned snapshot codec (train / encode / decode)
  laplace2d, laplace3d                    adjoint Laplacian image filter
  read_par                                `key= value` par files

Arrays: numpy arrays are host buffers; torch CUDA tensors are device
buffers and run on torch's current CUDA stream.
"""
from ._lib import (GEO_MEM_DEVICE, GEO_MEM_HOST, GEO_MODE_EXACT, GEO_MODE_FAST, GEO_VARIANT_CPU,
                   GEO_VARIANT_GPU, GEO_VARIANT_MPI, GeoError, lib)
from .api import (CPU_vti2dfd, FD3DPlan, GPU_vti2dfd, GPU_vti3dfd, fd2d_shot, fd3d_shot, laplace2d, laplace3d,
                  launch_count, read_par, rtm2d_batch, rtm3d, version, Codec, morton_order, tc_gemm_bf16, tti2d_shot,
                  su_read, su_write, su_replace_data, rtm2d_gpu, rtm2d_tti,
                  smooth2d, adcig_smooth_stack, mute_direct, smooth_model2d, smooth_model3d, fd2d_par, fd3d_par, rtm2d_par)

__all__ = ["GPU_vti2dfd", "CPU_vti2dfd", "GPU_vti3dfd", "fd2d_shot", "FD3DPlan", "fd3d_shot", "rtm2d_batch", "rtm2d_gpu", "rtm2d_tti", "smooth2d", "adcig_smooth_stack", "mute_direct", "smooth_model2d", "smooth_model3d", "fd2d_par", "fd3d_par", "rtm2d_par", "rtm3d", "tti2d_shot", "su_read", "su_write", "su_replace_data", "Codec", "morton_order", "tc_gemm_bf16",
           "laplace2d", "laplace3d", "read_par", "launch_count", "version", "lib", "GeoError",
           "GEO_MEM_HOST", "GEO_MEM_DEVICE", "GEO_VARIANT_CPU", "GEO_VARIANT_GPU", "GEO_VARIANT_MPI",
           "GEO_MODE_EXACT", "GEO_MODE_FAST"]
