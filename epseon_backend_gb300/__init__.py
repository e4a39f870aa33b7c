"""GB300-native vibrational-level solver behind epseon_backend's device/task API.

Layout:
  include/epscu.h            C ABI of libepseon_cuda (the drop-in boundary)
  csrc/*.cu                  sm_103a kernels + host orchestration (libepseon_cuda.so)
  csrc/host/                 C++ device/task object model + pybind11 module
  device/cuda/               ``_libepseon_cuda`` (mirror of ``_libepseon_gpu``)
  capi.py                    ctypes view of the C ABI
  autograd.py                torch.autograd.Function over the adjoint
  synth.py                   seeded synthetic workloads
"""
__version__ = "0.1.0"
