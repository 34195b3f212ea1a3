"""synkrotomo_gb300: GB300-native (sm_103a) parallel-beam projection and SIRT.

Layers:
  csrc/        CUDA kernels and the C ABI of libsynk.so (include/synk.h)
  build.py     nvcc build of libsynk.so
  _lib.py      ctypes binding of the C ABI (no CPU fallback)
  runtime.py   contexts on torch streams, device arrays, argument checks
  dropin.py    the classes of the ``futhark`` drop-in package
  phantom.py   seeded synthetic phantoms and geometries
"""
__version__ = "0.1.0"
