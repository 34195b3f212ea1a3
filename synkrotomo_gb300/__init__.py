"""synkrotomo_gb300: GB300-native (sm_103a) parallel-beam projection and SIRT.

Layers:
  csrc/        CUDA kernels and the C ABI of libsynk.so (include/synk.h)
  build.py     nvcc build of libsynk.so
  _lib.py      ctypes binding of the C ABI (no CPU fallback)
  runtime.py   contexts on torch streams, device arrays, argument checks
  dropin.py    the classes of the ``futhark`` drop-in package
  phantom.py   seeded synthetic phantoms and geometries
  autotune.py  launch shape and SIRT engine per size bucket, measured and cached
  shard.py     independent slices / problems split over ranks (one process per GPU)
  unet.py      the U-Net on the tcgen05 kernels; warmstart.py its training and use as a SIRT start
  fvalues.py   Futhark's value format; fbench.py ``futhark bench``-style timing and datasets
"""
__version__ = "0.1.0"
