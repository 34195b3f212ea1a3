"""Drop-in replacement for synkrotomo's ``futhark`` package (setup.py:8).

Modules and classes keep the reference's names:
``from futhark import SIRT; SIRT.SIRT().main(theta, rhozero, deltarho,
emptyimage, sinogram, iterations).get()`` (README.md:21-25), likewise
``forwardprojection``, ``backprojection``, their ``_sparse`` variants and
``SIRT3D``.  The computation runs on libsynk's sm_103a CUDA kernels.
"""
