"""Drop-in for the reference module `futhark.SIRT3D` (program futhark/SIRT3D.fut:18-29).

Usage as in the reference: ``SIRT3D.SIRT3D().main(...).get()``.
"""
from synkrotomo_gb300.dropin import SIRT3D

__all__ = ["SIRT3D"]
