"""Drop-in for the reference module `futhark.forwardprojection` (program futhark/forwardprojection.fut:71-84).

Usage as in the reference: ``forwardprojection.forwardprojection().main(...).get()``.
"""
from synkrotomo_gb300.dropin import forwardprojection

__all__ = ["forwardprojection"]
