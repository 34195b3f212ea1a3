"""Drop-in for the reference module `futhark.SIRT3D` (program futhark/SIRT3D.fut:18-29).

Usage as in the reference: ``SIRT3D.SIRT3D().main(...).get()``.
"""
from synkrotomo_gb300.dropin import SIRT3D

__all__ = ["SIRT3D"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("SIRT3D"))
