"""Drop-in for the reference module `futhark.SIRT` (program futhark/SIRT.fut:43-49).

Usage as in the reference: ``SIRT.SIRT().main(...).get()``.
"""
from synkrotomo_gb300.dropin import SIRT

__all__ = ["SIRT"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("SIRT"))
