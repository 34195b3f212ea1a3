"""Drop-in for the reference module `futhark.backprojection` (program futhark/backprojection.fut:82-93).

Usage as in the reference: ``backprojection.backprojection().main(...).get()``.
"""
from synkrotomo_gb300.dropin import backprojection

__all__ = ["backprojection"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("backprojection"))
