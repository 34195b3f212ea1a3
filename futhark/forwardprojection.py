"""Drop-in for the reference module `futhark.forwardprojection` (program futhark/forwardprojection.fut:71-84).

Usage as in the reference: ``forwardprojection.forwardprojection().main(...).get()``.
"""
from synkrotomo_gb300.dropin import forwardprojection

__all__ = ["forwardprojection"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("forwardprojection"))
