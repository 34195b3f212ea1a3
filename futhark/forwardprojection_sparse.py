"""Drop-in for the reference module `futhark.forwardprojection_sparse` (program futhark/forwardprojection_sparse.fut:26-40).

Usage as in the reference: ``forwardprojection_sparse.forwardprojection_sparse().main(...).get()``.
"""
from synkrotomo_gb300.dropin import forwardprojection_sparse

__all__ = ["forwardprojection_sparse"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("forwardprojection_sparse"))
