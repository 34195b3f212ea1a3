"""Drop-in for the reference module `futhark.backprojection_sparse` (program futhark/backprojection_sparse.fut:26-37).

Usage as in the reference: ``backprojection_sparse.backprojection_sparse().main(...).get()``.
"""
from synkrotomo_gb300.dropin import backprojection_sparse

__all__ = ["backprojection_sparse"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("backprojection_sparse"))
