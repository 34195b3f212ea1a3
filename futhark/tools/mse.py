"""Drop-in for the reference program `futhark/tools/mse.fut`.

As a library: ``mse.mse().main(sane, test)``.  As an executable, like the
compiled program: ``python -m futhark.tools.mse < values`` reads the two
arrays in Futhark's value format from standard input and prints the result.
"""
from synkrotomo_gb300.dropin import mse

__all__ = ["mse"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("mse"))
