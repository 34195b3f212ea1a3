"""Drop-in for the reference program `futhark/tools/diff.fut`.

As a library: ``diff.diff().main(sane, test)``.  As an executable, like the
compiled program: ``python -m futhark.tools.diff < values`` reads the two
arrays in Futhark's value format from standard input and prints the result.
"""
from synkrotomo_gb300.dropin import diff

__all__ = ["diff"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("diff"))
