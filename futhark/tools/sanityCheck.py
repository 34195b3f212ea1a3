"""Drop-in for the reference program `futhark/tools/sanityCheck.fut`.

As a library: ``sanityCheck.sanityCheck().main(sane, test)``.  As an executable, like the
compiled program: ``python -m futhark.tools.sanityCheck < values`` reads the two
arrays in Futhark's value format from standard input and prints the result.
"""
from synkrotomo_gb300.dropin import sanityCheck

__all__ = ["sanityCheck"]

if __name__ == "__main__":
    import sys

    from synkrotomo_gb300.fbench import run_executable

    sys.exit(run_executable("sanityCheck"))
