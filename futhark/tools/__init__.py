"""Drop-ins for the reference's validation programs (futhark/tools/*.fut):
``diff``, ``mse`` and ``sanityCheck``, computed on the GPU."""
