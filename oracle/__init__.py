"""Oracle for synkrotomo's projection + SIRT path.

TEST INFRASTRUCTURE ONLY. Nothing in the product (the ``synkrotomo_gb300``
package, the ``futhark`` drop-in package, the CUDA library) imports, links or
executes anything in this directory.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` use it, and only as the checker or the timed CPU stand-in
for the reference.

Two restatements of the reference's Futhark programs live here:

* ``fut_ref``  -- FP64 NumPy restatement (the accuracy judge).
* ``cpu_ref.c`` -- FP32 C + OpenMP line-by-line restatement (the reference's
  FP32 behaviour and the timed CPU baseline), loaded through ``cpu_ref.py``.

Parity pin: the reference ships no expected outputs for FP/BP/SIRT.  What pins
these restatements are the reference's own known-answer tests in
``archive/line_lib.fut:1-57`` (eight chord-length cases) and
``archive/projection_lib.fut:1-41`` (four first-detector index cases); see
``tests/test_oracle_kats.py``.
"""
