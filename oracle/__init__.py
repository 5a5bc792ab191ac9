"""ORACLE -- test infrastructure only.

A CPU restatement of dadi's diffusion-integrator path (the ADI sweeps in C,
the host time loop, grid, initial conditions, from_phi, extrapolation and the
Poisson likelihood in numpy), each function citing the dadi 2.4.3 file:line it
follows.  Only tests/, the smoke check and bench.py's CPU-baseline leg use it,
and only as the checker: the shipped package never imports anything here.

Build the C part with ``make -C oracle`` (``oracle/_build/liboracle.so``).
When the reference tree is present, the same Makefile also compiles the
reference C sweeps from their own sources into ``oracle/_ref/libdadi_ref.so``
so that tests can pin the restatement against them.
"""
