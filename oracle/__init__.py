"""CPU oracle (test infrastructure): numpy complex128 restatement of the
reference's Lindblad RK4 path.  Imported only by tests, the smoke check and
the benchmark's CPU-baseline leg."""
