"""GB300 (sm_103a) implementation of TeaLeaf's implicit heat-conduction solve.

The product is libtealeaf_gb300.so: hand-written CUDA kernels behind the
C ABI that UK-MAC/TeaLeaf_OpenCL's Fortran driver calls
(include/tealeaf_gb300.h), plus a C++ restatement of that driver.  This
package builds and binds it (lib.py) and writes workload decks (decks.py).
"""
from .lib import (Chunk, Driver, TeaError, load, run_deck, FIELD, PREC,  # noqa: F401
                  SOLVER, DRIVER_PER_CALL, DRIVER_RESIDENT)
from .decks import five_state_deck  # noqa: F401
