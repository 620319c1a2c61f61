"""CPU oracle for the MAC mr-SAV stage hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy/SciPy, the reference algorithm of
HaifengWang1031/MAC-mr-SAV-RK for the no-slip MAC model with the tensor
(DST/DCT + pressure Schur-CG) Stokes backend and the mr-SAV SDIRK schemes.
It is the checker the CUDA path is compared against: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product package never imports it and
has no CPU fallback.

Parity is pinned: ``tests/golden/make_golden.py`` imports the reference
itself (with an identity ``numba.njit`` stand-in, because numba is not
installed) and stores its outputs as fixtures under ``tests/golden/``;
``tests/test_oracle_golden.py`` checks this restatement against them.
"""
from .mac_oracle import *  # noqa: F401,F403
