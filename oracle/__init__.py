"""CPU oracle for the MFI mining path -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  It is the checker the CUDA engine is
compared against (and the CPU arm that is timed beside it), never a code path
of the engine: the engine has no CPU fallback.

``mfi_oracle.c`` restates the reference's arithmetic in plain C; ``oracle.py``
loads it through ctypes and restates the reference's threshold rules and the
two engines' root/stage semantics on top of it.
"""
from .oracle import *  # noqa: F401,F403
