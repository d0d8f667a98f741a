"""GB300-native time stepping for the 2-D velocity-stress Biot poroelastic
finite-difference simulator (drop-in for the TIME_LOOP of
David011/2D-VQSP-FD-Sim).

The compute path is the CUDA engine behind the C ABI in ``include/fdp.h``
(``libfdp.so``, built in-tree by :mod:`fdporo.build`); this package is its
Python host: the ctypes binding (:mod:`fdporo.native`), a host mirror of the
reference's time-loop seam (:mod:`fdporo.engine`), the shot set-up in the
reference's order (:mod:`fdporo.job`), synthetic media (:mod:`fdporo.media`)
and the reference's output formats (:mod:`fdporo.formats`).
"""
from .engine import Engine
from .native import FdpError, load

__all__ = ["Engine", "FdpError", "load"]
