"""lbm_gb300: GB300-native D2Q9 TRT lattice update with the jviquerat/lbm API.

* ``lattice``      drop-in for lbm/src/core/lattice.py (device-resident).
* ``run``          driver of lbm/src/core/run.py with the fused engine.
* ``apps``         cavity, turek, poiseuille, array, step, obstacle_array.
* ``engine``       fused pull-scheme engine over liblbm_gb300 (C-ABI in
                   include/lbm_gb300.h).
"""
from .lattice import lattice
from .run import run, run_methods, run_fused
from .obstacle import obstacle
from .buff import buff
from .apps import app_factory

__all__ = ["lattice", "run", "run_methods", "run_fused", "obstacle", "buff", "app_factory"]
