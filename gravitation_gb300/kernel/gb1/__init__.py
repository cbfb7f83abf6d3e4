# -*- coding: utf-8 -*-

"""GB300 kernel for the gravitation benchmark suite.

Drop-in kernel package: copy (or symlink) this ``gb1`` directory into the reference's
``src/gravitation/kernel/`` and make ``gravitation_gb300`` importable; the reference's
inventory (gravitation/lib/load.py:40-51) then lists it as ``gb1`` and reads the
metadata below by AST without importing it (load.py:77-99), so the assignments stay
plain literals.  ``from .._base_ import universe_base`` resolves to the reference's
base class there and to gravitation_gb300/kernel/_base_.py inside this repository.

Stage 1 and stage 2 run on one GB300 through libgravgb300.so (hand-written sm_103a
CUDA behind a C ABI); see gravitation_gb300.plugin for the options.
"""

__longname__ = 'gb300-backend (1)'
__version__ = '0.1.0'
__description__ = 'GB300 sm_103a CUDA: tiled all-pairs stage 1, FP64 stage 2, C ABI via ctypes'
__requirements__ = ['numpy', 'torch']
__externalrequirements__ = ['cuda']
__interpreters__ = ['python3']
__parallel__ = True
__license__ = 'GPLv2'
__authors__ = [
    'gravitation-gb300 contributors',
]

from .._base_ import universe_base
from gravitation_gb300.plugin import GB300Stages


class universe(GB300Stages, universe_base):
    """universe_base with stage 1 and stage 2 on the GPU (see GB300Stages)."""
