"""GB300-native ghost-cell MAC AB2/CN cylinder-flow step (drop-in for the reference's ghost path).

The compute lives in libghostmac.so (CUDA for sm_103a, C ABI in include/ghostmac.h);
``ghost.MAC_CylinderFlow`` mirrors the reference's ``MAC_CylinderFlow`` for
``boundary='ghost_cell', time_scheme='ab2_cn'``.
"""
from .build import build  # noqa: F401
from . import _lib  # noqa: F401  (loads libghostmac.so; fails loudly if missing)
from .ghost import CylinderBatch, GhostCellIntegrator, MAC_CylinderFlow  # noqa: F401
from .cutcell import CutCellFlow  # noqa: F401
from .staircase import LegacyGhostFlow, StaircaseFlow  # noqa: F401
from . import analysis, learned, taylor_green, validation  # noqa: F401

__all__ = ['MAC_CylinderFlow', 'GhostCellIntegrator', 'CylinderBatch', 'CutCellFlow', 'StaircaseFlow', 'LegacyGhostFlow', 'taylor_green', 'analysis', 'learned',
           'validation', 'build']
