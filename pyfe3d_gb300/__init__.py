r"""
pyfe3d_gb300: GB300-native element assembly and static solve for pyfe3d
=======================================================================

Drop-in for pyfe3d's Quad4/BeamC element path (and the reduced-integration
Tria3R/Quad4R shells).  The element classes keep the
reference API (``update_rotation_matrix``, ``update_probe_xe``,
``update_probe_ue``, ``update_KC0``/``update_KG``/``update_M`` writing the
caller's COO arrays at the ``*Data`` offsets); every computation runs in
hand-written sm_103a kernels of ``libfe3d_gb300.so``.
"""
import ctypes

import numpy as np

from .beamc import BeamC, BeamCData, BeamCProbe
from .quad4 import Quad4, Quad4Data, Quad4Probe
from .quad4r import Quad4R, Quad4RData, Quad4RProbe
from .shellprop import BeamProp, ShellProp
from .tria3r import Tria3R, Tria3RData, Tria3RProbe

__version__ = '0.1.0'

DOF = 6
if ctypes.sizeof(ctypes.c_long) == 8:
    INT = np.int64
else:
    INT = np.int32
DOUBLE = np.float64

__all__ = ['Quad4', 'Quad4Data', 'Quad4Probe', 'Quad4R', 'Quad4RData', 'Quad4RProbe', 'Tria3R',
           'Tria3RData', 'Tria3RProbe', 'BeamC', 'BeamCData', 'BeamCProbe', 'ShellProp', 'BeamProp', 'DOF',
           'INT', 'DOUBLE']
