"""quip_gb300: GB300-native GAP energy/force/virial evaluation behind QUIP's Potential API."""
from .atoms import Atoms, read_xyz, write_xyz  # noqa: F401
from .potential import Potential  # noqa: F401  (libgapgpu.so is loaded on first use)
