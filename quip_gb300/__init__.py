"""quip_gb300: GB300-native GAP energy/force/virial evaluation behind QUIP's Potential API."""
from .atoms import Atoms, read_xyz, write_xyz  # noqa: F401
