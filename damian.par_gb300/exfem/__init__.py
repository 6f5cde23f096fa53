"""exfem_gb300: GB300-native explicit time stepping for damian.par's 2-D Q4 solver."""
from . import abi, decks  # noqa: F401
from .model import Model, write_mass, write_sheet, write_step  # noqa: F401
