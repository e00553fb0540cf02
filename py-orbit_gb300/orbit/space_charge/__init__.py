"""Space-charge lattice nodes (py/orbit/space_charge/__init__.py)."""
from orbit.space_charge.scAccNodes import SC_Base_AccNode
from orbit.space_charge.scLatticeModifications import setSC_General_AccNodes

__all__ = ["SC_Base_AccNode", "setSC_General_AccNodes"]
