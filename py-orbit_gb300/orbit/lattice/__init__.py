"""Accelerator lattice engine (py/orbit/lattice): nodes with ENTRANCE,
BODY (per part, BEFORE/AFTER children) and EXIT stages, walked in the
reference's order."""
from orbit.lattice.AccActionsContainer import AccActionsContainer
from orbit.lattice.AccNode import AccNode
from orbit.lattice.AccLattice import AccLattice
from orbit.lattice.AccNodeBunchTracker import AccNodeBunchTracker

__all__ = ["AccActionsContainer", "AccNode", "AccLattice", "AccNodeBunchTracker"]
