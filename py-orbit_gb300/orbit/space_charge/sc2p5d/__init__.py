"""2.5D space-charge nodes (py/orbit/space_charge/sc2p5d/__init__.py)."""
from orbit.space_charge.sc2p5d.scAccNodes import SC2p5D_AccNode, SC2p5Drb_AccNode
from orbit.space_charge.sc2p5d.scLatticeModifications import setSC2p5DAccNodes, setSC2p5DrbAccNodes

__all__ = ["SC2p5D_AccNode", "SC2p5Drb_AccNode", "setSC2p5DAccNodes", "setSC2p5DrbAccNodes"]
