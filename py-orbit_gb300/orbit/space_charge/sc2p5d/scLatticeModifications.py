"""Insertion of 2.5D space-charge nodes
(py/orbit/space_charge/sc2p5d/scLatticeModifications.py:17-47)."""
from orbit.space_charge.sc2p5d.scAccNodes import SC2p5D_AccNode, SC2p5Drb_AccNode
from orbit.space_charge.scLatticeModifications import setSC_General_AccNodes


def setSC2p5DAccNodes(lattice, sc_path_length_min, space_charge_calculator, boundary=None):
    scNodes_arr = setSC_General_AccNodes(lattice, sc_path_length_min, space_charge_calculator, SC2p5D_AccNode)
    for scNode in scNodes_arr:
        scNode.setName(scNode.getName() + "SC2p5D")
        scNode.setBoundary(boundary)
    lattice.initialize()
    return scNodes_arr


def setSC2p5DrbAccNodes(lattice, sc_path_length_min, space_charge_calculator, pipe_radius):
    scNodes_arr = setSC_General_AccNodes(lattice, sc_path_length_min, space_charge_calculator, SC2p5Drb_AccNode)
    for scNode in scNodes_arr:
        scNode.setName(scNode.getName() + "SC2p5Drb")
        scNode.setPipeRadius(pipe_radius)
    lattice.initialize()
    return scNodes_arr
