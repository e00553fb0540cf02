"""TEAPOT elements and lattices (py/orbit/teapot/__init__.py)."""
from orbit.teapot.teapot import (TEAPOT_Lattice, TEAPOT_Ring, BaseTEAPOT, BendTEAPOT, DriftTEAPOT,
                                 FringeFieldTEAPOT, KickTEAPOT, MultipoleTEAPOT, QuadTEAPOT, RingRFTEAPOT,
                                 SolenoidTEAPOT, TiltTEAPOT, NodeTEAPOT, BunchWrapTEAPOT, MonitorTEAPOT,
                                 ApertureTEAPOT, TurnCounterTEAPOT, TPB)

__all__ = ["TEAPOT_Lattice", "TEAPOT_Ring", "BaseTEAPOT", "DriftTEAPOT", "BunchWrapTEAPOT", "BendTEAPOT",
           "QuadTEAPOT", "MultipoleTEAPOT", "SolenoidTEAPOT", "KickTEAPOT", "RingRFTEAPOT",
           "FringeFieldTEAPOT", "TiltTEAPOT", "NodeTEAPOT", "MonitorTEAPOT", "ApertureTEAPOT",
           "TurnCounterTEAPOT", "TPB"]
