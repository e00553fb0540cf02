"""2.5D space-charge node (py/orbit/space_charge/sc2p5d/scAccNodes.py:15-51)."""
from orbit.space_charge.scAccNodes import SC_Base_AccNode


class SC2p5D_AccNode(SC_Base_AccNode):
    """Calls SpaceChargeCalc2p5D.trackBunch(bunch, sc_length[, boundary])."""

    def __init__(self, sc_calculator, name="no name"):
        SC_Base_AccNode.__init__(self, sc_calculator, name)
        self.setType("SC2p5D")
        self.boundary = None

    def setBoundary(self, boundary):
        self.boundary = boundary

    def getBoundary(self):
        return self.boundary

    def track(self, paramsDict):
        if self.switcher is not True:
            return
        bunch = paramsDict["bunch"]
        if self.boundary is not None:
            self.sc_calculator.trackBunch(bunch, self.sc_length, self.boundary)
        else:
            self.sc_calculator.trackBunch(bunch, self.sc_length)


class SC2p5Drb_AccNode(SC_Base_AccNode):
    """Calls SpaceChargeCalc2p5Drb.trackBunch(bunch, sc_length, pipe_radius)
    (py/orbit/space_charge/sc2p5d/scAccNodes.py:53-84)."""

    def __init__(self, sc_calculator, name="no name"):
        SC_Base_AccNode.__init__(self, sc_calculator, name)
        self.setType("SC2p5Drb")
        self.pipe_radius = 1.0

    def setPipeRadius(self, pipe_radius):
        self.pipe_radius = pipe_radius

    def getPipeRadius(self):
        return self.pipe_radius

    def track(self, paramsDict):
        if self.switcher is not True:
            return
        bunch = paramsDict["bunch"]
        self.sc_calculator.trackBunch(bunch, self.sc_length, self.pipe_radius)
