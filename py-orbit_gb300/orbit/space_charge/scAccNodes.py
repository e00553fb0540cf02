"""Base space-charge node (py/orbit/space_charge/scAccNodes.py)."""
from orbit.lattice import AccNodeBunchTracker


class SC_Base_AccNode(AccNodeBunchTracker):
    """Space-charge node holding a calculator and the path length its kick
    represents."""

    def __init__(self, sc_calculator, name="no name"):
        AccNodeBunchTracker.__init__(self, name)
        self.setType("SC_Base")
        self.sc_length = 0.0
        self.switcher = True
        self.sc_calculator = sc_calculator

    def isRFGap(self):
        return False

    def setLengthOfSC(self, sc_length):
        self.sc_length = sc_length

    def getLengthOfSC(self):
        return self.sc_length

    def setCalculationOn(self, switcher):
        """As in the reference (scAccNodes.py), this leaves the node switched on."""
        self.switcher = True

    def getCalculationOn(self):
        return self.switcher

    def getCalculator(self):
        return self.sc_calculator

    def trackDesign(self, paramsDict):
        pass

    def track(self, paramsDict):
        pass
