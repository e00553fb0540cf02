"""Base of nodes that track a bunch (py/orbit/lattice/AccNodeBunchTracker.py)."""
from orbit.lattice.AccActionsContainer import AccActionsContainer
from orbit.lattice.AccNode import AccNode


class AccNodeBunchTracker(AccNode):
    def __init__(self, name="no name", type_in="bunch tracker"):
        AccNode.__init__(self, name, type_in)

    def trackBunch(self, bunch, paramsDict=None, actionContainer=None):
        if paramsDict is None:
            paramsDict = {}
        if actionContainer is None:
            actionContainer = AccActionsContainer("Bunch Tracking")
        paramsDict["bunch"] = bunch

        def track(pd):
            pd["node"].track(pd)

        actionContainer.addAction(track, AccActionsContainer.BODY)
        self.trackActions(actionContainer, paramsDict)
        actionContainer.removeAction(track, AccActionsContainer.BODY)

    def track(self, paramsDict):
        """Each element implements its own map."""
        pass
