"""Container of actions performed at node entrance, body and exit
(py/orbit/lattice/AccActionsContainer.py)."""
from orbit.utils import NamedObject


class AccActionsContainer(NamedObject):
    ENTRANCE = 0
    BODY = 1
    EXIT = 2
    BEFORE = 0
    AFTER = 1

    def __init__(self, name="no name container"):
        NamedObject.__init__(self, name)
        self.__actions = ([], [], [])

    def addAction(self, action, place):
        self.__actions[place].append(action)

    def removeAction(self, action, place):
        self.__actions[place].remove(action)

    def getActions(self, place):
        return self.__actions[place]

    def actionLists(self):
        """The (entrance, body, exit) action lists themselves (run in place
        by AccNode.trackActions)."""
        return self.__actions

    def performActions(self, paramsDict, place):
        for action in self.__actions[place]:
            action(paramsDict)
