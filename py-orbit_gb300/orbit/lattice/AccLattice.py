"""Accelerator lattice: an ordered list of first-level nodes
(py/orbit/lattice/AccLattice.py)."""
from orbit.lattice.AccActionsContainer import AccActionsContainer
from orbit.lattice.AccNode import AccNode
from orbit.utils import NamedObject, TypedObject, orbitFinalize


class AccLattice(NamedObject, TypedObject):
    ENTRANCE = AccActionsContainer.ENTRANCE
    BODY = AccActionsContainer.BODY
    EXIT = AccActionsContainer.EXIT
    BEFORE = AccActionsContainer.BEFORE
    AFTER = AccActionsContainer.AFTER

    def __init__(self, name="no name"):
        NamedObject.__init__(self, name)
        TypedObject.__init__(self, "lattice")
        self.__length = 0.0
        self.__isInitialized = False
        self.__children = []
        self.__childPositions = {}

    def initialize(self):
        """Initializes nodes, then measures the lattice length and first-level
        node positions with an EXIT action walk (AccLattice.py:33-77)."""
        seen = set()
        for node in self.__children:
            if id(node) in seen:
                orbitFinalize("The AccLattice class instance should not have duplicate nodes! node="
                              + node.getName())
            seen.add(id(node))
            node.initialize()
        actions = AccActionsContainer()
        d = [0.0]
        posn = {}

        def exit_action(pd):
            node = pd["node"]
            if isinstance(pd["parentNode"], AccLattice):
                before = d[0]
                d[0] += node.getLength()
                posn[node] = (before, d[0])

        actions.addAction(exit_action, AccNode.EXIT)
        self.trackActions(actions, {})
        self.__length = d[0]
        self.__childPositions = posn
        self.__isInitialized = True

    def isInitialized(self):
        return self.__isInitialized

    def addNode(self, node, index=-1):
        if isinstance(node, AccNode):
            if index < 0:
                self.__children.append(node)
            else:
                self.__children.insert(index, node)
            self.__isInitialized = False

    def getNodes(self):
        return self.__children

    def setNodes(self, nodes):
        self.__children = nodes

    def getNodeForName(self, name):
        nodes = self.getNodesForName(name)
        if len(nodes) == 1:
            return nodes[0]
        if not nodes:
            return None
        orbitFinalize("AccLattice.getNodeForName found many nodes for name=" + name)

    def getNodesForName(self, name):
        return [n for n in self.__children if n.getName().find(name) == 0]

    def getNodesOfClass(self, cls):
        return [n for n in self.__children if isinstance(n, cls)]

    def getNodesForSubstring(self, sub, no_sub=None):
        out = []
        for n in self.__children:
            nm = n.getName()
            if nm.find(sub) >= 0 and (no_sub is None or nm.find(no_sub) < 0):
                out.append(n)
        return out

    def getNodeIndex(self, node):
        return self.__children.index(node)

    def getNodePositionsDict(self):
        return self.__childPositions

    def getLength(self):
        return self.__length

    def reverseOrder(self):
        self.__children.reverse()
        for node in self.__children:
            node.reverseOrder()
        self.initialize()

    def structureToText(self):
        txt = "==== START ==== Lattice =" + self.getName() + "  L=" + str(self.getLength()) + "\n"
        for node in self.__children:
            txt += node.structureToText("")
        txt += "==== STOP  ==== Lattice =" + self.getName() + "  L=" + str(self.getLength()) + "\n"
        return txt

    def _getSubLattice(self, new, index_start=-1, index_stop=-1):
        if index_start < 0:
            index_start = 0
        if index_stop < 0:
            index_stop = len(self.__children) - 1
        new.setNodes([])
        for node in self.__children[index_start:index_stop + 1]:
            new.addNode(node)
        new.initialize()
        return new

    def getSubLattice(self, index_start=-1, index_stop=-1):
        return self._getSubLattice(AccLattice(), index_start, index_stop)

    def trackActions(self, actionsContainer, paramsDict=None, index_start=-1, index_stop=-1):
        """Walks first-level nodes index_start..index_stop inclusive
        (AccLattice.py:243-255)."""
        if paramsDict is None:
            paramsDict = {}
        paramsDict["lattice"] = self
        paramsDict["actions"] = actionsContainer
        if "path_length" not in paramsDict:
            paramsDict["path_length"] = 0.0
        if index_start < 0:
            index_start = 0
        if index_stop < 0:
            index_stop = len(self.__children) - 1
        for node in self.__children[index_start:index_stop + 1]:
            paramsDict["node"] = node
            paramsDict["parentNode"] = self
            node.trackActions(actionsContainer, paramsDict)
