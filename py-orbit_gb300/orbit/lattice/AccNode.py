"""Accelerator node with parts and child nodes (py/orbit/lattice/AccNode.py).

A node has ENTRANCE children, a BODY split into nParts parts (each with
BEFORE and AFTER children) and EXIT children.  ``trackActions`` walks them in
the reference's order (AccNode.py:302-350); the space-charge nodes sit as
BODY/BEFORE children, so the order of maps and kicks is fixed here.
"""
import math
import os

from orbit.lattice.AccActionsContainer import AccActionsContainer
from orbit.utils import NamedObject, ParamsDictObject, TypedObject, orbitFinalize

# ORBIT_NVTX=1: one NVTX range per node walked (orbit_nvtx_push/pop), shown
# by Nsight Systems and usable as an ncu --nvtx filter.
_NVTX = os.environ.get("ORBIT_NVTX", "0") == "1"


def _nvtx_push(name):
    from orbit_gb300 import call
    call("orbit_nvtx_push", str(name).encode())


def _nvtx_pop():
    from orbit_gb300 import call
    call("orbit_nvtx_pop")


class AccNode(NamedObject, TypedObject, ParamsDictObject):
    ENTRANCE = AccActionsContainer.ENTRANCE
    BODY = AccActionsContainer.BODY
    EXIT = AccActionsContainer.EXIT
    BEFORE = AccActionsContainer.BEFORE
    AFTER = AccActionsContainer.AFTER

    def __init__(self, name="no name", type_in="generic"):
        NamedObject.__init__(self, name)
        TypedObject.__init__(self, type_in)
        ParamsDictObject.__init__(self)
        self.__nParts = 1
        self.__lengthArr = [0.0]
        self.__length = 0.0
        self.__activePartIndex = 0
        # [entrance children, body parts [[before], [after]] ..., exit children]
        self.__children = [[], [[[], []]], []]
        self._setPartsLengthEvenly(self.__nParts)

    # ------------------------------------------------------------ parts
    def setnParts(self, n=1):
        if self.getNumberOfBodyChildren() != 0:
            orbitFinalize("You cannot set the number of AccNode parts after you added children! node="
                          + self.getName())
        self._setPartsLengthEvenly(n)
        self.initialize()

    def getnParts(self):
        return self.__nParts

    def setLength(self, L=0.0, index=-1):
        L = float(L)
        if math.fabs(L) < 1.0e-36:
            L = 0.0
        if index >= 0:
            self.__lengthArr[index] = L
            return
        self.__length = L
        self._setPartsLengthEvenly(self.__nParts)
        self.initialize()

    def getLength(self, index=-1):
        if index >= 0:
            return self.__lengthArr[index]
        return self.__length

    def getActivePartIndex(self):
        return self.__activePartIndex

    def setActivePartIndex(self, i):
        self.__activePartIndex = i

    def _setPartsLengthEvenly(self, n=1):
        if self.getNumberOfBodyChildren() != 0:
            orbitFinalize("AccNode._setPartsLengthEvenly would remove existing body children; node="
                          + self.getName())
        self.__nParts = n
        self.__lengthArr = [self.__length / self.__nParts for _ in range(self.__nParts)]
        self.__children[AccNode.BODY] = [[[], []] for _ in range(self.__nParts)]

    def initialize(self):
        """Overridden by elements whose parts are not of equal length."""
        pass

    # ---------------------------------------------------------- children
    def getNumberOfChildren(self):
        n = len(self.__children[0]) + len(self.__children[2])
        return n + self.getNumberOfBodyChildren()

    def getNumberOfBodyChildren(self):
        n = 0
        for part in self.__children[1]:
            n += len(part[0]) + len(part[1])
        return n

    def addChildNode(self, node, place, part_index=0, place_in_part=AccActionsContainer.BEFORE):
        if place == AccNode.ENTRANCE or place == AccNode.EXIT:
            nodes = self.__children[place]
        elif place == AccNode.BODY:
            nodes = self.__children[place][part_index][place_in_part]
        else:
            orbitFinalize("AccNode.addChildNode: place should be ENTRANCE, BODY or EXIT")
        nodes.append(node)

    def getChildNodes(self, place, part_index=0, place_in_part=AccActionsContainer.BEFORE):
        if place == AccNode.ENTRANCE or place == AccNode.EXIT:
            return self.__children[place]
        return self.__children[place][part_index][place_in_part]

    def getBodyChildren(self):
        nodes = []
        for part in self.__children[1]:
            nodes += part[0]
            nodes += part[1]
        return nodes

    def getAllChildren(self):
        return (self.getChildNodes(AccNode.ENTRANCE) + self.getBodyChildren()
                + self.getChildNodes(AccNode.EXIT))

    def reverseOrder(self):
        self.__lengthArr.reverse()
        self.__children.reverse()
        self.__children[AccNode.ENTRANCE].reverse()
        self.__children[AccNode.EXIT].reverse()
        for node in self.__children[AccNode.ENTRANCE] + self.__children[AccNode.EXIT]:
            node.reverseOrderNodeSpecific()
        self.__children[AccNode.BODY].reverse()
        for part in self.__children[AccNode.BODY]:
            part.reverse()
            part[AccNode.BEFORE].reverse()
            part[AccNode.AFTER].reverse()
            for node in part[AccNode.BEFORE] + part[AccNode.AFTER]:
                node.reverseOrderNodeSpecific()
        self.reverseOrderNodeSpecific()

    def reverseOrderNodeSpecific(self):
        pass

    def structureToText(self, txt="", txt_shift=""):
        sh = " "
        txt += txt_shift + "==== START AccNode = " + self.getName() + " L=" + str(self.getLength()) + "\n"
        txt += txt_shift + sh + "==== ENTRANCE\n"
        for node in self.getChildNodes(AccNode.ENTRANCE):
            txt = node.structureToText(txt, txt_shift + sh * 2)
        txt += txt_shift + sh * 2 + "==== BODY ENTRANCE n parts =" + str(self.getnParts()) + "\n"
        for ind in range(self.getnParts()):
            txt += txt_shift + sh * 3 + "==== BODY Part ind.=" + str(ind) + " L=" + str(self.getLength(ind)) + "\n"
            txt += txt_shift + sh * 4 + "==== BEFORE\n"
            for node in self.getChildNodes(AccNode.BODY, ind, AccNode.BEFORE):
                txt = node.structureToText(txt, txt_shift + sh * 5)
            txt += txt_shift + sh * 4 + "==== AFTER \n"
            for node in self.getChildNodes(AccNode.BODY, ind, AccNode.AFTER):
                txt = node.structureToText(txt, txt_shift + sh * 5)
        txt += txt_shift + sh * 2 + "==== BODY EXIT     n parts =" + str(self.getnParts()) + "\n"
        txt += txt_shift + sh + "==== EXIT\n"
        for node in self.getChildNodes(AccNode.EXIT):
            txt = node.structureToText(txt, txt_shift + sh * 2)
        txt += txt_shift + "==== END of AccNode = " + self.getName() + "\n"
        return txt

    # --------------------------------------------------------- traversal
    def trackActions(self, actionsContainer, paramsDict=None):
        """Entrance actions, entrance children, then per part: BEFORE
        children, body actions, AFTER children; then exit children and exit
        actions (AccNode.py:302-350).  The lattice walk records a device
        program on every trackBunch, so the common case is kept short: a
        plain AccActionsContainer's action lists are run in place (a
        subclass's performActions is called as usual), and the node and
        parent entries are rewritten only where a child walk changed them."""
        if paramsDict is None:
            paramsDict = {}
        if _NVTX:
            _nvtx_push(self.getName())
        plain = type(actionsContainer) is AccActionsContainer
        if plain:
            ent_a, body_a, exit_a = actionsContainer.actionLists()
        paramsDict["node"] = self
        parentNode = paramsDict.get("parentNode")
        if "path_length" not in paramsDict:
            paramsDict["path_length"] = 0.0
        has_length = self.getLength() > 0.0
        self.__activePartIndex = -1
        if plain:
            for action in ent_a:
                action(paramsDict)
        else:
            actionsContainer.performActions(paramsDict, AccNode.ENTRANCE)
        children = self.__children
        for node in children[AccNode.ENTRANCE]:
            paramsDict["node"] = node
            paramsDict["parentNode"] = self
            node.trackActions(actionsContainer, paramsDict)
        body_children = children[AccNode.BODY]
        for i in range(self.__nParts):
            paramsDict["node"] = self
            paramsDict["parentNode"] = parentNode
            self.__activePartIndex = i
            part = body_children[i]
            before = part[AccNode.BEFORE]
            if before:
                for node in before:
                    paramsDict["parentNode"] = self
                    node.trackActions(actionsContainer, paramsDict)
                paramsDict["node"] = self
                paramsDict["parentNode"] = parentNode
            if plain:
                for action in body_a:
                    action(paramsDict)
            else:
                actionsContainer.performActions(paramsDict, AccNode.BODY)
            if has_length:
                paramsDict["path_length"] += self.getLength(i)
            for node in part[AccNode.AFTER]:
                paramsDict["parentNode"] = self
                node.trackActions(actionsContainer, paramsDict)
        self.__activePartIndex = -1
        for node in children[AccNode.EXIT]:
            paramsDict["node"] = node
            paramsDict["parentNode"] = self
            node.trackActions(actionsContainer, paramsDict)
        paramsDict["node"] = self
        paramsDict["parentNode"] = parentNode
        if plain:
            for action in exit_a:
                action(paramsDict)
        else:
            actionsContainer.performActions(paramsDict, AccNode.EXIT)
        if _NVTX:
            _nvtx_pop()
