"""TEAPOT lattices and elements (py/orbit/teapot/teapot.py).

The node classes keep the reference's names, parameters and per-part map
schedules (drift teapot.py:548-566, multipole :685-823, quad :825-976,
bend :978-1151, kick :1184-1256, tilt/fringe :1258-1377).  Tracking a
``TEAPOT_Lattice`` records the walk once into a device program and replays it
with fused GPU passes (orbit.teapot.recording); a lattice whose nodes need the
coordinates on the host runs node by node.
"""
from __future__ import annotations

from bunch import BunchTwissAnalysis
from orbit.lattice import AccActionsContainer, AccLattice, AccNode, AccNodeBunchTracker
from orbit.teapot.recording import BunchRecorder, FusedProgram, NotRecordable, is_device_bunch
from orbit.teapot_base import TPB
from orbit.utils import orbitFinalize


class TEAPOT_Lattice(AccLattice):
    """Shell class for the TEAPOT nodes collection."""

    def __init__(self, name="no name"):
        AccLattice.__init__(self, name)
        self.useCharge = 1
        self._fused = True
        self._programs = {}

    def readMAD(self, mad_file_name, lineName):
        raise NotImplementedError("MAD parsing is outside the GPU hot path")

    def readMADX(self, madx_file_name, seqName):
        raise NotImplementedError("MADX parsing is outside the GPU hot path")

    def _addChildren(self):
        pass

    def initialize(self):
        AccLattice.initialize(self)
        ringRF = RingRFTEAPOT()
        for node in self.getNodes():
            if node.getType() == ringRF.getType():
                node.getParamsDict()["ring_length"] = self.getLength()
        self._programs = {}

    def getSubLattice(self, index_start=-1, index_stop=-1):
        new = self._getSubLattice(TEAPOT_Lattice(), index_start, index_stop)
        new.setUseRealCharge(self.getUseRealCharge())
        return new

    def setFusedTracking(self, fused=True):
        """Fused device programs (default) or one kernel per map call."""
        self._fused = bool(fused)

    def getFusedTracking(self):
        return self._fused

    def _program(self, bunch, paramsDict, index_start, index_stop):
        rec = BunchRecorder(bunch)
        pd = dict(paramsDict)
        pd["bunch"] = rec
        pd["useCharge"] = self.useCharge
        container = AccActionsContainer("Bunch Recording")

        def track(p):
            p["node"].track(p)

        container.addAction(track, AccActionsContainer.BODY)
        try:
            self.trackActions(container, pd, index_start, index_stop)
        except NotRecordable:
            return None
        key = (tuple(rec.ops), tuple(id(c) for c in rec.calcs), tuple(id(f) for f in rec.host_ops))
        prog = self._programs.get(key)
        if prog is None:
            if len(self._programs) > 16:
                self._programs.clear()
            prog = FusedProgram(rec.ops, rec.calcs, rec.host_ops, rec.boundaries)
            self._programs[key] = prog
        return prog

    def trackBunch(self, bunch, paramsDict=None, actionContainer=None, index_start=-1, index_stop=-1):
        """Tracks the bunch through nodes index_start..index_stop inclusive
        (teapot.py:127-143)."""
        if paramsDict is None:
            paramsDict = {}
        if actionContainer is None and self._fused and is_device_bunch(bunch):
            bunch._device_bunch(wait=False)  # the upload overlaps the walk
            prog = self._program(bunch, paramsDict, index_start, index_stop)
            if prog is not None:
                prog.run(bunch, 1)
                return
        if actionContainer is None:
            actionContainer = AccActionsContainer("Bunch Tracking")
        paramsDict["bunch"] = bunch
        paramsDict["useCharge"] = self.useCharge

        def track(p):
            p["node"].track(p)

        actionContainer.addAction(track, AccActionsContainer.BODY)
        self.trackActions(actionContainer, paramsDict, index_start, index_stop)
        actionContainer.removeAction(track, AccActionsContainer.BODY)

    def trackBunchTurns(self, bunch, turns, paramsDict=None):
        """Tracks ``turns`` passes through the whole lattice; with fused
        tracking the recorded program is replayed ``turns`` times from one
        CUDA graph per turn."""
        if paramsDict is None:
            paramsDict = {}
        if self._fused and is_device_bunch(bunch):
            bunch._device_bunch(wait=False)  # the upload overlaps the walk
            prog = self._program(bunch, paramsDict, -1, -1)
            if prog is not None:
                prog.run(bunch, int(turns))
                return
        for _ in range(int(turns)):
            self.trackBunch(bunch, dict(paramsDict))

    def fusedProgram(self, bunch, paramsDict=None):
        """The FusedProgram a trackBunch call would run (None if the lattice
        is not recordable)."""
        return self._program(bunch, paramsDict or {}, -1, -1)

    def setUseRealCharge(self, useCharge=1):
        self.useCharge = useCharge

    def getUseRealCharge(self):
        return self.useCharge


class TEAPOT_Ring(TEAPOT_Lattice):
    """Ring: bunch-wrap nodes at the exit of every first-level node with
    length, and a turn counter at the end (teapot.py:146-171)."""

    def __init__(self, name="no name"):
        TEAPOT_Lattice.__init__(self, name)

    def _addChildren(self):
        TEAPOT_Lattice.initialize(self)
        for node in self.getNodes():
            if node.getLength() > 0.0:
                w = BunchWrapTEAPOT(node.getName() + ":Bunch_Wrap:Exit")
                w.getParamsDict()["ring_length"] = self.getLength()
                node.addChildNode(w, AccNode.EXIT)
        self.getNodes().append(TurnCounterTEAPOT())


class BaseTEAPOT(AccNodeBunchTracker):
    """Base of the TEAPOT element hierarchy."""

    def __init__(self, name="no name"):
        AccNodeBunchTracker.__init__(self, name)
        self.setType("base teapot")


def _turn_counter(bunch):
    if bunch.hasBunchAttrInt("TurnNumber") != 0:
        bunch.bunchAttrInt("TurnNumber", bunch.bunchAttrInt("TurnNumber") + 1)


class TurnCounterTEAPOT(BaseTEAPOT):
    def __init__(self, name="TurnCounter"):
        BaseTEAPOT.__init__(self, name)
        self.setType("turn counter")

    def track(self, paramsDict):
        bunch = paramsDict["bunch"]
        rec = getattr(bunch, "_record_host", None)
        if rec is not None:
            rec(_turn_counter)
            return
        _turn_counter(bunch)


class NodeTEAPOT(BaseTEAPOT):
    """Element with tilt and fringe-field children at entrance and exit."""

    def __init__(self, name="no name"):
        BaseTEAPOT.__init__(self, name)
        self.__tiltIN = TiltTEAPOT()
        self.__tiltOUT = TiltTEAPOT()
        self.__fringeIN = FringeFieldTEAPOT(self)
        self.__fringeOUT = FringeFieldTEAPOT(self)
        self.__tiltIN.setName(name + "_tilt_in")
        self.__tiltOUT.setName(name + "_tilt_out")
        self.__fringeIN.setName(name + "_fringe_in")
        self.__fringeOUT.setName(name + "_fringe_out")
        self.addChildNode(self.__tiltIN, AccNode.ENTRANCE)
        self.addChildNode(self.__fringeIN, AccNode.ENTRANCE)
        self.addChildNode(self.__fringeOUT, AccNode.EXIT)
        self.addChildNode(self.__tiltOUT, AccNode.EXIT)
        self.addParam("tilt", self.__tiltIN.getTiltAngle())
        self.setType("node teapot")

    def setTiltAngle(self, angle=0.0):
        self.setParam("tilt", angle)
        self.__tiltIN.setTiltAngle(angle)
        self.__tiltOUT.setTiltAngle(-1.0 * angle)

    def getTiltAngle(self):
        return self.__tiltIN.getTiltAngle()

    def getNodeFringeFieldIN(self):
        return self.__fringeIN

    def getNodeFringeFieldOUT(self):
        return self.__fringeOUT

    def getNodeTiltIN(self):
        return self.__tiltIN

    def getNodeTiltOUT(self):
        return self.__tiltOUT

    def setFringeFieldFunctionIN(self, f=None):
        self.__fringeIN.setFringeFieldFunction(f)

    def setFringeFieldFunctionOUT(self, f=None):
        self.__fringeOUT.setFringeFieldFunction(f)

    def getFringeFieldFunctionIN(self):
        return self.__fringeIN.getFringeFieldFunction()

    def getFringeFieldFunctionOUT(self):
        return self.__fringeOUT.getFringeFieldFunction()

    def setUsageFringeFieldIN(self, usage=True):
        self.__fringeIN.setUsage(usage)

    def getUsageFringeFieldIN(self):
        return self.__fringeIN.getUsage()

    def setUsageFringeFieldOUT(self, usage=True):
        self.__fringeOUT.setUsage(usage)

    def getUsageFringeFieldOUT(self):
        return self.__fringeOUT.getUsage()


def _split_parts(node, what):
    """Part lengths L/(n-1)/2, L/(n-1), ..., L/(n-1)/2 (e.g. teapot.py:904-927)."""
    n = node.getnParts()
    if n < 2:
        orbitFinalize("The %s TEAPOT class instance should have more than 2 parts! name=%s nParts=%d"
                      % (what, node.getName(), n))
    lin = (node.getLength() / (n - 1)) / 2.0
    lout = (node.getLength() / (n - 1)) / 2.0
    step = lin + lout
    node.setLength(lin, 0)
    node.setLength(lout, n - 1)
    for i in range(n - 2):
        node.setLength(step, i + 1)


def _use_charge(paramsDict):
    return paramsDict.get("useCharge", 1)


class DriftTEAPOT(NodeTEAPOT):
    def __init__(self, name="drift no name"):
        NodeTEAPOT.__init__(self, name)
        self.setType("drift teapot")

    def track(self, paramsDict):
        TPB.drift(paramsDict["bunch"], self.getLength(self.getActivePartIndex()))


class ApertureTEAPOT(NodeTEAPOT):
    def __init__(self, name="aperture no name"):
        NodeTEAPOT.__init__(self, name)
        self.setType("aperture")
        self.addParam("aperture", [])
        self.addParam("apertype", 0.0)

    def track(self, paramsDict):
        raise NotImplementedError("apertures (particle loss) are outside the GPU hot path")


class MonitorTEAPOT(NodeTEAPOT):
    """Records the bunch centroid with BunchTwissAnalysis (host diagnostics)."""

    def __init__(self, name="Monitor no name"):
        NodeTEAPOT.__init__(self, name)
        self.setType("monitor teapot")
        self.twiss = BunchTwissAnalysis()

    def track(self, paramsDict):
        bunch = paramsDict["bunch"]
        self.twiss.analyzeBunch(bunch)
        self.addParam("xAvg", self.twiss.getAverage(0))
        self.addParam("xpAvg", self.twiss.getAverage(1))
        self.addParam("yAvg", self.twiss.getAverage(2))
        self.addParam("ypAvg", self.twiss.getAverage(3))


class BunchWrapTEAPOT(NodeTEAPOT):
    def __init__(self, name="drift no name"):
        NodeTEAPOT.__init__(self, name)
        self.setType("bunch_wrap_teapot")
        self.addParam("ring_length", 0.0)

    def track(self, paramsDict):
        TPB.wrapbunch(paramsDict["bunch"], self.getParam("ring_length"))


class SolenoidTEAPOT(NodeTEAPOT):
    def __init__(self, name="solenoid no name"):
        NodeTEAPOT.__init__(self, name)
        self.setType("solenoid teapot")
        self.addParam("B", 0.0)
        self.waveform = None

    def track(self, paramsDict):
        raise NotImplementedError("solenoids are outside the GPU hot path")

    def setWaveform(self, waveform):
        self.waveform = waveform


class MultipoleTEAPOT(NodeTEAPOT):
    """Multipole: drift / multp sandwich (teapot.py:685-823)."""

    def __init__(self, name="multipole no name"):
        NodeTEAPOT.__init__(self, name)
        self.addParam("poles", [])
        self.addParam("kls", [])
        self.addParam("skews", [])
        self.setnParts(2)
        self.waveform = None
        outer = self

        def fringe(node, paramsDict, inout):
            if not node.getUsage():
                return
            length = paramsDict["parentNode"].getLength()
            if length == 0.0:
                return
            strength = outer.waveform.getStrength() if outer.waveform else 1.0
            bunch = paramsDict["bunch"]
            uc = _use_charge(paramsDict)
            f = TPB.multpfringeIN if inout == 0 else TPB.multpfringeOUT
            for pole, kl, skew in zip(node.getParam("poles"), node.getParam("kls"), node.getParam("skews")):
                f(bunch, pole, strength * kl / length, skew, uc)

        self.setFringeFieldFunctionIN(lambda node, pd: fringe(node, pd, 0))
        self.setFringeFieldFunctionOUT(lambda node, pd: fringe(node, pd, 1))
        self.setType("multipole teapot")

    def initialize(self):
        _split_parts(self, "Multipole")

    def track(self, paramsDict):
        n = self.getnParts()
        index = self.getActivePartIndex()
        length = self.getLength(index)
        strength = self.waveform.getStrength() if self.waveform else 1.0
        bunch = paramsDict["bunch"]
        uc = _use_charge(paramsDict)
        if index == 0:
            TPB.drift(bunch, length)
            return
        for pole, kl, skew in zip(self.getParam("poles"), self.getParam("kls"), self.getParam("skews")):
            TPB.multp(bunch, pole, strength * kl / (n - 1), skew, uc)
        TPB.drift(bunch, length)

    def setWaveform(self, waveform):
        self.waveform = waveform


class QuadTEAPOT(NodeTEAPOT):
    """Quadrupole: quad1 / quad2 / multp sandwich with hard-edge fringes
    (teapot.py:825-976)."""

    def __init__(self, name="quad no name"):
        NodeTEAPOT.__init__(self, name)
        self.addParam("kq", 0.0)
        self.addParam("poles", [])
        self.addParam("kls", [])
        self.addParam("skews", [])
        self.setnParts(2)
        self.waveform = None
        outer = self

        def fringe(node, paramsDict, inout):
            if not node.getUsage():
                return
            strength = outer.waveform.getStrength() if outer.waveform else 1.0
            kq = strength * node.getParam("kq")
            length = paramsDict["parentNode"].getLength()
            bunch = paramsDict["bunch"]
            uc = _use_charge(paramsDict)
            (TPB.quadfringeIN if inout == 0 else TPB.quadfringeOUT)(bunch, kq, uc)
            if length == 0.0:
                return
            f = TPB.multpfringeIN if inout == 0 else TPB.multpfringeOUT
            for pole, kl, skew in zip(node.getParam("poles"), node.getParam("kls"), node.getParam("skews")):
                f(bunch, pole, strength * kl / length, skew, uc)

        self.setFringeFieldFunctionIN(lambda node, pd: fringe(node, pd, 0))
        self.setFringeFieldFunctionOUT(lambda node, pd: fringe(node, pd, 1))
        self.getNodeTiltIN().setType("quad tilt in")
        self.getNodeTiltOUT().setType("quad tilt out")
        self.getNodeFringeFieldIN().setType("quad fringe in")
        self.getNodeFringeFieldOUT().setType("quad fringe out")
        self.setType("quad teapot")

    def initialize(self):
        _split_parts(self, "Quad Combined Function")

    def track(self, paramsDict):
        n = self.getnParts()
        index = self.getActivePartIndex()
        length = self.getLength(index)
        strength = self.waveform.getStrength() if self.waveform else 1.0
        kq = strength * self.getParam("kq")
        bunch = paramsDict["bunch"]
        uc = _use_charge(paramsDict)
        mps = list(zip(self.getParam("poles"), self.getParam("kls"), self.getParam("skews")))
        if index == 0:
            TPB.quad1(bunch, length, kq, uc)
            return
        # middle parts use length/2 in quad2; the last part uses the full
        # part length (teapot.py:958-970)
        l2 = length / 2.0 if index < n - 1 else length
        TPB.quad2(bunch, l2)
        for pole, kl, skew in mps:
            TPB.multp(bunch, pole, strength * kl / (n - 1), skew, uc)
        TPB.quad2(bunch, l2)
        TPB.quad1(bunch, length, kq, uc)

    def setWaveform(self, waveform):
        self.waveform = waveform


class BendTEAPOT(NodeTEAPOT):
    """Sector bend: bend1..bend4 / multp sandwich (teapot.py:978-1151)."""

    def __init__(self, name="bend no name"):
        NodeTEAPOT.__init__(self, name)
        self.addParam("poles", [])
        self.addParam("kls", [])
        self.addParam("skews", [])
        self.addParam("ea1", 0.0)
        self.addParam("ea2", 0.0)
        self.addParam("rho", 0.0)
        self.addParam("theta", 1.0e-36)
        self.setnParts(2)

        def fringe(node, paramsDict, inout):
            usage = node.getUsage()
            e = node.getParam("ea1" if inout == 0 else "ea2")
            rho = node.getParam("rho")
            mps = list(zip(node.getParam("poles"), node.getParam("kls"), node.getParam("skews")))
            length = paramsDict["parentNode"].getLength()
            bunch = paramsDict["bunch"]
            uc = _use_charge(paramsDict)
            if e != 0.0:
                # wedges need the combined-function wedge map (wedgebendCF),
                # which is outside the GPU hot path
                TPB.wedgebendCF(bunch, e, inout, rho, len(mps), [], [], [], 0, uc)
                return
            if not usage:
                return
            (TPB.bendfringeIN if inout == 0 else TPB.bendfringeOUT)(bunch, rho)
            if length != 0.0:
                f = TPB.multpfringeIN if inout == 0 else TPB.multpfringeOUT
                for pole, kl, skew in mps:
                    f(bunch, pole, kl / length, skew, uc)

        self.setFringeFieldFunctionIN(lambda node, pd: fringe(node, pd, 0))
        self.setFringeFieldFunctionOUT(lambda node, pd: fringe(node, pd, 1))
        self.setType("bend teapot")

    def initialize(self):
        n = self.getnParts()
        if n < 2:
            orbitFinalize("The Bend Combined Functions TEAPOT class instance should have more than 2 parts!")
        self.addParam("rho", self.getLength() / self.getParam("theta"))
        _split_parts(self, "Bend Combined Functions")

    def track(self, paramsDict):
        n = self.getnParts()
        index = self.getActivePartIndex()
        length = self.getLength(index)
        bunch = paramsDict["bunch"]
        uc = _use_charge(paramsDict)
        theta = self.getParam("theta") / (n - 1)
        if index == 0:
            TPB.bend1(bunch, length, theta / 2.0)
            return
        last = index == n - 1
        l2 = length if last else length / 2.0
        TPB.bend2(bunch, l2)
        TPB.bend3(bunch, theta / 2.0)
        TPB.bend4(bunch, theta / 2.0)
        for pole, kl, skew in zip(self.getParam("poles"), self.getParam("kls"), self.getParam("skews")):
            TPB.multp(bunch, pole, kl / (n - 1), skew, uc)
        TPB.bend4(bunch, theta / 2.0)
        TPB.bend3(bunch, theta / 2.0)
        TPB.bend2(bunch, l2)
        TPB.bend1(bunch, length, theta / 2.0 if last else theta)


class RingRFTEAPOT(NodeTEAPOT):
    def __init__(self, name="RingRF no name"):
        NodeTEAPOT.__init__(self, name)
        self.addParam("harmonics", [])
        self.addParam("voltages", [])
        self.addParam("phases", [])
        self.addParam("ring_length", 0.0)
        self.setType("RingRF teapot")
        self.setnParts(1)

    def addRF(self, harmonic, voltage, phase):
        self.getParam("harmonics").append(harmonic)
        self.getParam("voltages").append(voltage)
        self.getParam("phases").append(phase)

    def track(self, paramsDict):
        if self.getParam("harmonics"):
            TPB.RingRF(paramsDict["bunch"])


class KickTEAPOT(NodeTEAPOT):
    """Kicker: drift / kick sandwich (teapot.py:1184-1256)."""

    def __init__(self, name="kick no name"):
        NodeTEAPOT.__init__(self, name)
        self.addParam("kx", 0.0)
        self.addParam("ky", 0.0)
        self.addParam("dE", 0.0)
        self.setType("kick teapot")
        self.setnParts(2)
        self.waveform = None

    def initialize(self):
        _split_parts(self, "Kick")

    def track(self, paramsDict):
        n = self.getnParts()
        index = self.getActivePartIndex()
        length = self.getLength(index)
        strength = self.waveform.getStrength() if self.waveform else 1.0
        kx = strength * self.getParam("kx") / (n - 1)
        ky = strength * self.getParam("ky") / (n - 1)
        dE = self.getParam("dE") / (n - 1)
        bunch = paramsDict["bunch"]
        uc = _use_charge(paramsDict)
        TPB.drift(bunch, length)
        if index < n - 1:
            TPB.kick(bunch, kx, ky, dE, uc)

    def setWaveform(self, waveform):
        self.waveform = waveform


class TiltTEAPOT(BaseTEAPOT):
    """Rotation by the tilt angle at an element's entrance or exit."""

    def __init__(self, name="tilt no name", angle=0.0):
        AccNode.__init__(self, name)
        self.__angle = angle
        self.setType("tilt teapot")

    def setTiltAngle(self, angle=0.0):
        self.__angle = angle

    def getTiltAngle(self):
        return self.__angle

    def track(self, paramsDict):
        if self.__angle != 0.0:
            TPB.rotatexy(paramsDict["bunch"], self.__angle)


class FringeFieldTEAPOT(BaseTEAPOT):
    """Fringe-field child node sharing its parent's parameters."""

    def __init__(self, parentNode, trackFunction=None, name="fringe field no name"):
        AccNode.__init__(self, name)
        self.setParamsDict(parentNode.getParamsDict())
        self.__trackFunc = trackFunction
        self.__usage = True
        self.setType("fringeField teapot")

    def track(self, paramsDict):
        if self.__trackFunc is not None:
            self.__trackFunc(self, paramsDict)

    def setFringeFieldFunction(self, trackFunction=None):
        self.__trackFunc = trackFunction

    def getFringeFieldFunction(self):
        return self.__trackFunc

    def setUsage(self, usage=True):
        self.__usage = usage

    def getUsage(self):
        return self.__usage
