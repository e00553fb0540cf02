"""Recording a lattice walk into a device program.

``TEAPOT_Lattice.trackBunch`` walks the node tree exactly as the reference
does (AccNode.trackActions), but with a ``BunchRecorder`` in place of the
bunch: every TEAPOT map call and space-charge kick is appended to an op list
instead of being executed.  The op list is compiled once into fused device
passes (liborbit_gb300 ``orbit_program_*``) and replayed from a CUDA graph.
Nodes that need the coordinates on the host (monitors, user code) make the
walk unrecordable, and the lattice then runs node by node instead.
"""
from __future__ import annotations

from orbit_gb300 import OP, DeviceProgram


class NotRecordable(Exception):
    """A node touched the bunch in a way a device program cannot replay."""


class BunchRecorder:
    """Stands in for a ``Bunch`` while a lattice walk is recorded."""

    _READS = {"getSize", "getSizeGlobal", "getSizeGlobalFromMemory", "getTotalCount", "macroSize", "mass",
              "charge", "classicalRadius", "hasBunchAttrInt", "hasBunchAttrDouble", "hasPartAttr",
              "getPartAttrNames", "bunchAttrIntNames", "bunchAttrDoubleNames", "B_Rho"}

    def __init__(self, bunch):
        self._bunch = bunch
        self.ops = []
        self.calcs = []
        self._cidx = {}
        self.boundaries = []
        self._bidx = {}
        self.host_ops = []

    # --- called by teapot_base and SpaceChargeCalc2p5D
    def _record_op(self, code, ints, dbls):
        self.ops.append((int(code), tuple(ints), tuple(dbls)))

    def _record_sc(self, calc, length, pipe_radius=0.0, boundary=None):
        k = self._cidx.get(id(calc))
        if k is None:
            k = len(self.calcs)
            self._cidx[id(calc)] = k
            self.calcs.append(calc)
        b = 0
        if boundary is not None:
            b = self._bidx.get(id(boundary))
            if b is None:
                self.boundaries.append(boundary)
                b = len(self.boundaries)
                self._bidx[id(boundary)] = b
        self.ops.append((OP["SC"], (k, b), (float(length), float(pipe_radius))))

    def _record_host(self, fn):
        """fn(bunch) runs on the host once per replayed turn (turn counters)."""
        self.host_ops.append(fn)

    # --- bunch reads that do not depend on coordinates
    def bunchAttrInt(self, name, value=None):
        if value is not None:
            raise NotRecordable("bunchAttrInt set")
        return self._bunch.bunchAttrInt(name)

    def bunchAttrDouble(self, name, value=None):
        if value is not None:
            raise NotRecordable("bunchAttrDouble set")
        return self._bunch.bunchAttrDouble(name)

    def __getattr__(self, name):
        if name in BunchRecorder._READS:
            real = getattr(self._bunch, name)

            def read_only(*args):
                if args and name in ("macroSize", "mass", "charge"):
                    raise NotRecordable(name + " set")
                return real(*args)
            return read_only
        raise NotRecordable(name)


class FusedProgram:
    """A recorded op list compiled for the GPU."""

    def __init__(self, ops, calcs, host_ops, boundaries=()):
        self.ops = list(ops)
        self.calcs = list(calcs)
        self.host_ops = list(host_ops)
        self.boundaries = list(boundaries)
        self.device = DeviceProgram(self.ops, [c._calc for c in self.calcs], [b._dev for b in self.boundaries])

    def run(self, bunch, turns=1):
        dev = bunch._device_bunch()
        try:
            self.device.run(dev, turns)
        finally:
            bunch._device_modified()
            for c in self.calcs:
                c._version += 1
        for _ in range(turns):
            for fn in self.host_ops:
                fn(bunch)

    def launches_per_turn(self):
        return self.device.launches_per_turn()


def is_device_bunch(bunch) -> bool:
    return hasattr(bunch, "_device_bunch")
