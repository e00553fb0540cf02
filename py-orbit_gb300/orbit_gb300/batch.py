"""Batched tracking of many bunches: the points of an intensity or
quadrupole-strength scan, each a Bunch with its own TEAPOT lattice and
SpaceChargeCalc2p5D, advanced together on one GPU.

In the reference a scan is a Python loop that tracks one bunch after the
other (AccLattice.trackBunch, py/orbit/lattice/AccLattice.py:243-255).
Here every stage of a kick interval runs as one kernel launch for all bunches
of a grid size, and a turn of the whole scan replays from one CUDA graph.
Each bunch ends where tracking it alone would leave it (up to the rounding
of the FFT schedule the autotuner picks)."""
from __future__ import annotations

from . import DeviceBatch


class BunchBatch:
    """``BunchBatch([(bunch, lattice), ...])``; ``trackTurns(n)`` tracks
    every bunch through its own lattice ``n`` times.  The lattices must
    share one node structure (the same node types and SC nodes in the same
    places; strengths, intensities and grid sizes may differ), each with one
    plain-form SpaceChargeCalc2p5D of its own."""

    def __init__(self, members):
        self.members = list(members)
        if not self.members:
            raise ValueError("no bunches")
        self._batch = None
        self._key = None

    def _prepare(self):
        progs = []
        for bunch, lat in self.members:
            prog = lat.fusedProgram(bunch)
            if prog is None:
                raise ValueError("lattice %r cannot be recorded into a device program" % lat.getName())
            progs.append(prog)
        devs = [b._device_bunch() for b, _ in self.members]
        key = tuple(id(p.device) for p in progs) + tuple(id(d) for d in devs)
        if key != self._key:
            self._batch = DeviceBatch([p.device for p in progs], devs)
            self._key = key
        return progs

    def trackTurns(self, turns: int):
        progs = self._prepare()
        try:
            self._batch.run(int(turns))
        finally:
            for (bunch, _), prog in zip(self.members, progs):
                bunch._device_modified()
                for c in prog.calcs:
                    c._version += 1
        for _ in range(int(turns)):
            for (bunch, _), prog in zip(self.members, progs):
                for fn in prog.host_ops:
                    fn(bunch)

    def enqueueTurns(self, turns: int):
        """As trackTurns without waiting (``sync()`` waits and reports
        device errors); host-side per-turn bookkeeping is not run."""
        progs = self._prepare()
        self._batch.enqueue(int(turns))
        for (bunch, _), prog in zip(self.members, progs):
            bunch._device_modified()
            for c in prog.calcs:
                c._version += 1

    def sync(self):
        self._batch.sync()

    def classes(self):
        """Grid classes with the launch shapes the autotuner picked."""
        self._prepare()
        return self._batch.classes()

    def profile(self):
        """One eager turn with every launch timed: {kernel kind: (ms, launches)}."""
        progs = self._prepare()
        try:
            return self._batch.profile()
        finally:
            for (bunch, _), prog in zip(self.members, progs):
                bunch._device_modified()
                for c in prog.calcs:
                    c._version += 1

    def launchesPerTurn(self) -> int:
        return self._batch.info()[1] if self._batch is not None else 0
