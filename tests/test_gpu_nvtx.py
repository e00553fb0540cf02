"""NVTX ranges: with the per-node ranges of the lattice walk switched on
(ORBIT_NVTX=1, here set on the module), node-by-node tracking gives the
same coordinates bit for bit as without them (the ranges only mark the
timeline)."""
import contextlib
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_nvtx_ranges_leave_tracking_unchanged(monkeypatch):
    import sys

    import orbit.lattice.AccNode  # noqa: F401  (the package re-exports the class under the same name)
    accnode = sys.modules["orbit.lattice.AccNode"]
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = W.c2_coords(5000, seed=71)

    def run(nvtx):
        monkeypatch.setattr(accnode, "_NVTX", nvtx)
        b = W.make_bunch(soa, 1e9)
        with contextlib.redirect_stdout(io.StringIO()):
            lat = W.fodo_lattice(SpaceChargeCalc2p5D(32, 32, 8), cells=2)
        lat.setFusedTracking(False)
        lat.trackBunch(b)
        return b.getCoordinates()

    assert np.array_equal(run(True), run(False))
