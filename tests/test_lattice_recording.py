"""Host logic of the lattice layer (no GPU): node order, part lengths, SC
node placement, and the recorded device programs, checked against the
reference's rules and -- where the compiled reference is present -- against
the reference executing the same op sequence."""
import numpy as np
import pytest

import oracle as O
from helpers import coord_err


class RecCalc:
    """Stands in for SpaceChargeCalc2p5D: records kicks, allocates nothing."""

    def trackBunch(self, bunch, length, boundary=None):
        bunch._record_sc(self, length)


def record(lat, bunch):
    from orbit.lattice import AccActionsContainer
    from orbit.teapot.recording import BunchRecorder
    rec = BunchRecorder(bunch)
    cont = AccActionsContainer()
    cont.addAction(lambda p: p["node"].track(p), AccActionsContainer.BODY)
    lat.trackActions(cont, {"bunch": rec, "useCharge": 1})
    return rec


def names(ops):
    from orbit_gb300 import OP
    inv = {v: k for k, v in OP.items()}
    return [inv[o[0]] for o in ops]


def test_fodo_order_and_sc_lengths(capsys):
    from orbit_gb300 import workloads as W
    lat = W.fodo_lattice(RecCalc(), cells=3)
    b = W.make_bunch(W.c2_coords(100), 1e9)
    rec = record(lat, b)
    cell = ["QFRIN", "SC", "QUAD1", "QUAD2", "QUAD2", "QUAD1", "QFROUT", "SC", "DRIFT"]
    assert names(rec.ops) == cell * 6
    sc_lengths = [o[2][0] for o in rec.ops if o[0] == 32]
    assert sc_lengths == [0.5, 2.0] * 6
    assert abs(sum(sc_lengths) - lat.getLength()) < 1e-12
    # quad part lengths: L/(n-1)/2 at both ends (teapot.py:904-927)
    q = lat.getNodes()[0]
    assert q.getnParts() == 2 and q.getLength(0) == 0.25 and q.getLength(1) == 0.25


def test_quad_parts_schedule():
    """nParts = 4: quad1(L0), then middle parts quad2(L/2) quad2(L/2) quad1(L),
    last part quad2(L) quad2(L) quad1(L) (teapot.py:945-970)."""
    from orbit.teapot import QuadTEAPOT, TEAPOT_Lattice
    q = QuadTEAPOT("q")
    q.setnParts(4)
    q.setLength(1.2)
    q.addParam("kq", 0.3)
    lat = TEAPOT_Lattice()
    lat.addNode(q)
    lat.initialize()
    from orbit_gb300 import workloads as W
    rec = record(lat, W.make_bunch(W.c2_coords(10), 1e9))
    ops = [(n, o[2]) for n, o in zip(names(rec.ops), rec.ops)]
    step = 1.2 / 3
    assert ops[0] == ("QFRIN", (0.3,))
    assert ops[1] == ("QUAD1", (step / 2, 0.3))
    assert ops[2] == ("QUAD2", (step / 2,)) and ops[3] == ("QUAD2", (step / 2,)) and ops[4] == ("QUAD1", (step, 0.3))
    assert ops[8] == ("QUAD2", (step / 2,)) and ops[9] == ("QUAD2", (step / 2,))
    assert ops[-1] == ("QFROUT", (0.3,))


def test_bend_schedule_and_fringes():
    from orbit.teapot import BendTEAPOT, TEAPOT_Lattice
    from orbit_gb300 import workloads as W
    bd = BendTEAPOT("b")
    bd.setLength(2.0)
    bd.addParam("theta", 0.2)
    bd.setnParts(3)
    lat = TEAPOT_Lattice()
    lat.addNode(bd)
    lat.initialize()
    rec = record(lat, W.make_bunch(W.c2_coords(10), 1e9))
    nm = names(rec.ops)
    assert nm[0] == "BFRIN" and nm[-1] == "BFROUT"
    assert nm[1] == "BEND1"
    assert nm[2:10] == ["BEND2", "BEND3", "BEND4", "BEND4", "BEND3", "BEND2", "BEND1", "BEND2"]
    assert abs(rec.ops[0][2][0] - 10.0) < 1e-12  # rho = L/theta


def test_monitor_makes_walk_unrecordable():
    from orbit.teapot import DriftTEAPOT, MonitorTEAPOT, TEAPOT_Lattice
    from orbit.teapot.recording import NotRecordable
    from orbit_gb300 import workloads as W
    lat = TEAPOT_Lattice()
    d = DriftTEAPOT("d")
    d.setLength(1.0)
    lat.addNode(d)
    lat.addNode(MonitorTEAPOT("m"))
    lat.initialize()
    with pytest.raises(NotRecordable):
        record(lat, W.make_bunch(W.c2_coords(10), 1e9))


def test_ring_adds_wraps_and_turn_counter():
    from orbit.teapot import DriftTEAPOT, TEAPOT_Ring
    from orbit_gb300 import workloads as W
    ring = TEAPOT_Ring("r")
    for i in range(3):
        d = DriftTEAPOT("d%d" % i)
        d.setLength(2.0)
        ring.addNode(d)
    ring._addChildren()
    ring.initialize()
    b = W.make_bunch(W.c2_coords(10), 1e9)
    b.bunchAttrInt("TurnNumber", 0)
    rec = record(ring, b)
    assert names(rec.ops) == ["DRIFT", "WRAP"] * 3
    assert rec.ops[1][2][0] == 6.0
    assert len(rec.host_ops) == 1
    rec.host_ops[0](b)
    assert b.bunchAttrInt("TurnNumber") == 1


def test_sc_placement_matches_reference_rule():
    """setSC_General_AccNodes: a node at a part start once the running path
    exceeds the minimum; the first node takes the rest of the lattice."""
    from orbit.space_charge.sc2p5d import setSC2p5DAccNodes
    from orbit.teapot import DriftTEAPOT, TEAPOT_Lattice
    lat = TEAPOT_Lattice()
    lens = [0.3, 0.3, 0.3, 0.7, 0.2]
    for i, L in enumerate(lens):
        d = DriftTEAPOT("d%d" % i)
        d.setLength(L)
        lat.addNode(d)
    lat.initialize()
    nodes = setSC2p5DAccNodes(lat, 0.5, RecCalc())
    # running path: 0 | 0.3 | 0.6>0.5 -> node at d2 (0.6) | 0.3 | 1.0 -> node at d4
    got = [(n.getName(), round(n.getLengthOfSC(), 12)) for n in nodes]
    assert got == [("d0:0:SC2p5D", 0.6), ("d2:0:SC2p5D", 1.0), ("d4:0:SC2p5D", 0.2)]


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present on this host")
def test_recorded_fodo_program_reference_vs_oracle():
    """The oracle's program executor reproduces the reference running the
    same recorded op sequence call by call."""
    from orbit_gb300 import workloads as W
    lat = W.fodo_lattice(RecCalc(), cells=2)
    soa = W.c2_coords(3000, seed=4)
    b = W.make_bunch(soa, 1e10)
    ops = record(lat, b).ops
    rb = O.RefBunch(soa, 1.0, 1e10)
    rs = O.RefSC(32, 32, 8)
    for turn in range(2):
        for code, iv, dv in ops:
            if code == 32:
                rs.track(rb, dv[0])
            else:
                from orbit_gb300 import OP
                inv = {v: k for k, v in OP.items()}
                nm = {"DRIFT": "drift", "QUAD1": "quad1", "QUAD2": "quad2", "QFRIN": "quadfringeIN",
                      "QFROUT": "quadfringeOUT"}[inv[code]]
                rb.tpb(nm, *dv)
    k = rb.kinematics()
    sync = O.make_sync(beta=k["beta"], gamma=k["gamma"], momentum=k["momentum"], macrosize=1e10)
    a = np.ascontiguousarray(soa.copy())
    assert O.run_program(ops, 2, a, sync, [O.OracleSC(32, 32, 8)]) == 0
    assert coord_err(a, rb.coords()) == 0.0
    assert sync.time == k["time"]
