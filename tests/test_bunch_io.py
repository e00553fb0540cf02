"""Bunch text I/O (Bunch.dumpBunch / readBunch) against files the reference
wrote (tests/golden/bunch_dump_ref.txt: the reference's Bunch::print of a
40-particle bunch with three particle attribute controllers, two bunch
attributes and a sync-particle time; bunch_dump_ref_reread.txt: the
reference reading that file into a new bunch and printing it again).

Host only: the bunch's text I/O touches no device.  Exact: the texts must
match byte for byte."""
import os

import numpy as np
import pytest

import oracle as O
from helpers import GOLDEN

REF_FILE = os.path.join(GOLDEN, "bunch_dump_ref.txt")
REREAD_FILE = os.path.join(GOLDEN, "bunch_dump_ref_reread.txt")


def golden_bunch_coords():
    """The coordinates tests/golden/make_golden.py gave the reference bunch
    (its gaussian(40, 151))."""
    rng = np.random.Generator(np.random.PCG64(151))
    n = 40
    soa = np.empty((6, n))
    for c, s in enumerate((5e-3, 1e-3, 4e-3, 1e-3, 10.0, 1e-3)):
        soa[c] = rng.normal(0, s, n)
    return soa


def build_like_reference():
    from bunch import Bunch
    soa = golden_bunch_coords()
    b = Bunch()
    b.getSyncParticle().kinEnergy(1.3)
    b.macroSize(2.5e9)
    for i in range(soa.shape[1]):
        b.addParticle(*soa[:, i])
    b.addPartAttr("macrosize")
    b.addPartAttr("ParticleIdNumber")
    b.addPartAttr("Amplitudes", {"size": 3})
    for i in range(soa.shape[1]):
        b.partAttrValue("macrosize", i, 0, 1e9 * (1.0 + 0.01 * i))
        b.partAttrValue("ParticleIdNumber", i, 0, 1000 + i)
        for j in range(3):
            b.partAttrValue("Amplitudes", i, j, 0.1 * j - 0.003 * i)
    b.bunchAttrInt("TurnNumber", 7)
    b.bunchAttrDouble("beam_current", 0.0123456789)
    b.getSyncParticle().time(1.234567890123e-6)
    return b


def test_dump_writes_the_reference_file(tmp_path):
    """The same bunch built through this API prints the reference's text."""
    out = tmp_path / "b.txt"
    build_like_reference().dumpBunch(str(out))
    assert out.read_text() == open(REF_FILE).read()


def test_read_then_dump_matches_the_reference_doing_the_same(tmp_path):
    from bunch import Bunch
    b = Bunch()
    assert b.readBunch(REF_FILE) == 40
    out = tmp_path / "b.txt"
    b.dumpBunch(str(out))
    assert out.read_text() == open(REREAD_FILE).read()


def test_read_reference_file_values():
    from bunch import Bunch
    b = Bunch()
    b.readBunch(REF_FILE)
    soa = golden_bunch_coords()
    got = b.getCoordinates()
    # the file holds 8 significant digits
    assert np.allclose(got, soa, rtol=1e-7, atol=0)
    assert b.hasPartAttr("Amplitudes") and b._part_attr["Amplitudes"].shape[1] == 3
    assert b.partAttrValue("ParticleIdNumber", 39, 0) == 1039
    assert abs(b.partAttrValue("macrosize", 5, 0) - 1.05e9) < 1e-6 * 1.05e9
    assert abs(b.partAttrValue("Amplitudes", 10, 2) - (0.2 - 0.03)) < 1e-9
    assert b.bunchAttrInt("TurnNumber") == 7
    assert abs(b.bunchAttrDouble("beam_current") - 0.0123457) < 1e-12
    assert b.getSyncParticle().time() == 1.234567890123e-6
    assert abs(b.getSyncParticle().momentum() - 2.0321189024759) < 1e-13


def test_read_appends_and_limits_particles():
    """readBunch appends to the particles already there and reads at most
    nParts (Bunch.cc:1116-1264)."""
    from bunch import Bunch
    b = Bunch()
    b.addParticle(1e-3, 0, 0, 0, 0, 0)
    assert b.readBunch(REF_FILE, 10) == 11
    assert b.x(0) == 1e-3
    assert abs(b.x(1) - golden_bunch_coords()[0, 0]) < 1e-10


def test_dead_particles_are_not_written(tmp_path):
    b = build_like_reference()
    b.deleteParticleFast(3)
    b.deleteParticleFast(17)
    out = tmp_path / "b.txt"
    b.dumpBunch(str(out))
    rows = [ln for ln in out.read_text().splitlines() if not ln.startswith("%")]
    assert len(rows) == 38
    assert not any(ln.split()[7] in ("1003", "1017") for ln in rows)


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present on this host")
def test_reference_reads_a_file_this_library_wrote(tmp_path):
    out = tmp_path / "b.txt"
    b = build_like_reference()
    b.dumpBunch(str(out))
    r = O.RefBunch(np.zeros((6, 0)), 1.0, 1.0)
    r.read(str(out))
    assert r.n == 40
    assert np.allclose(r.coords(), golden_bunch_coords(), rtol=1e-7, atol=0)
    assert r.attr_size("Amplitudes") == 3
    assert r.attr("ParticleIdNumber", 12, 0) == 1012
    assert r.bunch_attr_int("TurnNumber") == 7
