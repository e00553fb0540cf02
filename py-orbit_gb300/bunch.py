"""Module ``bunch``: the PyORBIT ``Bunch`` / ``SyncPart`` /
``BunchTwissAnalysis`` / ``BunchTuneAnalysis`` interface (src/orbit/wrap_bunch.cc,
src/orbit/wrap_syncpart.cc, src/orbit/BunchDiagnostics/) over a
device-resident bunch.

The coordinates live in HBM as six FP64 arrays once any GPU map or
space-charge kick has touched the bunch; per-particle accessors such as
``x(i)`` download them on demand, and host-side edits are uploaded before
the next device operation.  Host-only use (building a bunch, reading it
back) needs no GPU.
"""
from __future__ import annotations

import math
import os

import numpy as np

_COORDS = ("x", "xp", "y", "yp", "z", "dE")

# OrbitConst.cc:34-36
MASS_PROTON = 0.938272013
CLASSICAL_RADIUS_PROTON = 1.534698e-18
CHARGE_PROTON = 1.0

# ParticlePhaseAttributes.cc: six values per particle {xLastPhase,
# yLastPhase, xLastTune, yLastTune, xAction, yAction}
PHASE_ATTR = "ParticlePhaseAttributes"


class SyncPart:
    """Synchronous (reference) particle: momentum vector, kinetic energy,
    beta, gamma and time (src/orbit/SyncPart.cc)."""

    def __init__(self, bunch: "Bunch"):
        self._bunch = bunch
        self._time = 0.0
        self._xyz = [0.0, 0.0, 0.0]
        self._pxyz = [0.0, 0.0, 0.0]
        self._nx = [1.0, 0.0, 0.0]  # x-axis ort (SyncPart.cc: normal vector, printed and read only)
        self._p_abs = 0.0
        self._energy = 0.0
        self._beta = 0.0
        self._gamma = 1.0

    # SyncPart::updateKinematics (SyncPart.cc:236-306), kinematics part
    def _update(self):
        p2 = self._pxyz[0] * self._pxyz[0] + self._pxyz[1] * self._pxyz[1] + self._pxyz[2] * self._pxyz[2]
        self._p_abs = math.sqrt(p2)
        m = self._bunch.mass()
        m2 = m * m
        w = math.sqrt(m2 + p2)
        self._energy = p2 / (math.sqrt(m2 + p2) + m)
        self._beta = self._p_abs / w
        self._gamma = w / m
        self._bunch._sync_changed()

    def energyToMomentum(self, ek: float) -> float:  # SyncPart.cc:314-317
        m = self._bunch.mass()
        return math.sqrt(ek * (ek + 2.0 * m))

    def momentumToEnergy(self, p: float) -> float:  # SyncPart.cc:308-312
        m = self._bunch.mass()
        return p * p / (math.sqrt(m * m + p * p) + m)

    def kinEnergy(self, value=None) -> float:
        """kinEnergy() -> GeV; kinEnergy(ek) sets pz (wrap_syncpart.cc:70-93)."""
        if value is None:
            return self._energy
        p = self.energyToMomentum(float(value))
        self._pxyz = [0.0, 0.0, p]
        self._update()
        return self.momentumToEnergy(p)

    def momentum(self, value=None) -> float:
        if value is None:
            return self._p_abs
        self._pxyz = [0.0, 0.0, float(value)]
        self._update()
        return self._p_abs

    def beta(self) -> float:
        return self._beta

    def gamma(self) -> float:
        return self._gamma

    def mass(self) -> float:
        return self._bunch.mass()

    def time(self, value=None) -> float:
        if value is not None:
            self._bunch._sync_changed()
            self._time = float(value)
        else:
            self._bunch._pull_time()
        return self._time

    def _coord(self, arr, i, value):
        if value is not None:
            arr[i] = float(value)
            if arr is self._pxyz:
                self._update()
        return arr[i]

    def x(self, v=None): return self._coord(self._xyz, 0, v)
    def y(self, v=None): return self._coord(self._xyz, 1, v)
    def z(self, v=None): return self._coord(self._xyz, 2, v)
    def px(self, v=None): return self._coord(self._pxyz, 0, v)
    def py(self, v=None): return self._coord(self._pxyz, 1, v)
    def pz(self, v=None): return self._coord(self._pxyz, 2, v)

    def pVector(self, v=None):
        if v is not None:
            self._pxyz = [float(a) for a in v]
            self._update()
        return tuple(self._pxyz)

    def rVector(self, v=None):
        if v is not None:
            self._xyz = [float(a) for a in v]
        return tuple(self._xyz)


class Bunch:
    """Macroparticle bunch with the reference's Python interface."""

    def __init__(self):
        self._n = 0
        self._host = np.zeros((6, 16), dtype=np.float64)
        self._flag = np.ones(16, dtype=np.int8)
        self._host_ok = True     # host copy holds the current coordinates
        self._dev_ok = False     # device copy holds the current coordinates
        self._dev = None         # orbit_gb300.DeviceBunch, created on first device use
        self._upload_pending = False  # an enqueued upload may still read the host rows
        self._mass = MASS_PROTON
        self._charge = CHARGE_PROTON
        self._classical_radius = CLASSICAL_RADIUS_PROTON
        self._macrosize = 0.0
        self._attr_double = {"mass": self._mass, "charge": self._charge,
                             "classical_radius": self._classical_radius, "macro_size": 0.0}
        self._attr_int = {}
        self._part_attr = {}     # name -> (n, k) array
        self._part_attr_dict = {}
        self._sync = SyncPart(self)
        self._sync_dirty = True
        self._phase_dev = False  # device phase rows newer than the host attribute

    # ------------------------------------------------------------ storage
    def _pull_attrs(self):
        """Brings the ParticlePhaseAttributes rows that a device tune
        analysis wrote back into the host attribute."""
        if self._phase_dev:
            self._phase_dev = False
            arr = self._part_attr.get(PHASE_ATTR)
            if arr is not None and self._n > 0:
                arr[: self._n, :6] = self._dev.phase_get().T

    def _ensure_host(self):
        if self._upload_pending:
            # an upload may still read the host rows: let it finish first
            self._dev.sync()
            self._upload_pending = False
        self._pull_attrs()
        if not self._host_ok:
            if self._host.shape[1] < self._n:
                self._host = np.zeros((6, max(self._n, 16)), dtype=np.float64)
            rows = [self._host[c, : self._n] for c in range(6)]
            rows = [np.ascontiguousarray(r) for r in rows]
            self._dev.download_rows(rows)
            for c in range(6):
                self._host[c, : self._n] = rows[c]
            self._host_ok = True

    def _grow(self, need):
        cap = self._host.shape[1]
        if need <= cap:
            return
        newcap = max(need, 2 * cap)
        h = np.zeros((6, newcap), dtype=np.float64)
        h[:, : self._n] = self._host[:, : self._n]
        f = np.ones(newcap, dtype=np.int8)
        f[: self._n] = self._flag[: self._n]
        self._host, self._flag = h, f
        for name, arr in list(self._part_attr.items()):
            a = np.zeros((newcap, arr.shape[1]))
            a[: self._n] = arr[: self._n]
            self._part_attr[name] = a

    def _device_bunch(self, wait=True):
        """Device copy with current coordinates and reference-particle data.
        wait=False: an upload is only enqueued on the bunch's stream (so that
        host work can overlap it); the next host access to the coordinates
        (_ensure_host) waits for it first."""
        from orbit_gb300 import DeviceBunch, Sync  # noqa: WPS433
        if self._dev is None:
            self._dev = DeviceBunch()
            self._dev_ok = False
            self._sync_dirty = True
        if not self._dev_ok:
            self.compress()
            rows = [np.ascontiguousarray(self._host[c, : self._n]) for c in range(6)]
            self._dev.upload_rows(rows, self._n)
            self._upload_keepalive = rows
            if "macrosize" in self._part_attr:
                self._dev.set_macrosizes(self._part_attr["macrosize"][: self._n, 0])
            else:
                self._dev.set_macrosizes(None)
            if wait:
                self._dev.sync()
            else:
                self._upload_pending = True
            self._dev_ok = True
        if self._sync_dirty:
            s = self._sync
            self._dev.set_sync(Sync(s._beta, s._gamma, s._p_abs, self._mass, self._charge,
                                    self._classical_radius, self._macrosize, s._time))
            self._sync_dirty = False
        return self._dev

    def _device_modified(self):
        """Called after a device operation changed coordinates."""
        self._host_ok = False

    def _sync_changed(self):
        # keep the time the device maps advanced before the host copy wins
        if self._dev is not None and not self._sync_dirty:
            self._sync._time = self._dev.get_sync().time
        self._sync_dirty = True

    def _pull_time(self):
        if self._dev is not None and not self._sync_dirty:
            self._sync._time = self._dev.get_sync().time

    def _host_modified(self):
        self._dev_ok = False

    # -------------------------------------------------------- particles
    def addParticle(self, x, xp, y, yp, z, dE) -> int:
        self._ensure_host()
        self._grow(self._n + 1)
        i = self._n
        self._host[:, i] = (x, xp, y, yp, z, dE)
        self._flag[i] = 1
        for arr in self._part_attr.values():
            arr[i] = 0.0
        self._n += 1
        self._host_modified()
        return self._n

    def deleteParticleFast(self, index: int):
        self._ensure_host()
        self._flag[index] = 0
        self._host_modified()

    def deleteParticle(self, index: int):
        self.deleteParticleFast(index)
        self.compress()

    def deleteAllParticles(self):
        self._phase_dev = False
        self._n = 0
        self._host_ok = True
        self._host_modified()

    def compress(self):
        """Removes particles flagged dead (Bunch.cc:704-770)."""
        if self._n == 0 or bool(np.all(self._flag[: self._n] == 1)):
            return
        self._ensure_host()
        keep = np.nonzero(self._flag[: self._n] == 1)[0]
        m = keep.shape[0]
        self._host[:, :m] = self._host[:, keep]
        for name, arr in self._part_attr.items():
            arr[:m] = arr[keep]
        self._flag[:] = 1
        self._n = m
        self._host_modified()

    def flag(self, index: int) -> int:
        return int(self._flag[index])

    def _coord(self, c, index, value):
        self._ensure_host()
        if index < 0 or index >= self._n:
            raise IndexError("particle index %d out of range [0, %d)" % (index, self._n))
        if value is not None:
            self._host[c, index] = float(value)
            self._host_modified()
        return float(self._host[c, index])

    def x(self, i, v=None): return self._coord(0, i, v)
    def xp(self, i, v=None): return self._coord(1, i, v)
    def px(self, i, v=None): return self._coord(1, i, v)
    def y(self, i, v=None): return self._coord(2, i, v)
    def yp(self, i, v=None): return self._coord(3, i, v)
    def py(self, i, v=None): return self._coord(3, i, v)
    def z(self, i, v=None): return self._coord(4, i, v)
    def dE(self, i, v=None): return self._coord(5, i, v)
    def pz(self, i, v=None): return self._coord(5, i, v)

    # numpy extensions
    def getCoordinates(self, out=None) -> np.ndarray:
        """(6, n) copy of x, xp, y, yp, z, dE (into ``out`` if given)."""
        if out is not None and not self._host_ok and out.shape == (6, self._n) and out.dtype == np.float64 \
                and out.flags.c_contiguous:
            self._dev.download_rows([out[c] for c in range(6)])
            return out
        self._ensure_host()
        if out is None:
            return self._host[:, : self._n].copy()
        out[...] = self._host[:, : self._n]
        return out

    def setCoordinates(self, soa, copy=True):
        """Replaces all particles by the (6, n) array.  With copy=False a
        C-contiguous float64 array (e.g. in pinned memory) becomes the host
        storage itself, so uploads read it directly; an upload that
        trackBunch enqueued may still read it until the next host access to
        the coordinates, so write new values into it only after such an
        access (e.g. getCoordinates) and pass it here again."""
        soa = np.asarray(soa, dtype=np.float64)
        if soa.ndim != 2 or soa.shape[0] != 6:
            raise ValueError("expected a (6, n) array")
        n = soa.shape[1]
        if copy or not soa.flags.c_contiguous:
            self._host = np.array(soa, dtype=np.float64, order="C", copy=True)
        else:
            self._host = soa
        if n == 0:
            self._host = np.zeros((6, 16))
        self._flag = np.ones(max(n, 16), dtype=np.int8)
        for name, arr in list(self._part_attr.items()):
            self._part_attr[name] = np.zeros((max(n, 16), arr.shape[1]))
        self._phase_dev = False
        self._n = n
        self._host_ok = True
        self._host_modified()

    def ringwrap(self, ring_length: float):
        from orbit.teapot_base import TPB
        TPB.wrapbunch(self, ring_length)

    # --------------------------------------------------------- sizes
    def getSize(self) -> int:
        return self._n

    def getSizeGlobal(self) -> int:
        return self._n

    def getSizeGlobalFromMemory(self) -> int:
        return self._n

    def getTotalCount(self) -> int:
        return self._n

    def getCapacity(self) -> int:
        return self._host.shape[1]

    # --------------------------------------------------- bunch params
    def mass(self, value=None) -> float:
        if value is not None:  # Bunch::setMass (Bunch.cc:789-794)
            self._mass = float(value)
            self._attr_double["mass"] = self._mass
            self._update_classical_radius_attr()
            self._sync._update()
        return self._mass

    def charge(self, value=None) -> float:
        if value is not None:
            self._charge = float(value)
            self._attr_double["charge"] = self._charge
            self._update_classical_radius_attr()
            self._sync_changed()
        return self._charge

    def _update_classical_radius_attr(self):
        # Bunch::updateClassicalRadius (Bunch.cc:804-812) updates the
        # attribute only; the value the calculators read is unchanged.
        v = CLASSICAL_RADIUS_PROTON * MASS_PROTON / self._mass * self._charge * self._charge
        self._attr_double["classical_radius"] = v

    def classicalRadius(self) -> float:
        return self._classical_radius

    def macroSize(self, value=None) -> float:
        if value is not None:
            self._macrosize = float(value)
            self._attr_double["macro_size"] = self._macrosize
            self._sync_changed()
        return self._macrosize

    def B_Rho(self) -> float:  # Bunch.cc:781-787
        if self._charge != 0.0:
            return 3.335640952 * self._sync.momentum() / self._charge
        return 1.0e36

    def getSyncParticle(self) -> SyncPart:
        return self._sync

    # ---------------------------------------------- bunch attributes
    def bunchAttrDouble(self, name, value=None):
        if value is not None:
            self._attr_double[name] = float(value)
            if name == "mass":
                self._mass = float(value)
            elif name == "charge":
                self._charge = float(value)
            elif name == "classical_radius":
                self._classical_radius = float(value)
            elif name == "macro_size":
                self._macrosize = float(value)
            self._sync_changed()
        return self._attr_double[name]

    def bunchAttrInt(self, name, value=None):
        if value is not None:
            self._attr_int[name] = int(value)
        return self._attr_int[name]

    def bunchAttrDoubleNames(self):
        return tuple(self._attr_double.keys())

    def bunchAttrIntNames(self):
        return tuple(self._attr_int.keys())

    def hasBunchAttrDouble(self, name) -> int:
        return 1 if name in self._attr_double else 0

    def hasBunchAttrInt(self, name) -> int:
        return 1 if name in self._attr_int else 0

    # --------------------------------------- particle attributes
    _PART_ATTR_SIZES = {"macrosize": 1, "ParticleIdNumber": 1, "TurnNumber": 1, PHASE_ATTR: 6}

    def addPartAttr(self, name, params=None):
        if name in self._part_attr:
            return
        k = self._PART_ATTR_SIZES.get(name, 1)
        if params and "size" in params:
            k = int(params["size"])
        self._part_attr[name] = np.zeros((self._host.shape[1], k))
        self._part_attr_dict[name] = dict(params or {})
        if name == "macrosize":
            self._host_modified()

    def removePartAttr(self, name):
        if name == PHASE_ATTR:
            self._phase_dev = False
        self._part_attr.pop(name, None)
        self._part_attr_dict.pop(name, None)
        if name == "macrosize":
            self._host_modified()

    def removeAllPartAttr(self):
        for name in list(self._part_attr):
            self.removePartAttr(name)

    def hasPartAttr(self, name) -> int:
        return 1 if name in self._part_attr else 0

    def getPartAttrNames(self):
        return tuple(self._part_attr.keys())

    def getPartAttrSize(self, name) -> int:
        return self._part_attr[name].shape[1]

    def partAttrValue(self, name, index, attr_index, value=None):
        self._pull_attrs()
        arr = self._part_attr[name]
        if value is not None:
            arr[index, attr_index] = float(value)
            if name == "macrosize":
                self._host_modified()
        return float(arr[index, attr_index])

    # ----------------------------------------------------- copies
    def copyEmptyBunchTo(self, other: "Bunch"):
        other._mass, other._charge = self._mass, self._charge
        other._classical_radius, other._macrosize = self._classical_radius, self._macrosize
        other._attr_double = dict(self._attr_double)
        other._attr_int = dict(self._attr_int)
        other._sync._pxyz = list(self._sync._pxyz)
        other._sync._xyz = list(self._sync._xyz)
        other._sync._time = self._sync.time()
        other._sync._update()
        for name in self._part_attr:
            other.addPartAttr(name, self._part_attr_dict.get(name))

    def copyBunchTo(self, other: "Bunch"):
        self.copyEmptyBunchTo(other)
        other.deleteAllParticles()
        self.addParticlesTo(other)

    def addParticlesTo(self, other: "Bunch"):
        self._ensure_host()
        other._ensure_host()
        m = self._n
        base = other._n
        other._grow(base + m)
        other._host[:, base:base + m] = self._host[:, :m]
        other._flag[base:base + m] = self._flag[:m]
        for name, arr in self._part_attr.items():
            if name in other._part_attr:
                other._part_attr[name][base:base + m] = arr[:m]
        other._n = base + m
        other._host_modified()

    # ----------------------------------------------------- I/O
    # Column descriptions the reference's attribute classes print
    # (attrDescr in src/orbit/ParticlesAttributes/*.cc), by factory name
    # (ParticleAttributesFactory.cc).
    _ATTR_DESCR = {"empty": "no attributes", "macrosize": "macro_size", "ParticleIdNumber": "Particle_Id_Number",
                   "LostParticleAttributes": "Pos (m)", PHASE_ATTR: "PhaseVars", "Amplitudes": "Ampls",
                   "Populations": "Pops", "pq_coords": "Coords", "part_time": "time", "Evolution": "Evol",
                   "TurnNumber": "TurnNumber"}

    @staticmethod
    def _g(v, prec):
        """A double as a C++ ostream prints it with setprecision(prec)."""
        return "%.*g" % (prec, v)

    def dumpBunch(self, fileName=None):
        """Text dump in the layout of Bunch::print (Bunch.cc:894-980) and
        SyncPart::print (SyncPart.cc:465-536): attribute controller names
        and their parameter dictionaries (keys in std::map order), bunch
        attributes by name, the synchronous particle at 14 digits, then one
        line per live particle at 8 digits."""
        self._ensure_host()
        g = self._g
        names = list(self._part_attr.keys())
        lines = ["% PARTICLE_ATTRIBUTES_CONTROLLERS_NAMES " + "".join(n + " " for n in names)]
        for n in names:
            d = dict(self._part_attr_dict.get(n) or {})
            d["size"] = float(self._part_attr[n].shape[1])
            lines.append("% PARTICLE_ATTRIBUTES_CONTROLLER_DICT " + n + " " +
                         "".join("%s %s " % (k, g(d[k], 6)) for k in sorted(d)))
        for name in sorted(self._attr_int):
            lines.append("%% BUNCH_ATTRIBUTE_INT %s   %d " % (name, self._attr_int[name]))
        for name in sorted(self._attr_double):
            lines.append("%% BUNCH_ATTRIBUTE_DOUBLE %s   %s " % (name, g(self._attr_double[name], 6)))
        s = self._sync
        t = s.time()
        lines += [
            "%%  SYNC_PART_COORDS %s %s %s  x, y, z positions in [m]" % tuple(g(v, 14) for v in s._xyz),
            "%%  SYNC_PART_MOMENTUM %s %s %s  px, py, pz momentum component in GeV/c" % tuple(g(v, 14) for v in s._pxyz),
            "%%  SYNC_PART_X_AXIS %s %s %s  nxx, nxy, pxz - x-axis ort coordinates" % tuple(g(v, 14) for v in s._nx),
            "%%  info only: energy of the synchronous particle [GeV] = %s " % g(s.kinEnergy(), 14),
            "%%  info only: momentum of the synchronous particle [GeV/c] = %s " % g(s.momentum(), 14),
            "%%  info only: beta=v/c of the synchronous particle = %s " % g(s.beta(), 14),
            "%%  info only: gamma=1/sqrt(1-(v/c)**2) of the synchronous particle = %s " % g(s.gamma(), 14),
            "%%  SYNC_PART_TIME %s  time in [sec]" % g(t, 14),
            "% x[m] px[rad] y[m] py[rad] z[m]  (pz or dE [GeV]) " +
            "".join(self._ATTR_DESCR.get(n, "no attributes") + " " for n in names),
        ]
        live = np.nonzero(self._flag[: self._n] > 0)[0]
        cols = [self._host[:, : self._n]] + [self._part_attr[n][: self._n].T for n in names]
        table = np.vstack(cols)[:, live].T
        body = ["".join("%.8g " % v for v in row) for row in table]
        text = "\n".join(lines + body) + "\n"
        if fileName is None:
            print(text, end="")
        else:
            with open(fileName, "w") as f:
                f.write(text)

    def readBunch(self, fileName, nParts=-1):
        """Reads a bunch text file as the reference's readBunch does
        (wrap_bunch.cc:1087-1119): bunch attributes and the synchronous
        particle from the header (Bunch::initBunchAttributes,
        SyncPart.cc:360-460), the particle attribute controllers with their
        parameter dictionaries (Bunch.cc:1287-1420: every existing attribute
        is removed first), then the particle lines appended to the bunch
        (Bunch.cc:1116-1264: 6 or 6 + attribute-width numbers per line, at
        most nParts particles).  Returns the bunch size."""
        names, dicts = [], {}
        header = []
        with open(fileName) as f:
            lines = f.read().splitlines()
        k = 0
        while k < len(lines) and lines[k].startswith("%"):
            tok = lines[k].split()
            header.append(tok)
            if len(tok) > 2 and tok[1] == "PARTICLE_ATTRIBUTES_CONTROLLERS_NAMES":
                names = tok[2:]
            elif len(tok) > 2 and tok[1] == "PARTICLE_ATTRIBUTES_CONTROLLER_DICT":
                dicts[tok[2]] = {tok[i]: float(tok[i + 1]) for i in range(3, len(tok) - 1, 2)}
            k += 1
        for tok in header:
            if len(tok) > 3 and tok[1] == "BUNCH_ATTRIBUTE_INT":
                self.bunchAttrInt(tok[2], int(tok[3]))
            elif len(tok) > 3 and tok[1] == "BUNCH_ATTRIBUTE_DOUBLE":
                self.bunchAttrDouble(tok[2], float(tok[3]))
            elif len(tok) > 4 and tok[1] == "SYNC_PART_COORDS":
                self._sync.rVector([float(t) for t in tok[2:5]])
            elif len(tok) > 4 and tok[1] == "SYNC_PART_MOMENTUM":
                self._sync.pVector([float(t) for t in tok[2:5]])
            elif len(tok) > 4 and tok[1] == "SYNC_PART_X_AXIS":
                self._sync._nx = [float(t) for t in tok[2:5]]
            elif len(tok) > 2 and tok[1] == "SYNC_PART_TIME":
                self._sync.time(float(tok[2]))
        self.removeAllPartAttr()
        for n in names:
            self.addPartAttr(n, dicts.get(n))
        width = 6 + sum(self._part_attr[n].shape[1] for n in names)
        rows = []
        for ln in lines[k:]:
            tok = ln.split()
            if not tok or tok[0].startswith("%"):
                continue
            if len(tok) != width and len(tok) != 6:
                raise ValueError("readBunch: %s: a particle line has %d numbers, expected 6 or %d"
                                 % (fileName, len(tok), width))
            rows.append([float(t) for t in tok] + [0.0] * (width - len(tok)))
            if 0 <= nParts <= len(rows):
                break
        self._ensure_host()
        base = self._n
        m = len(rows)
        self._grow(base + m)
        if m:
            arr = np.array(rows, dtype=np.float64)
            self._host[:, base:base + m] = arr[:, :6].T
            self._flag[base:base + m] = 1
            col = 6
            for n in names:
                w = self._part_attr[n].shape[1]
                self._part_attr[n][base:base + m] = arr[:, col:col + w]
                col += w
        self._n = base + m
        self._host_modified()
        return self._n


class BunchTwissAnalysis:
    """First and second moments, rms emittances, Twiss parameters and
    dispersion (src/orbit/BunchDiagnostics/BunchTwissAnalysis.cc:49-140,
    343-531).  analyzeBunch reduces the moments on the device where the
    coordinates live (a deterministic two-level sum: per-block partials, then
    the blocks in a fixed order) and reads back 29 numbers; the getters are
    the reference's host formulas over those moments."""

    def __init__(self):
        self._avg = np.zeros(6)
        self._corr = np.zeros((6, 6))
        self._count = 0
        self._total_m = 0.0
        self._momentum = 0.0
        self._beta = 0.0
        self._gamma = 1.0
        self._kin = 0.0
        self._mass = 0.0

    def analyzeBunch(self, bunch: Bunch):
        bunch.compress()
        self._load(bunch._device_bunch().moments(), bunch.getSyncParticle())

    def computeBunchMoments(self, bunch: Bunch, order, dispersionflag=0, emitnormflag=0):
        """The x-y moment table of BunchTwissAnalysis::computeBunchMoments
        (BunchTwissAnalysis.cc:146-340), summed on the device with the
        reference's recurrences, normalisation and fixed cells: centred on
        the averages of analyzeBunch (its dispersion-corrected average is
        never taken: dispterm is zero where the reference tests it), divided
        by sqrt(beta) (emitnormflag: sqrt(beta * emittance)) per power, x
        corrected by D dE / (E_kin + m) / beta^2 with dispersionflag.  The
        reference's uniform-macrosize loop also adds momX[2] momY[order]
        once per particle after its loops (cell [2][order], not
        normalised), reproduced here.  order >= 2 (for order 1 that write
        falls outside the reference's table)."""
        order = int(order)
        if order < 2:
            raise ValueError("computeBunchMoments: order >= 2")
        self.analyzeBunch(bunch)
        D = self.getDispersion(0) if dispersionflag > 0 else 0.0
        if emitnormflag > 0:
            xb = math.sqrt(self.getBeta(0) * self.getEmittance(0))
            yb = math.sqrt(self.getBeta(1) * self.getEmittance(1))
        else:
            xb = math.sqrt(self.getBeta(0))
            yb = math.sqrt(self.getBeta(1))
        params = [D, self._kin + self._mass, self._beta * self._beta, self.getAverage(0), self.getAverage(2), xb, yb]
        self._order = order
        self._mom_xy = bunch._device_bunch().xy_moments(order, params)

    def getBunchMoment(self, i, j):
        """(BunchTwissAnalysis.cc:350-353)"""
        order = getattr(self, "_order", -1)
        if i < 0 or i > order or j < 0 or j > order:
            return 0.0
        return float(self._mom_xy[i, j])

    def _load(self, mom, s):
        """Takes the 29 moments {count, total macrosize, averages, <c_i c_j>
        (i >= j)} and the reference particle's kinematics."""
        self._count = int(mom[0])
        self._total_m = float(mom[1])
        self._avg = mom[2:8].copy()
        corr = np.zeros((6, 6))
        k = 8
        for i in range(6):  # BunchTwissAnalysis.cc:126-133: symmetric fill
            for j in range(i + 1):
                corr[i, j] = corr[j, i] = mom[k]
                k += 1
        self._corr = corr
        self._momentum, self._beta, self._gamma = s.momentum(), s.beta(), s.gamma()
        self._kin, self._mass = s.kinEnergy(), s.mass()

    # The getters compute in numpy float64 so that a zero denominator gives
    # inf or nan as the reference's C arithmetic does, not an exception.
    def getCorrelation(self, i, j):
        if i < 0 or i > 5 or j < 0 or j > 5:
            return 0.0
        return float(np.float64(self._corr[i, j]) - np.float64(self._avg[i]) * np.float64(self._avg[j]))

    def getAverage(self, i):
        if i < 0 or i > 5:
            return 0.0
        return float(self._avg[i])

    def getGlobalCount(self):
        return self._count

    def getGlobalMacrosize(self):
        return self._total_m

    def _plane(self, ic):
        C = lambda a, b: np.float64(self.getCorrelation(a, b))  # noqa: E731
        return (abs(C(2 * ic, 2 * ic)), abs(C(2 * ic + 1, 2 * ic + 1)), C(2 * ic, 2 * ic + 1),
                C(2 * ic, 5), C(2 * ic + 1, 5), abs(C(5, 5)))

    def getEmittance(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        x2, xp2, xxp, xdE, xpdE, dE2 = self._plane(ic)
        with np.errstate(all="ignore"):
            if ic == 2 or dE2 == 0:
                return float(np.sqrt(abs(x2 * xp2 - xxp * xxp)))
            return float(np.sqrt(abs((x2 - xdE * xdE / dE2) * (xp2 - xpdE * xpdE / dE2)
                                     - (xxp - xdE * xpdE / dE2) * (xxp - xdE * xpdE / dE2))))

    def getEmittanceNormalized(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        if ic == 2:
            return self.getEmittance(ic)
        return float(np.float64(self.getEmittance(ic)) * self._gamma * self._beta)

    def getAlpha(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        x2, xp2, xxp, xdE, xpdE, dE2 = self._plane(ic)
        e = np.float64(self.getEmittance(ic))
        with np.errstate(all="ignore"):
            if ic == 2:
                return float(-xxp / e)
            return float(-(xxp - xdE * xpdE / dE2) / e)

    def getBeta(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        x2, xp2, xxp, xdE, xpdE, dE2 = self._plane(ic)
        e = np.float64(self.getEmittance(ic))
        with np.errstate(all="ignore"):
            if ic == 2:
                return float(x2 / e)
            return float((x2 - xdE * xdE / dE2) / e)

    def getGamma(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        x2, xp2, xxp, xdE, xpdE, dE2 = self._plane(ic)
        e = np.float64(self.getEmittance(ic))
        with np.errstate(all="ignore"):
            if ic == 2:
                return float(xp2 / e)
            return float((xp2 - xpdE * xpdE / dE2) / e)

    def getDispersion(self, ic):
        if ic < 0 or ic > 1:
            return 0.0
        x2, xp2, xxp, xdE, xpdE, dE2 = self._plane(ic)
        with np.errstate(all="ignore"):
            return float(xdE / dE2 * self._momentum * self._beta)

    def getDispersionDerivative(self, ic):
        if ic < 0 or ic > 1:
            return 0.0
        x2, xp2, xxp, xdE, xpdE, dE2 = self._plane(ic)
        with np.errstate(all="ignore"):
            return float(xpdE / dE2 * self._momentum * self._beta)

    def _effective(self, ic):
        x2, xp2, xxp = self._plane(ic)[:3]
        return x2, xp2, xxp, x2 * xp2 - xxp * xxp

    def getEffectiveEmittance(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        e2 = self._effective(ic)[3]
        return float(np.sqrt(abs(e2)))

    def getEffectiveAlpha(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        x2, xp2, xxp, e2 = self._effective(ic)
        if e2 <= 0.0:
            return 0.0
        return float(-xxp / np.sqrt(e2))

    def getEffectiveBeta(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        x2, xp2, xxp, e2 = self._effective(ic)
        if e2 <= 0.0:
            return 0.0
        return float(x2 / np.sqrt(e2))

    def getEffectiveGamma(self, ic):
        if ic < 0 or ic > 2:
            return 0.0
        x2, xp2, xxp, e2 = self._effective(ic)
        if e2 <= 0.0:
            return float(np.finfo(np.float64).max)  # DBL_MAX
        return float(xp2 / np.sqrt(e2))


class BunchTuneAnalysis:
    """Per-particle betatron phases, phase advances ("tunes") and actions
    (src/orbit/BunchDiagnostics/BunchTuneAnalysis.cc:27-108).  The six
    values per particle live in the bunch's ParticlePhaseAttributes; while
    successive analyses run on the device they stay there, and the host
    attribute is refreshed only when the host reads it."""

    def __init__(self):
        self._twiss = np.zeros(6)

    def assignTwiss(self, betax, alphax, etax, etapx, betay, alphay):
        self._twiss = np.array([betax, alphax, etax, etapx, betay, alphay], dtype=np.float64)

    def analyzeBunch(self, bunch: Bunch):
        bunch.compress()
        if not bunch.hasPartAttr(PHASE_ATTR):
            bunch.addPartAttr(PHASE_ATTR)
        dev = bunch._device_bunch()
        if not bunch._phase_dev:
            dev.phase_set(np.ascontiguousarray(bunch._part_attr[PHASE_ATTR][: bunch._n, :6].T))
        s = bunch.getSyncParticle()
        dev.tune_analysis(self._twiss, s.kinEnergy() + s.mass())  # BunchTuneAnalysis.cc:63
        bunch._phase_dev = True


__all__ = ["Bunch", "SyncPart", "BunchTwissAnalysis", "BunchTuneAnalysis"]
