"""The reference's input and output files, read and written by the host driver.

What a ``metrosim`` user hands the simulator and gets back, restated from the
reference's host code so that a run of this package starts from the same
SimBox rows and writes files the reference reads:

* ``.config``   key=value settings             ConfigScanner.cpp:20-227
* OPLS ``.par`` atom parameter table             OplsScanner.cpp:19-110
* ``.z``        z-matrix molecule templates      ZmatrixScanner.cpp:21-286, 290-573
* ``oplsaa.sb`` bond and angle parameter table   SBScanner.cpp:11-148
* z-matrix -> XYZ of each template               MathLibrary.cpp:751-903
* box of N molecules on an FCC lattice           FileUtilities.cpp:285-642
* ``.state``    text checkpoint (read and write) StateScanner.cpp:18-597
* SimBox rows (coordinates, sigma/epsilon/charge, molecule ranges, primary
  indexes) after Simulation::run's keepMoleculeInBox   SimBoxBuilder.cpp:10-299,
                                                       Box.cpp:84-109, 170-179
* SimBox bond, angle and exclusion rows          SimBoxBuilder.cpp:44-278
* ``.pdb`` and ``.results`` outputs              Simulation.cpp:296-417
* long-range LJ correction                       SerialCalcs.cpp:37-107

Scalars are parsed the way the C library and the C++ streams parse them
(``atof``/``atoi`` take the longest numeric prefix; ``stream >> int`` stops at
the first non-digit) and printed the way ``std::ostream`` prints them (``%g``,
six significant digits), so a file written here is byte-identical to the
reference's for the same rows.  Where the reference reads out of bounds or
dereferences a null name on malformed input, this module raises
``FileFormatError`` instead; where its behaviour is odd but defined (a
``[section]`` line is an error, the FCC builder uses the x edge for all three
dimensions, a three-atom first template stops the XYZ build of later ones),
it is kept.
"""
from __future__ import annotations

import math
import os
import re
import time
from dataclasses import dataclass, field

import numpy as np

from .workloads import PAIR_EXCLUDED, PAIR_FUDGE, PAIR_FULL, BoxData, Topology

# MathLibrary.h:51 -- the reference's truncated pi (z-matrix angles, LRC)
REF_PI = 3.14159265
# SimBox.h:16
K_BOLTZ = 0.00198717
# FileUtilities.cpp:17
DEFAULT_STEP_COUNT = 100
# FileUtilities.h:22
_TRIMMED = " \n\r\t"


class FileFormatError(ValueError):
    """An input file the reference rejects (its message), or one it would
    read out of bounds."""


# ---- C scalar parsing -----------------------------------------------------------

_NUM = r"[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)"
_ATOF = re.compile(r"[ \t\n\v\f\r]*(" + _NUM + ")", re.IGNORECASE)
_ATOI = re.compile(r"[ \t\n\v\f\r]*([+-]?\d+)")


def atof(s: str) -> float:
    """C atof: the longest numeric prefix after leading white space, else 0."""
    m = _ATOF.match(s)
    return float(m.group(1)) if m else 0.0


def _wrap_int(v: int) -> int:
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= (1 << 31) else v


def atoi(s: str) -> int:
    """C atoi: the longest integer prefix after leading white space, else 0."""
    m = _ATOI.match(s)
    return _wrap_int(int(m.group(1))) if m else 0


class _Stream:
    """``std::istringstream`` extraction (>> int, >> double, >> string) with
    the stream's sticky fail state."""

    _INT = re.compile(r"[+-]?\d+")
    _DBL = re.compile(r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?")

    def __init__(self, s: str):
        self.s = s
        self.i = 0
        self.ok = True

    def _skip(self) -> None:
        while self.i < len(self.s) and self.s[self.i] in " \t\n\v\f\r":
            self.i += 1

    def _num(self, rx, conv):
        if not self.ok:
            return None
        self._skip()
        m = rx.match(self.s, self.i)
        if not m:
            self.ok = False
            return None
        self.i = m.end()
        return conv(m.group(0))

    def int(self):
        return self._num(self._INT, int)

    def float(self):
        return self._num(self._DBL, float)

    def str(self):
        if not self.ok:
            return None
        self._skip()
        j = self.i
        while j < len(self.s) and self.s[j] not in " \t\n\v\f\r":
            j += 1
        if j == self.i:
            self.ok = False
            return None
        tok, self.i = self.s[self.i:j], j
        return tok

    def peek(self) -> str:
        return self.s[self.i] if self.i < len(self.s) else ""


def fmt_g(v: float) -> str:
    """``std::ostream << double`` with default flags (six significant digits)."""
    return "%g" % v


def _lines(path: str) -> list[str]:
    """The lines ``while (good()) getline(...)`` sees: split on '\\n' only
    (a '\\r' stays part of its line), a final empty line after a trailing
    newline."""
    with open(path, "rb") as f:
        data = f.read().decode("latin-1")
    return data.split("\n")


def _strtok(s: str) -> list[str]:
    """strtok(line, " ") tokens: runs of characters other than ' '."""
    return [t for t in s.split(" ") if t]


# ---- structures (StructLibrary.h) ----------------------------------------------

@dataclass
class Atom:
    id: int
    x: float
    y: float
    z: float
    sigma: float
    epsilon: float
    charge: float
    name: str


@dataclass
class Bond:
    atom1: int
    atom2: int
    distance: float
    variable: bool = False


@dataclass
class Angle:
    atom1: int
    atom2: int
    value: float
    variable: bool = False
    common: int = 0


@dataclass
class Dihedral:
    atom1: int
    atom2: int
    value: float
    variable: bool = False


@dataclass
class Hop:
    atom1: int
    atom2: int
    hop: int


@dataclass
class Molecule:
    id: int
    type: int
    atoms: list
    bonds: list = field(default_factory=list)
    angles: list = field(default_factory=list)
    dihedrals: list = field(default_factory=list)
    hops: list = field(default_factory=list)

    def copy(self) -> "Molecule":
        c = lambda xs: [type(v)(**v.__dict__) for v in xs]
        return Molecule(self.id, self.type, c(self.atoms), c(self.bonds), c(self.angles),
                        c(self.dihedrals), c(self.hops))


@dataclass
class Environment:
    """Environment (StructLibrary.h:296-360) with its constructor defaults."""
    x: float = 0.0
    y: float = 0.0
    z: float = 0.0
    cutoff: float = 0.0
    temp: float = 0.0
    max_translation: float = 0.0
    max_rotation: float = 0.0
    max_bond_delta: float = 0.06
    max_angle_delta: float = 3.1
    n_atoms: int = 0
    n_molecules: int = 0
    primary_line: str = "0"
    primary_defs: int = 0
    primary: list = field(default_factory=list)   # per molecule type: 0-based atom slots
    random_seed: int = 0
    pressure: float = 0.0

    def copy(self) -> "Environment":
        e = Environment(**self.__dict__)
        e.primary = [list(v) for v in self.primary]
        return e


def parse_primary_definitions(definitions: str, lists: list) -> int:
    """parsePrimaryIndexDefinitions (ConfigScanner.cpp:230-271,
    StateScanner.cpp:499-540): comma-separated 1-based atom numbers, one
    definition per molecule type, appended to ``lists`` (0-based slots)
    from index 0 of it; ``[a,b,...]`` gives one type several primary atoms.
    Every number also appends an empty list, as the reference's parser
    does, so ``lists`` can be longer than the definition count (only the
    count is checked against the templates).  Returns the count."""
    toks = [t for t in definitions.split(",") if t]
    ndef = 0
    k = 0
    i = 0
    while k < len(toks):
        tok = toks[k]
        ndef += 1
        if "[" in tok:
            tok = tok[1:]
            while "]" not in tok:
                lists.append([])
                lists[i].append(atoi(tok) - 1)
                k += 1
                if k >= len(toks):
                    raise FileFormatError("unterminated '[' in primary atom definitions: "
                                          + definitions)
                tok = toks[k]
            tok = tok[:tok.index("]")]
        lists.append([])
        lists[i].append(atoi(tok) - 1)
        k += 1
        i += 1
    return ndef


# ---- .config (ConfigScanner.cpp:20-227) -----------------------------------------

@dataclass
class Config:
    env: Environment
    path: str = ""
    steps: int = 0
    opls_path: str = ""
    zmatrix_path: str = ""
    state_path: str = ""
    state_output: str = ""
    pdb_output: str = ""
    sim_name: str = ""
    strategy: str = ""
    ensemble: str = ""
    ewald_radius: int = 0
    volume_interval: int = 0
    use_zmatrix: bool = False
    use_state: bool = False
    notes: list = field(default_factory=list)   # the reference's INFO messages


def read_config(path: str) -> Config:
    """ConfigScanner::readInConfig: ``key=value`` lines, ``#``/``;``
    comments, blank lines ignored; an unknown key or a line without '=' is an
    error.  The key is everything before the first '=' (no trimming), so
    ``x = 1`` is the unknown key ``'x '``, as in the reference."""
    if not path:
        raise FileFormatError("Configuration File path is empty")
    if not os.path.isfile(path):
        raise FileFormatError("Unable to open configuration file (" + path + ")")
    cfg = Config(env=Environment(), path=path)
    env = cfg.env
    safe = True

    def need(value: str, msg: str) -> str:
        if not value:
            raise FileFormatError(msg)
        return value

    for line in _lines(path):
        line = line.rstrip(_TRIMMED).lstrip(_TRIMMED)
        if not line or line[0] in "#;":
            continue
        split = line.find("=")
        if split < 0:
            raise FileFormatError('Error: Configuration File not well formed.\n'
                                  'Offending line: "' + line + '"')
        key, value = line[:split], line[split + 1:]
        if key == "x":
            env.x = atof(need(value, "Error: Config File: Missing environment X value."))
        elif key == "y":
            env.y = atof(need(value, "Error: Config File: Missing environment Y value."))
        elif key == "z":
            env.z = atof(need(value, "Configuration file not well formed. Missing environment "
                                     "z value."))
        elif key == "temp":
            env.temp = atof(need(value, "Configuration file not well formed. Missing "
                                        "environment temperature value."))
        elif key == "max-translation":
            env.max_translation = atof(need(value, "Configuration file not well formed. "
                                                   "Missing environment max translation value."))
        elif key == "steps":
            cfg.steps = atoi(need(value, "Configuration file not well formed. Missing number "
                                         "of steps value."))
        elif key == "molecules":
            env.n_molecules = atoi(need(value, "Configuration file not well formed. Missing "
                                               "number of molecules value."))
        elif key == "opla.par":
            cfg.opls_path = need(value, "Configuration file not well formed. Missing "
                                        "oplsuapar path value.")
        elif key == "z-matrix":
            if value:
                cfg.zmatrix_path = value
                cfg.use_zmatrix = cfg.use_state = True
            else:
                cfg.notes.append("INFO: Configuration file not well formed. Missing z-matrix "
                                 "path value. Attempting to rely on prior state information...")
                safe = False
                cfg.use_zmatrix = False
                cfg.use_state = True
        elif key == "state-input":
            if value:
                cfg.state_path = value
                cfg.use_zmatrix = False
                cfg.use_state = True
            elif not safe:
                raise FileFormatError("Configuration file not well formed. Missing value "
                                      "pointing to prior state file path. Cannot safely "
                                      "continue with program execution.")
            else:
                cfg.notes.append("INFO: Value pointing to prior state file path not found in "
                                 "main config file. Environment setup defaulting to clean "
                                 "simulation.")
                cfg.use_zmatrix = True
                cfg.use_state = False
                safe = True
        elif key == "state-output":
            cfg.state_output = need(value, "Configuration file not well formed. Missing state "
                                           "file output path value.")
        elif key == "pdb-output":
            cfg.pdb_output = need(value, "Configuration file not well formed. Missing PDB "
                                         "output path value.")
        elif key == "cutoff":
            env.cutoff = atof(need(value, "Configuration file not well formed. Missing "
                                          "environment cutoff value."))
        elif key == "max-rotation":
            env.max_rotation = atof(need(value, "Configuration file not well formed. Missing "
                                                "environment max rotation value."))
        elif key == "random-seed":
            env.random_seed = atoi(value) if value else (int(time.time()) & 0xFFFFFFFF)
            env.random_seed = _wrap_int(env.random_seed)
        elif key == "primary-atom":
            need(value, "Configuration file not well formed. Missing environment primary "
                        "atom index value.")
            env.primary_line = value
            env.primary_defs += parse_primary_definitions(value, env.primary)
        elif key == "sim-name":
            if value:
                cfg.sim_name = value
        elif key == "strategy":
            if value:
                cfg.strategy = value
        elif key == "max-bond-delta":
            env.max_bond_delta = atof(value)
        elif key == "max-angle-delta":
            env.max_angle_delta = atof(value)
        elif key == "ensemble":
            if value:
                cfg.ensemble = value
        elif key == "pressure":
            env.pressure = atof(need(value, "Configuration file not well formed. Missing "
                                            "environment pressure value."))
        elif key == "ewald-radius":
            if value:
                cfg.ewald_radius = atoi(value)
        elif key == "volume-interval":
            if value:
                cfg.volume_interval = atoi(value)
        else:
            raise FileFormatError("Unexpected key encountered: " + key)
    return cfg


# ---- OPLS parameter table (OplsScanner.cpp:19-110) -------------------------------

@dataclass
class OplsTable:
    atoms: dict = field(default_factory=dict)      # hash -> (sigma, epsilon, charge, name)
    fourier: dict = field(default_factory=dict)    # hash -> (v0, v1, v2, v3)
    bad_lines: list = field(default_factory=list)
    duplicate_atoms: list = field(default_factory=list)
    duplicate_fourier: list = field(default_factory=list)

    def atom(self, key: str) -> Atom:
        """OplsScanner::getAtom.  The reference returns a nameless atom for an
        unknown type and crashes when it is written out; this raises."""
        if key not in self.atoms:
            raise FileFormatError("Index does not exist: " + key)
        s, e, q, name = self.atoms[key]
        return Atom(0, -1.0, -1.0, -1.0, s, e, q, name)


def _opls_format(line: str) -> int:
    """OplsScanner::checkFormat: 2 = dihedral V-values line (int + 4 reals),
    1 = atom line (hash, int, name, charge, sigma, epsilon), -1 neither."""
    s = _Stream(line)
    if s.int() is not None and all(s.float() is not None for _ in range(4)):
        return 2
    s = _Stream(line)
    if (s.int() is not None and s.int() is not None and s.str() is not None
            and all(s.float() is not None for _ in range(3))):
        return 1
    return -1


def read_opls(path: str) -> OplsTable:
    """OplsScanner::readInOpls: the first line is a title; lines starting
    with '#' and empty lines are skipped; the first entry of a hash wins."""
    if not path:
        raise FileFormatError("Error: readInOpls(): empty filename given")
    if not os.path.isfile(path):
        raise FileFormatError("Error: readInOpls(): could not open file (" + path + ")")
    t = OplsTable()
    for n, line in enumerate(_lines(path), 1):
        if not line or line[0] == "#" or n <= 1:
            continue
        fmt = _opls_format(line)
        s = _Stream(line)
        if fmt == 1:
            key = s.str()
            s.int()
            name = s.str()
            q, sg, ep = s.float(), s.float(), s.float()
            if key in t.atoms:
                t.duplicate_atoms.append(key)
            else:
                t.atoms[key] = (sg, ep, q, name)
        elif fmt == 2:
            key = s.str()
            v = tuple(s.float() for _ in range(4))
            if key in t.fourier:
                t.duplicate_fourier.append(key)
            else:
                t.fourier[key] = v
        else:
            t.bad_lines.append(n)
    return t


# ---- bond and angle table (SBScanner.cpp) -----------------------------------------

@dataclass
class SbTable:
    """SBScanner's maps: bond (force constant, equilibrium distance) by the
    two atom names, angle (force constant, equilibrium angle) by end, middle
    and end name.  Later lines overwrite earlier ones; each entry is stored
    under both orders of its ends (SBScanner.cpp:11-61)."""
    bonds: dict = field(default_factory=dict)     # a1 -> a2 -> (k, eq)
    angles: dict = field(default_factory=dict)    # e1 -> mid -> e2 -> (k, eq)

    def k_bond(self, a1: str, a2: str) -> float:
        """getKBond (:124-128): -1 when the pair is not in the table."""
        return self.bonds.get(a1, {}).get(a2, (-1.0, -1.0))[0]

    def eq_bond(self, a1: str, a2: str) -> float:
        """getEqBondDist (:130-134): -1 when the pair is not in the table."""
        return self.bonds.get(a1, {}).get(a2, (-1.0, -1.0))[1]

    def k_angle(self, e1: str, mid: str, e2: str) -> float:
        """getKAngle (:136-141): -1 when the triple is not in the table."""
        return self.angles.get(e1, {}).get(mid, {}).get(e2, (-1.0, -1.0))[0]

    def eq_angle(self, e1: str, mid: str, e2: str) -> float:
        """getEqAngle (:143-148): -1 when the first end or the middle is
        missing, but 0 when only the second end is (the reference's own
        return value for that branch)."""
        if e1 not in self.angles or mid not in self.angles[e1]:
            return -1.0
        return self.angles[e1][mid].get(e2, (-1.0, 0.0))[1]


def _substr(s: str, pos: int, n: int) -> str:
    """std::string::substr: out_of_range when pos > size."""
    if pos > len(s):
        raise IndexError(pos)
    return s[pos:pos + max(n, 0)]


def _sb_values(rest: str) -> tuple[float, float]:
    """``ss >> a >> b``: a failed first extraction writes 0 and stops the
    stream; the second value is then left as the reference left it
    (uninitialised there; 0 here)."""
    s = _Stream(rest)
    a = s.float()
    b = s.float()
    return (0.0 if a is None else a), (0.0 if b is None else b)


def read_sb(path: str) -> SbTable:
    """SBScanner::readInSB (SBScanner.cpp:76-108): every line not starting
    with '*', '"' or '#' is an angle when its sixth character is '-'
    (``E1-MD-E2 k theta``: names in columns 1-2, 4-5, 7-8, one-letter names
    padded with a blank), else a bond (``A1-A2 k r``, columns 1-2 and 4-5,
    values from column 7).  A line too short for its fields is skipped, as
    the reference's out_of_range handler skips it."""
    if not path:
        raise FileFormatError("Error: readInOpls(): empty filename given")
    if not os.path.isfile(path):
        raise FileFormatError("Error: readInOpls(): could not open file (" + path + ")")
    t = SbTable()
    for line in _lines(path):
        if not line or line[0] in "*\"#":
            continue
        try:
            if len(line) > 5 and line[5] == "-":
                e1, mid, e2 = _substr(line, 0, 2), _substr(line, 3, 2), _substr(line, 6, 2)
                if _substr(line, 1, 1) == " ":
                    e1 = e1[:1]
                if _substr(line, 4, 1) == " ":
                    mid = mid[:1]
                if _substr(line, 7, 1) == " ":
                    e2 = e2[:1]
                k, eq = _sb_values(_substr(line, 8, len(line) - 8))
                t.angles.setdefault(e1, {}).setdefault(mid, {})[e2] = (k, eq)
                t.angles.setdefault(e2, {}).setdefault(mid, {})[e1] = (k, eq)
            else:
                a1 = _substr(line, 0, 1) if _substr(line, 1, 1) == " " else _substr(line, 0, 2)
                a2 = _substr(line, 3, 1) if _substr(line, 4, 1) == " " else _substr(line, 3, 2)
                if len(line) < 6:
                    raise IndexError(6)
                k, eq = _sb_values(_substr(line, 6, len(line) - 6))
                t.bonds.setdefault(a1, {})[a2] = (k, eq)
                t.bonds.setdefault(a2, {})[a1] = (k, eq)
        except IndexError:
            continue
    return t


# ---- z-matrix (ZmatrixScanner.cpp) ------------------------------------------------

_ZMARKERS = (("TERZ", 2), ("Geometry Variations", 3), ("Variable Bonds", 4),
             ("Additional Bonds", 5), ("Harmonic Constraints", 6),
             ("Variable Bond Angles", 7), ("Additional Bond Angles", 8),
             ("Variable Dihedrals", 9), ("Additional Dihedrals", 10),
             ("Domain Definitions", 11), ("Final blank line", -2))


def _z_format(line: str) -> int:
    """ZmatrixScanner::checkFormat (ZmatrixScanner.cpp:175-219)."""
    s = _Stream(line)
    if (s.int() is not None and s.str() is not None and s.int() is not None
            and s.int() is not None and s.int() is not None and s.float() is not None
            and s.int() is not None and s.float() is not None and s.int() is not None
            and s.float() is not None and s.int() is not None):
        return 1
    for marker, fmt in _ZMARKERS:
        if marker in line:
            return fmt
    return -1


def _common_atom(bonds: list, a1: int, a2: int) -> int:
    """getCommonAtom (MathLibrary.cpp:150-178); -1 when there is none."""
    def opp(b, a):
        return b.atom2 if b.atom1 == a else (b.atom1 if b.atom2 == a else None)
    l1 = [o for o in (opp(b, a1) for b in bonds) if o is not None]
    l2 = [o for o in (opp(b, a2) for b in bonds) if o is not None]
    for c in l1:
        if c in l2:
            return c
    return -1


def _add_implied_angles(angles: list, bonds: list) -> None:
    """ZmatrixScanner::addImpliedAngles (ZmatrixScanner.cpp:513-573)."""
    for a in angles:
        a.common = _common_atom(bonds, a.atom1, a.atom2)
    add = []
    for i in range(len(angles)):
        for j in range(i + 1, len(angles)):
            p, q = angles[i], angles[j]
            if p.common != q.common:
                continue
            a1 = a2 = 0
            if p.atom1 == q.atom1:
                a1, a2 = p.atom2, q.atom2
            elif p.atom1 == q.atom2:
                a1, a2 = p.atom2, q.atom1
            elif p.atom2 == q.atom1:
                a1, a2 = p.atom1, q.atom2
            elif p.atom2 == q.atom2:
                a1, a2 = p.atom1, q.atom1
            if a1 != 0 and a2 != 0:
                na = Angle(a1, a2, 0.0, p.variable and q.variable, _common_atom(bonds, a1, a2))
                dup = any(na.common == c.common and ((c.atom1 == a1 and c.atom2 == a2)
                                                     or (c.atom1 == a2 and c.atom2 == a1))
                          for c in angles)
                if not dup:
                    add.append(na)
    angles.extend(add)


def read_zmatrix(path: str, opls: OplsTable, implied_angles: bool = False) -> list:
    """ZmatrixScanner::readInZmatrix: one molecule template per block ended
    by a ``TERZ`` or ``Geometry Variations`` line; the title line is
    skipped; dummy atoms (OPLS type -1) get sigma = epsilon = -1, charge 0
    and their z-matrix name.  The first data line after a ``Variable Bonds``
    / ``Variable Bond Angles`` / ``Variable Dihedrals`` header marks the
    first template's entries whose first atom lies in the listed range
    (handleZAdditions, ZmatrixScanner.cpp:221-286).  Returns the templates
    with z-matrix (1-based) atom ids.

    ``implied_angles`` is the starting value of the reference's
    ``hasAdditionalBondAngles`` flag, which its constructor leaves
    uninitialised: when set, the first template also gets the angles
    implied by two angles about one atom (addImpliedAngles).  The
    command-line program has been seen to start with it clear, a build
    that constructs the scanner elsewhere with it set; both are defined
    outcomes of the reference, so the caller chooses (default clear).
    The angle list only reaches the .state file."""
    if not path:
        raise FileFormatError("Error: readInZmatrix(): Given filename is NULL")
    if not os.path.isfile(path):
        raise FileFormatError("Error: Unable to open Z-Matrix file (" + path + ")")
    patterns: list = []
    atoms, bonds, angles, dihedrals = [], [], [], []
    new_mol = False
    extra_angles = bool(implied_angles)
    prev = 0
    mol_num = -1
    for n, line in enumerate(_lines(path), 1):
        if line and line[0] != "#" and n > 1:
            fmt = _z_format(line)
            if fmt == 1:
                tok = line.split()
                aid, atype, oa = tok[0], tok[1], tok[2]
                bw, bd, aw, am, dw, dm = tok[4], tok[5], tok[6], tok[7], tok[8], tok[9]
                if oa != "-1":
                    a = opls.atom(oa)
                    a.id = atoi(aid)
                    a.x = a.y = a.z = 0.0
                else:
                    a = Atom(atoi(aid), -1.0, -1.0, -1.0, -1.0, -1.0, 0.0, atype)
                atoms.append(a)
                if bw != "0":
                    bonds.append(Bond(a.id, atoi(bw), atof(bd), False))
                if aw != "0":
                    angles.append(Angle(a.id, atoi(aw), atof(am), False, 0))
                if dw != "0":
                    dihedrals.append(Dihedral(a.id, atoi(dw), atof(dm), False))
            elif fmt in (2, 3):
                new_mol = True
            if prev >= 3 and fmt == -1:
                extra_angles |= _z_additions(line, prev, patterns)
            prev = fmt
        if new_mol:
            mol_num += 1
            if extra_angles:
                _add_implied_angles(angles, bonds)
            patterns.append(Molecule(-1, mol_num, atoms, bonds, angles, dihedrals, []))
            atoms, bonds, angles, dihedrals = [], [], [], []
            new_mol = False
            extra_angles = False
    return patterns


def _z_additions(line: str, fmt: int, patterns: list) -> bool:
    """handleZAdditions: an atom range (``I4`` or ``I4-I4`` in the first 15
    columns) after a header.  Returns True for ``Additional Bond Angles``."""
    if "AUTO" in line:
        return False
    s = _Stream(line[:15])
    ids = []
    while True:
        v = s.int()
        if v is None:
            break
        ids.append(v)
        if s.peek() in ("-", ",", " "):
            s.i += 1
    if len(ids) == 1:
        lo = hi = ids[0]
    elif len(ids) == 2:
        lo, hi = ids
    else:
        lo, hi = 1, 0            # the reference's end = 0: nothing in range
    if fmt == 8:
        return True
    if fmt in (4, 7, 9):
        if not patterns:
            raise FileFormatError("z-matrix: a variable-geometry range precedes the first "
                                  "molecule")
        entries = {4: patterns[0].bonds, 7: patterns[0].angles, 9: patterns[0].dihedrals}[fmt]
        for e in entries:
            if lo <= e.atom1 <= hi:
                e.variable = True
    return False


def _hops(mol: Molecule) -> list:
    """ZmatrixScanner::calculateHops (:290-303, :322-387): atom pairs three or
    more bonds apart (breadth-first over the template's own bonds)."""
    size = len(mol.atoms)
    if size == 0:
        return []
    start = mol.atoms[0].id
    last = start + size - 1
    adj = [[] for _ in range(size)]
    graph = [[0] * size for _ in range(size)]
    for b in mol.bonds:
        if start <= b.atom1 <= last and start <= b.atom2 <= last:
            graph[b.atom1 - start][b.atom2 - start] = 1
            graph[b.atom2 - start][b.atom1 - start] = 1
    for r in range(size):
        adj[r] = [c for c in range(size) if graph[r][c] == 1]
    out = []
    for a1 in range(size):
        dist = {a1: 0}
        queue = [a1]
        qi = 0
        while qi < len(queue):
            t = queue[qi]
            qi += 1
            for c in adj[t]:
                if c not in dist:
                    dist[c] = dist[t] + 1
                    queue.append(c)
        for a2 in range(a1 + 1, size):
            d = dist.get(a2, -1)
            if d >= 3:
                out.append(Hop(a1 + start, a2 + start, d))
    return out


def _cross(a, b):
    """cross (MathLibrary.cpp:946-962): normalised a x b."""
    x = a[1] * b[2] - b[1] * a[2]
    y = b[0] * a[2] - a[0] * b[2]
    z = a[0] * b[1] - b[0] * a[1]
    ln = math.sqrt(max(1.0e-36, x * x + y * y + z * z))
    return [x / ln, y / ln, z / ln]


def _rad(deg: float) -> float:
    """degreesToRadians (MathLibrary.cpp:112-114) with the reference's pi."""
    return deg * REF_PI / 180.0


def build_xyz(mols: list) -> None:
    """buildMoleculeXYZ (MathLibrary.cpp:751-903): Cartesian coordinates of
    every template from its internal coordinates -- the first atom at the
    origin, the second on +x, the third in the xy plane, the rest from bond,
    angle and dihedral in the local frame of the three reference atoms.
    The bond/angle/dihedral of atom k is the first entry whose first atom is
    k among all templates' entries with first atom <= k.  As in the
    reference, a template of fewer than four atoms (or a missing second or
    third-atom entry) ends the build of the templates after it."""
    every_b = [b for m in mols for b in m.bonds]
    every_a = [a for m in mols for a in m.angles]
    every_d = [d for m in mols for d in m.dihedrals]

    def first(entries, aid):
        for e in entries:
            if e.atom1 <= aid and e.atom1 == aid:
                return e
        return None

    def opposite(e, aid):
        return e.atom2 if e.atom1 == aid else (e.atom1 if e.atom2 == aid else -1)

    before = 0
    for m in mols:
        at = m.atoms
        if len(at) < 2:
            break
        at[0].x = at[0].y = at[0].z = 0.0
        b = first(every_b, at[1].id)
        if b is None:
            break
        at[1].x, at[1].y, at[1].z = b.distance, 0.0, 0.0
        if len(at) < 3:
            break
        a = first(every_a, at[2].id)
        if a is None:
            break
        b = first(every_b, at[2].id)
        if b is None:
            raise FileFormatError("z-matrix: atom %d has an angle but no bond" % at[2].id)
        bonded = opposite(b, at[2].id) - before
        th = _rad(a.value)
        if bonded == 1:
            at[2].x = b.distance * math.cos(th)
        elif bonded == 2:
            at[2].x = at[1].x - b.distance * math.cos(th)
        at[2].y = b.distance * math.sin(th)
        at[2].z = 0.0
        if len(at) < 4:
            break
        for k in range(3, len(at)):
            aid = at[k].id
            b, a, d = first(every_b, aid), first(every_a, aid), first(every_d, aid)
            if b is None or a is None or d is None:
                raise FileFormatError("z-matrix: atom %d lacks a bond, angle or dihedral" % aid)
            th, ph = _rad(a.value), _rad(d.value)
            sv = math.sin(th)
            xbs = b.distance * sv * math.cos(ph)
            ybs = b.distance * sv * math.sin(ph)
            zbs = -b.distance * math.cos(th)
            bt = opposite(b, aid) - before
            aw = opposite(a, aid) - before
            dw = opposite(d, aid) - before
            for idx in (bt, aw, dw):
                if not 1 <= idx <= len(at):
                    raise FileFormatError("z-matrix: atom %d refers outside its molecule" % aid)
            ia = (at[dw - 1].x, at[dw - 1].y, at[dw - 1].z)
            ib = (at[aw - 1].x, at[aw - 1].y, at[aw - 1].z)
            ic = (at[bt - 1].x, at[bt - 1].y, at[bt - 1].z)
            vdih = [ia[i] - ic[i] for i in range(3)]
            vbnd = [ib[i] - ic[i] for i in range(3)]
            vy = _cross(vdih, vbnd)
            vx = _cross(vbnd, vy)
            vz = _cross(vx, vy)
            at[k].x = vx[0] * xbs + vy[0] * ybs + vz[0] * zbs + ic[0]
            at[k].y = vx[1] * xbs + vy[1] * ybs + vz[1] * zbs + ic[1]
            at[k].z = vx[2] * xbs + vy[2] * ybs + vz[2] * zbs + ic[2]
        before += len(at)


def build_templates(patterns: list, starting_id: int = 0) -> list:
    """ZmatrixScanner::buildMolecule (:389-511): copies of the templates with
    their hop lists and XYZ coordinates, atom ids renumbered from
    starting_id (0-based, consecutive over the templates)."""
    mols = [p.copy() for p in patterns]
    for m, p in zip(mols, patterns):
        m.hops = _hops(p)
    build_xyz(mols)
    for i, m in enumerate(mols):
        m.id = starting_id if i == 0 else mols[i - 1].id + len(mols[i - 1].atoms)
    for m in mols:
        for a in m.atoms:
            a.id = a.id - 1 + starting_id
        for e in m.bonds + m.angles + m.dihedrals + m.hops:
            e.atom1 = e.atom1 - 1 + starting_id
            e.atom2 = e.atom2 - 1 + starting_id
    return mols


# ---- the box (FileUtilities.cpp, Box.cpp) ----------------------------------------

@dataclass
class Box:
    """The reference's Box: its environment (as the box copied it) and its
    molecules (all that were allocated, possibly more than env.n_molecules).
    file_seed: the seed field of the .state file it was read from."""
    env: Environment
    molecules: list
    start_step: int = 0
    file_seed: int | None = None


def _angle_deg(p, q, r) -> float:
    """getAngle (MathLibrary.cpp:195-215), law of cosines, degrees."""
    def dist(a, b):
        return math.sqrt(math.pow(a.x - b.x, 2) + math.pow(a.y - b.y, 2) + math.pow(a.z - b.z, 2))
    d12, d23, d31 = dist(p, q), dist(q, r), dist(r, p)
    num = math.pow(d31, 2) - math.pow(d12, 2) - math.pow(d23, 2)
    den = -2 * d12 * d23
    deg = math.acos(num / den) * 180 / REF_PI
    return deg - 180 if deg > 180 else deg


def fcc_place(env: Environment, molecules: list) -> None:
    """generatefccBox (FileUtilities.cpp:550-642): four molecules per cubic
    cell of edge x/cells (the x edge sets every dimension), cells the
    smallest count with 4 cells^3 >= N, then every position shifted by
    -cell/2.  Molecule i copies the atoms of unit-cell molecule i mod 4
    (slot by slot over the contiguous atom array)."""
    n = env.n_molecules
    if len(molecules) < 4 or n < 4:
        raise FileFormatError("the FCC builder needs at least 4 molecules (the reference "
                              "indexes its four unit-cell molecules unchecked)")
    cells = float(int(math.pow(0.25 * float(n), 1.0 / 3.0) + 0.5))
    while 4 * cells * cells * cells < n:
        cells += 1
    cell = env.x / cells
    half = 0.5 * cell
    flat = [a for m in molecules for a in m.atoms]
    starts = np.cumsum([0] + [len(m.atoms) for m in molecules])
    X = np.array([a.x for a in flat])
    Y = np.array([a.y for a in flat])
    Z = np.array([a.z for a in flat])
    for k, (ox, oy, oz) in ((1, (half, half, 0.0)), (2, (0.0, half, half)), (3, (half, 0.0, half))):
        s, e = starts[k], starts[k + 1]
        X[s:e] += ox
        Y[s:e] += oy
        Z[s:e] += oz
    offset = 0
    nc = int(cells)
    for zc in range(1, nc + 1):
        for yc in range(1, nc + 1):
            for xc in range(1, nc + 1):
                for a in range(4):
                    i = a + offset
                    if i < n:
                        ln = starts[i + 1] - starts[i]
                        src = slice(starts[a], starts[a] + ln)
                        dst = slice(starts[i], starts[i] + ln)
                        if starts[a] + ln > len(flat):
                            raise FileFormatError("FCC copy reads past the last atom")
                        X[dst] = X[src] + cell * (xc - 1)
                        Y[dst] = Y[src] + cell * (yc - 1)
                        Z[dst] = Z[src] + cell * (zc - 1)
                offset += 4
    e = starts[n]
    X[:e] -= half
    Y[:e] -= half
    Z[:e] -= half
    for a, xv, yv, zv in zip(flat, X.tolist(), Y.tolist(), Z.tolist()):
        a.x, a.y, a.z = xv, yv, zv


def build_box(cfg_env: Environment, templates: list) -> Box:
    """buildBoxData (FileUtilities.cpp:285-547) after the box copied the
    environment: N rounded up to a multiple of the template count is
    allocated, copy m of template t is molecule m*T+t with ids and bonded
    entries shifted by m * (atoms per template set); then the FCC lattice
    and the implied angle values.  The box keeps the environment as it was
    before the rounding (N as configured, zero atoms), as the reference's
    does; cfg_env gets the rounded N and the atom count."""
    if not templates:
        raise FileFormatError("Error: buildBoxData(): Could not load molecule data.")
    box_env = cfg_env.copy()
    T = len(templates)
    if cfg_env.n_molecules % T:
        cfg_env.n_molecules += T - cfg_env.n_molecules % T
    if cfg_env.n_molecules < 1:
        raise FileFormatError("The simulation environment should have at least 1 molecule. "
                              "(The current count? %d)." % cfg_env.n_molecules)
    div = cfg_env.n_molecules // T
    per = sum(len(t.atoms) for t in templates)
    mols = [t.copy() for t in templates]
    bonds_so_far: list = []
    for m in mols:
        bonds_so_far.extend(m.bonds)
        for a in m.angles:
            if a.common != 0:
                a.common = _common_atom(bonds_so_far, a.atom1, a.atom2)
    first = mols
    out = list(first)
    for k in range(1, div):
        sh = k * per
        for t, base in enumerate(first):
            c = base.copy()
            c.id = k * T + t
            for a in c.atoms:
                a.id = a.id + sh
            for e in c.bonds + c.dihedrals + c.hops:
                e.atom1 += sh
                e.atom2 += sh
            for e in c.angles:
                e.atom1 += sh
                e.atom2 += sh
                e.common += sh
            out.append(c)
    # the reference renumbers atoms of copies m >= 1 to their array index
    flat = [a for m in out for a in m.atoms]
    for i in range(per, len(flat)):
        flat[i].id = i
    cfg_env.n_atoms = per * div
    fcc_place(box_env, out)
    for m in out:
        for a in m.angles:
            if a.value == 0:
                if not (0 <= a.atom1 < len(flat) and 0 <= a.atom2 < len(flat)
                        and 0 <= a.common < len(flat)):
                    raise FileFormatError("implied angle refers to a missing atom")
                a.value = _angle_deg(flat[a.atom1], flat[a.common], flat[a.atom2])
    return Box(box_env, out)


def keep_in_box(box: Box) -> None:
    """Box::keepMoleculeInBox for every molecule (Simulation.cpp:70-72,
    Box.cpp:84-109, 170-179): shift the whole molecule by one edge in each
    dimension where its first primary atom is below 0 or above the edge."""
    env = box.env
    for i in range(env.n_molecules):
        m = box.molecules[i]
        if m.type >= len(env.primary) or not env.primary[m.type]:
            raise FileFormatError("no primary atom for molecule type %d" % m.type)
        p = m.atoms[env.primary[m.type][0]]
        shifts = []
        for v, L in ((p.x, env.x), (p.y, env.y), (p.z, env.z)):
            shifts.append(L if v < 0 else (-L if v > L else 0.0))
        for a in m.atoms:
            if shifts[0]:
                a.x += shifts[0]
            if shifts[1]:
                a.y += shifts[1]
            if shifts[2]:
                a.z += shifts[2]


def box_rows(box: Box) -> BoxData:
    """SimBoxBuilder::build (SimBoxBuilder.cpp:10-42, 44-135, 282-299): the
    SimBox rows of the first env.n_molecules molecules -- coordinates and
    sigma/epsilon/charge per atom, start/length per molecule, and each
    molecule's primary atoms (its type's slots) as absolute indexes."""
    env = box.env
    n = env.n_molecules
    if n > len(box.molecules):
        raise FileFormatError("the environment counts %d molecules, the box holds %d"
                              % (n, len(box.molecules)))
    mols = box.molecules[:n]
    lens = np.array([len(m.atoms) for m in mols], dtype=np.int32)
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int32) if n else \
        np.zeros(0, np.int32)
    atoms = [a for m in mols for a in m.atoms]
    pidx, pstart, pcount = [], [], []
    for i, m in enumerate(mols):
        if m.type >= len(env.primary):
            raise FileFormatError("no primary atom definition for molecule type %d" % m.type)
        slots = env.primary[m.type]
        pstart.append(len(pidx))
        pcount.append(len(slots))
        for s in slots:
            if not 0 <= s < len(m.atoms):
                raise FileFormatError("primary atom %d outside molecule %d" % (s + 1, i))
            pidx.append(int(starts[i]) + s)
    f = lambda k: np.array([getattr(a, k) for a in atoms], dtype=np.float64)
    return BoxData(x=f("x"), y=f("y"), z=f("z"), sigma=f("sigma"), epsilon=f("epsilon"),
                   charge=f("charge"), mol_start=starts, mol_len=lens,
                   mol_pidx_start=np.array(pstart, np.int32),
                   mol_pidx_count=np.array(pcount, np.int32), pidx=np.array(pidx, np.int32),
                   size=np.array([env.x, env.y, env.z], np.float64), cutoff=float(env.cutoff),
                   temperature=float(env.temp), max_translate=float(env.max_translation),
                   max_rotate=float(env.max_rotation)).normalise()


def box_topology(box: Box, sb: SbTable) -> Topology:
    """SimBoxBuilder::addMolecules' bond, angle and exclusion rows
    (SimBoxBuilder.cpp:44-278) of the first env.n_molecules molecules.

    Atom ids resolve through the id -> index map the reference fills molecule
    by molecule, so an id must belong to this or an earlier molecule (the
    reference would read a null name otherwise; this raises).  An angle's
    middle atom is its ``common`` id as the loader leaves it: z-matrix angles
    carry 0 shifted by the copy's first atom (FileUtilities.cpp:508), so
    their middle row is the first atom of their copy set, not the angle's
    vertex -- the reference's rows, kept.  Force constants and equilibrium
    values come from the ``.sb`` table by atom name (-1 when missing).  The
    pair codes of each type come from its first molecule: excluded for the
    atoms of a bond and the ends of an angle, 0.5 for atoms exactly three
    bonds apart (the hop list), full otherwise; an exclusion wins over a
    fudge, as the reference scans its exclusion list first
    (SimulationStep.cpp:95-117).  The step counter starts at 0, for a
    resumed run too (SimBoxBuilder.cpp:37)."""
    env = box.env
    n = env.n_molecules
    if n > len(box.molecules):
        raise FileFormatError("the environment counts %d molecules, the box holds %d"
                              % (n, len(box.molecules)))
    mols = box.molecules[:n]
    n_types = max(len(env.primary), max((m.type + 1 for m in mols), default=0))
    id_idx: dict = {}
    id_name: dict = {}
    b_rows = {k: [] for k in ("a1", "a2", "k", "eq", "len", "var")}
    a_rows = {k: [] for k in ("a1", "a2", "mid", "k", "eq", "size", "var")}
    mb_start, mb_count, ma_start, ma_count, mtype = [], [], [], [], []
    first_of_type: dict = {}
    atom_idx = 0

    def idx(aid: int, what: str) -> int:
        if aid not in id_idx:
            raise FileFormatError("%s refers to atom id %d, not in this or an earlier molecule"
                                  % (what, aid))
        return id_idx[aid]

    for i, m in enumerate(mols):
        start = atom_idx
        for a in m.atoms:
            id_idx[a.id] = atom_idx
            id_name[a.id] = a.name
            atom_idx += 1
        mb_start.append(len(b_rows["a1"]))
        mb_count.append(len(m.bonds))
        ma_start.append(len(a_rows["a1"]))
        ma_count.append(len(m.angles))
        mtype.append(m.type)
        for b in m.bonds:
            i1, i2 = idx(b.atom1, "a bond"), idx(b.atom2, "a bond")
            n1, n2 = id_name[b.atom1], id_name[b.atom2]
            b_rows["a1"].append(i1)
            b_rows["a2"].append(i2)
            b_rows["k"].append(sb.k_bond(n1, n2))
            b_rows["eq"].append(sb.eq_bond(n1, n2))
            b_rows["len"].append(b.distance)
            b_rows["var"].append(1 if b.variable else 0)
        for a in m.angles:
            i1, i2 = idx(a.atom1, "an angle"), idx(a.atom2, "an angle")
            im = idx(a.common, "an angle's middle")
            n1, n2, nm = id_name[a.atom1], id_name[a.atom2], id_name[a.common]
            a_rows["a1"].append(i1)
            a_rows["a2"].append(i2)
            a_rows["mid"].append(im)
            a_rows["k"].append(sb.k_angle(n1, nm, n2))
            a_rows["eq"].append(sb.eq_angle(n1, nm, n2))
            a_rows["size"].append(a.value)
            a_rows["var"].append(1 if a.variable else 0)
        if m.type not in first_of_type:
            first_of_type[m.type] = (m, start)
    natom = np.zeros(n_types, np.int32)
    codes = []
    for t in range(n_types):
        if t not in first_of_type:
            continue
        m, start = first_of_type[t]
        na = len(m.atoms)
        natom[t] = na
        excl = [[] for _ in range(na)]
        fudge = [[] for _ in range(na)]

        def local(aid: int) -> int:
            return id_idx.get(aid, -1) - start if aid in id_idx else -1

        for e in list(m.bonds) + list(m.angles):
            l1, l2 = local(e.atom1), local(e.atom2)
            if 0 <= l1 < na and 0 <= l2 < na:
                excl[l1].append(l2)
                excl[l2].append(l1)
        for h in m.hops:
            l1, l2 = local(h.atom1), local(h.atom2)
            if 0 <= l1 < na and 0 <= l2 < na and h.hop == 3:
                fudge[l1].append(l2)
                fudge[l2].append(l1)
        c = np.full((na, na), PAIR_FULL, np.uint8)
        for r in range(na):
            for j in fudge[r]:
                c[r, j] = PAIR_FUDGE
            for j in excl[r]:
                c[r, j] = PAIR_EXCLUDED
        codes.append(c.ravel())
    i32 = lambda v: np.array(v, np.int32)
    f64 = lambda v: np.array(v, np.float64)
    return Topology(
        bond_a1=i32(b_rows["a1"]), bond_a2=i32(b_rows["a2"]), bond_k=f64(b_rows["k"]),
        bond_eq=f64(b_rows["eq"]), bond_len=f64(b_rows["len"]), bond_var=i32(b_rows["var"]),
        angle_a1=i32(a_rows["a1"]), angle_a2=i32(a_rows["a2"]), angle_mid=i32(a_rows["mid"]),
        angle_k=f64(a_rows["k"]), angle_eq=f64(a_rows["eq"]), angle_size=f64(a_rows["size"]),
        angle_var=i32(a_rows["var"]), mol_bond_start=i32(mb_start), mol_bond_count=i32(mb_count),
        mol_angle_start=i32(ma_start), mol_angle_count=i32(ma_count), mol_type=i32(mtype),
        type_natom=natom,
        pair_code=np.concatenate(codes).astype(np.uint8) if codes else np.zeros(0, np.uint8),
        max_bond_delta=float(env.max_bond_delta), max_angle_delta=float(env.max_angle_delta),
        max_intra_moves=15, step_num=0).normalise()


# ---- .state (StateScanner.cpp) ----------------------------------------------------

def _state_env(line: str) -> Environment:
    """StateScanner::getEnvironmentFromLine (:412-470).  The seed field is
    parsed into env.random_seed here; see read_state for the seed the
    reference actually continues with."""
    env = Environment()
    pos = 0
    idx = 0
    while True:
        while pos < len(line) and line[pos] == " ":
            pos += 1
        if pos >= len(line):
            break
        end = line.find(" ", pos)
        end = len(line) if end < 0 else end
        tok = line[pos:end]
        if idx == 0:
            env.x = atof(tok)
        elif idx == 1:
            env.y = atof(tok)
        elif idx == 2:
            env.z = atof(tok)
        elif idx == 3:
            env.n_molecules = atoi(tok)
        elif idx == 4:
            env.n_atoms = atoi(tok)
        elif idx == 5:
            env.temp = atof(tok)
        elif idx == 6:
            env.cutoff = atof(tok)
        elif idx == 7:
            env.max_translation = atof(tok)
        elif idx == 8:
            env.max_rotation = atof(tok)
        elif idx == 9:
            env.primary_line = tok
            env.primary_defs += parse_primary_definitions(tok, env.primary)
            env.random_seed = atoi(line[end + 1:]) if end + 1 <= len(line) else 0
            break
        idx += 1
        pos = end + 1
    return env


# The seed a run resumed from a .state file continues with.  The reference
# parses the seed field (StateScanner.cpp:461-463) and then calls strtok on,
# as token 10, the freed copy of the primary-definition string, assigning
# atoi() of whatever it finds there to the seed: its command-line program was
# seen to continue with 0 in one run and 1 in another (and writes that value
# into the .state files it saves), and glibc's srand gives 0 and 1 the same
# sequence -- the one of seed 1.
RESUMED_SEED = 1


def read_state(path: str, seed_from_file: bool = False) -> Box:
    """loadBoxData's state branch (FileUtilities.cpp:119-163) with
    StateScanner::readInEnvironment / readInStepNumber / readInMolecules:
    line 1 the environment, line 2 the step, then per molecule its id,
    ``= Type``, type, ``= Atoms`` (id x y z sigma epsilon charge name),
    ``= Bonds``, ``= Dihedrals``, ``= Hops``, ``= Angles`` sections and
    ``==``.  env.random_seed is RESUMED_SEED, as the reference continues
    (seed_from_file=True takes the file's field instead); the field itself
    is kept in Box.file_seed."""
    if not os.path.isfile(path):
        raise FileFormatError("Error: Unable to read environment from State File")
    lines = _lines(path)
    env = _state_env(lines[0] if lines else "")
    step = _Stream(lines[1]).int() if len(lines) > 1 else None
    step = -1 if step is None else step
    mols = []
    section = 0
    cur = Molecule(0, 0, [])
    for line in lines[3:]:
        head = line[:2]
        if section in (0, 1, 2, 3, 4, 5) and head == "= ":
            section += 1
            continue
        if section == 0:
            cur.id = atoi(line)
        elif section == 1:
            cur.type = atoi(line)
        elif section == 2:
            cur.atoms.append(_state_atom(line))
        elif section == 3:
            t = _strtok(line)
            cur.bonds.append(Bond(atoi(t[0]) if t else 0, atoi(t[1]) if len(t) > 1 else 0,
                                  atof(t[2]) if len(t) > 2 else 0.0,
                                  len(t) > 3 and atoi(t[3]) == 1))
        elif section == 4:
            t = _strtok(line)
            cur.dihedrals.append(Dihedral(atoi(t[0]) if t else 0, atoi(t[1]) if len(t) > 1 else 0,
                                          atof(t[2]) if len(t) > 2 else 0.0,
                                          len(t) > 3 and atoi(t[3]) == 1))
        elif section == 5:
            t = _strtok(line)
            cur.hops.append(Hop(atoi(t[0]) if t else 0, atoi(t[1]) if len(t) > 1 else 0,
                                atoi(t[2]) if len(t) > 2 else 0))
        elif section == 6:
            if head == "==":
                mols.append(cur)
                cur = Molecule(0, 0, [])
                section = 0
            else:
                t = _strtok(line)
                cur.angles.append(Angle(atoi(t[0]) if t else 0, atoi(t[1]) if len(t) > 1 else 0,
                                        atof(t[2]) if len(t) > 2 else 0.0,
                                        len(t) > 3 and atoi(t[3]) == 1, 0))
    if not mols:
        raise FileFormatError("Error: Unable to read molecule data from State file")
    if step < 0:
        raise FileFormatError("Error: State file does not have a starting step number")
    file_seed = env.random_seed
    if not seed_from_file:
        env.random_seed = RESUMED_SEED
    return Box(env, mols, start_step=step, file_seed=file_seed)


def _state_atom(line: str) -> Atom:
    """StateScanner::getAtomFromLine (:224-268)."""
    a = Atom(-1, -1.0, -1.0, -1.0, -1.0, -1.0, 0.0, "")
    t = _strtok(line)
    conv = [("id", atoi), ("x", atof), ("y", atof), ("z", atof), ("sigma", atof),
            ("epsilon", atof), ("charge", atof), ("name", str)]
    for (k, f), v in zip(conv, t):
        setattr(a, k, f(v))
    return a


def format_state(env: Environment, molecules: list, step: int, coords) -> str:
    """StateScanner::outputState (:545-597) as text: the environment line,
    the step, then every molecule with its atoms at the given coordinates
    (x, y, z arrays over the molecules' atoms in order)."""
    x, y, z = coords
    out = [" ".join([fmt_g(env.x), fmt_g(env.y), fmt_g(env.z), str(env.n_molecules),
                     str(env.n_atoms), fmt_g(env.temp), fmt_g(env.cutoff),
                     fmt_g(env.max_translation), fmt_g(env.max_rotation), env.primary_line,
                     str(env.random_seed), ""]) + "\n" + str(step) + "\n\n"]
    ai = 0
    natom = len(x)
    for m in molecules:
        out.append("%d\n= Type\n%d\n= Atoms\n" % (m.id, m.type))
        for a in m.atoms:
            if ai >= natom:
                raise FileFormatError("more atoms in the molecules than coordinates")
            out.append("%d %s %s %s %s %s %s %s \n" % (a.id, fmt_g(x[ai]), fmt_g(y[ai]),
                                                        fmt_g(z[ai]), fmt_g(a.sigma),
                                                        fmt_g(a.epsilon), fmt_g(a.charge),
                                                        a.name))
            ai += 1
        out.append("= Bonds\n")
        out.extend("%d %d %s %d\n" % (b.atom1, b.atom2, fmt_g(b.distance), 1 if b.variable else 0)
                   for b in m.bonds)
        out.append("= Dihedrals\n")
        out.extend("%d %d %s %d\n" % (d.atom1, d.atom2, fmt_g(d.value), 1 if d.variable else 0)
                   for d in m.dihedrals)
        out.append("= Hops\n")
        out.extend("%d %d %d\n" % (h.atom1, h.atom2, h.hop) for h in m.hops)
        out.append("= Angles\n")
        out.extend("%d %d %s %d\n" % (a.atom1, a.atom2, fmt_g(a.value), 1 if a.variable else 0)
                   for a in m.angles)
        out.append("==\n")
    return "".join(out)


def write_state(path: str, box: Box, step: int, coords) -> None:
    """Simulation::saveState's file: every molecule the box holds."""
    with open(path, "w", newline="\n") as f:
        f.write(format_state(box.env, box.molecules, step, coords))


def state_path(base: str, step: int, out_dir: str = "") -> str:
    """Simulation::saveState's file name: [dir/]base_step.state."""
    p = (out_dir + "/") if out_dir else ""
    return p + base + "_" + str(step) + ".state"


# ---- .pdb and .results (Simulation.cpp:296-417) -----------------------------------

def format_pdb(env: Environment, molecules: list, coords) -> str:
    """Simulation::writePDB: ATOM records (serial = atom id + 1, name right
    in 3 columns, residue UNK, residue number = molecule + 1, coordinates
    %12.3f %8.3f %8.3f), TER after each molecule, END."""
    x, y, z = coords
    out = ["REMARK Created by MCGPU\n"]
    ai = 0
    for i in range(env.n_molecules):
        for a in molecules[i].atoms:
            out.append("%-6s%5d%3s%6s%6d%12.3f%8.3f%8.3f\n"
                       % ("ATOM", a.id + 1, a.name, "UNK", i + 1, x[ai], y[ai], z[ai]))
            ai += 1
        out.append("TER\n")
    out.append("END\n")
    return "".join(out)


def write_pdb(path: str, box: Box, coords) -> None:
    with open(path, "w", newline="\n") as f:
        f.write(format_pdb(box.env, box.molecules, coords))


def pdb_path(sim_name: str, out_dir: str = "") -> str:
    p = (out_dir + "/") if out_dir else ""
    return p + (sim_name or "run") + ".pdb"


def format_results(*, sim_name: str, mode: str, start_step: int, steps: int, n_molecules: int,
                   energy: float, run_time: float, accepted: int, rejected: int,
                   lj: float = 0.0, charge: float = 0.0) -> str:
    """The ``.results`` file of Simulation::run (Simulation.cpp:316-350)."""
    total = np.float32(accepted + rejected)
    rate = float(np.float32(100.0) * np.float32(accepted) / total) if total else 0.0
    lines = ["######### MCGPU Results File #############", "[Information]",
             "Timestamp = " + time.strftime("%Y-%m-%d %X")]
    if sim_name:
        lines.append("Simulation-Name = " + sim_name)
    lines += ["Simulation-Mode = " + mode, "Starting-Step = %d" % start_step,
              "Steps = %d" % steps, "Molecule-Count = %d" % n_molecules, "", "[Results]",
              "LJ-Energy Subtotal: " + fmt_g(lj), "Charge Energy Subtotal: " + fmt_g(charge),
              "Final-Energy = " + fmt_g(energy), "Run-Time = " + fmt_g(run_time) + " seconds",
              "Accepted-Moves = %d" % accepted, "Rejected-Moves = %d" % rejected,
              "Acceptance-Rate = " + fmt_g(rate) + "%"]
    return "\n".join(lines) + "\n"


# ---- long-range correction (SerialCalcs.cpp:37-107) -------------------------------

def energy_lrc(env: Environment, molecules: list, volume: float | None = None) -> float:
    """SerialCalcs::calcEnergy_LRC: the tail correction of the LJ energy for
    two solvents (molecules 0 and 1 stand for them, N/2 of each by integer
    division), with A6 = sqrt(4 eps sigma^6), A12 = sqrt(4 eps sigma^12)
    per atom (dummies count zero) and

        E = sum_ij 2 pi N1^2/(3V) (A12_i A12_j rc^-9/3 - A6_i A6_j rc^-3)
                 + 2 pi N2^2/(3V) (B..)  + 4 pi N1 N2/(3V) (A_i B_j ..)

    It scales as 1/V at fixed N; ``volume`` evaluates it at another volume
    (the reference evaluates it once, at the starting box).  Raises
    FileFormatError when molecules 0 and 1 differ in atom count (the
    reference then reads past its arrays)."""
    if len(molecules) < 2:
        raise FileFormatError("the long-range correction reads molecules 0 and 1")
    V = env.x * env.y * env.z if volume is None else volume
    rc3 = 1.00 / math.pow(env.cutoff, 3)
    rc9 = math.pow(rc3, 3)
    n1 = float(env.n_molecules // 2)
    n2 = float(env.n_molecules // 2)

    def coeffs(m):
        a6, a12 = [], []
        for a in m.atoms:
            s, e = (0.0, 0.0) if (a.sigma < 0 or a.epsilon < 0) else (a.sigma, a.epsilon)
            s2 = math.pow(s, 2)
            s6 = math.pow(s2, 3)
            s12 = math.pow(s6, 2)
            a6.append(math.sqrt(4 * e * s6))
            a12.append(math.sqrt(4 * e * s12))
        return a6, a12

    A6, A12 = coeffs(molecules[0])
    B6, B12 = coeffs(molecules[1])
    if len(A6) != len(B6):
        # the reference's loops index A12[j] and B12[i] with i over molecule
        # 0's atoms and j over molecule 1's: past the end of one of its
        # per-atom arrays unless the two have the same atom count
        raise FileFormatError("the long-range correction is defined for molecules 0 and 1 of "
                              "equal atom counts (%d and %d here)" % (len(A6), len(B6)))
    ecut = 0.0
    for i in range(len(A6)):
        for j in range(len(B6)):
            ecut += (2 * REF_PI * n1 * n1 / (3.0 * V)) * (A12[i] * A12[j] * rc9 / 3.0
                                                          - A6[i] * A6[j] * rc3)
            ecut += (2 * REF_PI * n2 * n2 / (3.0 * V)) * (B12[i] * B12[j] * rc9 / 3.0
                                                          - B6[i] * B6[j] * rc3)
            ecut += (4 * REF_PI * n1 * n2 / (3.0 * V)) * (A12[i] * B12[j] * rc9 / 3.0
                                                          - A6[i] * B6[j] * rc3)
    return ecut


# ---- loading (FileUtilities.cpp:19-168) -------------------------------------------

def extension(path: str) -> str:
    """getExtension (Parsing.cpp:6-14)."""
    dot = path.rfind(".")
    delim = max(path.rfind("/"), path.rfind("\\"))
    if delim < 0 or delim < dot:
        return path[dot + 1:] if dot >= 0 else path
    return ""


@dataclass
class SimInput:
    """What Simulation's constructor and run() start from.  ``topology``:
    the bond, angle and exclusion rows (flexible-molecule terms); a
    ``.state`` start has no ``.sb`` table behind it (the reference reads the
    table for configurations only), so its force constants are -1."""
    box: Box
    rows: BoxData
    steps: int
    start_step: int
    config: Config | None = None
    topology: Topology | None = None


def load(path: str, implied_angles: bool = False, seed_from_file: bool = False,
         env: dict | None = None) -> SimInput:
    """loadBoxData: a ``.config`` builds the box from its z-matrix and OPLS
    table on the FCC lattice; a ``.state`` restores the box it holds.  Then
    Simulation::run's keepMoleculeInBox and the SimBox rows.  ``env``
    overrides settings of a ``.config`` (Environment field names, e.g.
    ``{"n_molecules": 512, "x": 41.8}``) before the box is built."""
    ext = extension(path)
    if ext == "config":
        cfg = read_config(path)
        for k, v in (env or {}).items():
            if not hasattr(cfg.env, k):
                raise FileFormatError("no environment setting " + k)
            setattr(cfg.env, k, v)
        par = cfg.opls_path
        cut = par.rfind("/")
        sb_dir = par[:cut] if cut >= 0 else par
        if not os.path.isfile(sb_dir + "/oplsaa.sb"):
            raise FileFormatError("Error: readInOpls(): could not open file (" + sb_dir
                                  + "/oplsaa.sb)")
        opls = read_opls(par)
        templates = build_templates(read_zmatrix(cfg.zmatrix_path, opls, implied_angles), 0)
        if len(templates) != cfg.env.primary_defs:
            raise FileFormatError(
                "Error: loadBoxData(): The number of molecules read from the Z Matrix file (%d)"
                " does not equal the number of primary index definitions in the config file "
                "(%d)" % (len(templates), cfg.env.primary_defs))
        sb = read_sb(sb_dir + "/oplsaa.sb")
        box = build_box(cfg.env, templates)
        keep_in_box(box)
        return SimInput(box, box_rows(box), cfg.steps, 0, cfg, box_topology(box, sb))
    if ext == "state":
        box = read_state(path, seed_from_file)
        keep_in_box(box)
        return SimInput(box, box_rows(box), DEFAULT_STEP_COUNT, box.start_step, None,
                        box_topology(box, SbTable()))
    raise FileFormatError("Must specify a config or state file")
