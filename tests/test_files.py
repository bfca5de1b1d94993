"""The reference's input and output files (mcgpu_gb300.files) against the
reference itself: the SimBox rows its loader builds from a .config (z-matrix
+ OPLS table on the FCC lattice) or a .state, its long-range correction, and
the .state / .pdb text its program and StateScanner write.  The reference
outputs are committed fixtures (tests/golden/make_file_fixtures.py ran the
compiled reference on the synthetic inputs beside them); where the compiled
reference is present, the loader is also compared live."""
import contextlib
import os
from pathlib import Path

import numpy as np
import pytest

from mcgpu_gb300 import files as F
from mcgpu_gb300 import metrosim as M

FILES = Path(__file__).resolve().parent / "golden" / "files"
REF = FILES / "ref"
CONFIGS = ["wat", "mix", "mixp", "mixv", "trip", "tri3"]
ROWS = ("x", "y", "z", "sigma", "epsilon", "charge", "mol_start", "mol_len", "mol_pidx_start",
        "mol_pidx_count", "pidx", "size")


@contextlib.contextmanager
def cwd(path):
    old = os.getcwd()
    os.chdir(path)
    try:
        yield
    finally:
        os.chdir(old)


def load(name, **kw):
    with cwd(FILES):
        return F.load(name, **kw)


def assert_rows(si, ref):
    r = si.rows
    for k in ROWS:
        a, b = getattr(r, k), ref[k]
        assert a.shape == b.shape and np.array_equal(a, b), k
    n = r.n_mol
    assert [m.type for m in si.box.molecules[:n]] == list(ref["mol_type"])
    p = ref["params"]
    assert (r.cutoff, r.temperature, r.max_translate, r.max_rotate) == (p[0], p[1], p[3], p[4])
    assert r.temperature * F.K_BOLTZ == p[2]


@pytest.mark.parametrize("name", CONFIGS)
def test_config_rows_match_reference_loader(name):
    """Rows bit-identical to the reference's loadBoxData + keepMoleculeInBox +
    SimBoxBuilder: two templates, a bracketed two-primary definition, three
    templates with N rounded up and the FCC copy crossing molecules, and a
    three-atom first template that stops the XYZ build of the next."""
    si = load(name + ".config")
    ref = np.load(REF / (name + "_rows.npz"))
    assert_rows(si, ref)
    assert si.box.env.random_seed == int(ref["seed"])


def test_tri3_second_template_not_built():
    """The reference's XYZ builder breaks out of its template loop at a
    template of fewer than four atoms: the amine keeps its initial
    coordinates (0 for real atoms) plus the lattice offsets."""
    si = load("tri3.config")
    tpl = si.box.molecules[1]
    assert len(tpl.atoms) == 4
    rel = np.array([[a.x - tpl.atoms[0].x, a.y - tpl.atoms[0].y, a.z - tpl.atoms[0].z]
                    for a in tpl.atoms])
    assert np.all(rel == 0.0)


def test_state_rows_match_reference_loader():
    si = load("ref/wat_300.state")
    ref = np.load(REF / "wat300_rows.npz")
    assert_rows(si, ref)
    assert si.start_step == int(ref["start_step"]) == 300
    assert si.steps == F.DEFAULT_STEP_COUNT
    assert si.box.file_seed == 12345 and si.box.env.random_seed == F.RESUMED_SEED


def test_lrc_matches_reference():
    si = load("wat.config")
    ref = np.load(REF / "wat_rows.npz")
    assert F.energy_lrc(si.box.env, si.box.molecules) == float(ref["lrc"])
    run = np.load(REF / "wat_run.npz")
    assert "%.3f" % F.energy_lrc(si.box.env, si.box.molecules) == "%.3f" % run["lrc_printed"]
    # 1/V scaling at fixed N
    V = si.box.env.x * si.box.env.y * si.box.env.z
    e2 = F.energy_lrc(si.box.env, si.box.molecules, volume=2 * V)
    assert abs(e2 * 2 - float(ref["lrc"])) <= 1e-15 * abs(e2)


def test_lrc_unequal_templates_raises():
    si = load("mix.config")
    with pytest.raises(F.FileFormatError):
        F.energy_lrc(si.box.env, si.box.molecules)


def same_state(a: str, b: str, resumed: bool) -> bool:
    if not resumed:
        return a == b
    la, lb = a.split("\n", 1), b.split("\n", 1)
    return la[1] == lb[1] and la[0].split()[:-1] == lb[0].split()[:-1]


@pytest.mark.parametrize("name,inp,step", [("wat", "wat.config", 300),
                                           ("watres", "ref/wat_300.state", 400),
                                           ("mix", "mix.config", 200),
                                           ("mixp", "mixp.config", 200)])
def test_state_writer_reproduces_reference(name, inp, step):
    """format_state of the reference's own final coordinates is the text the
    reference wrote (the program for wat/watres, StateScanner through the
    harness for the mixtures; after a resume the seed field is the
    reference's indeterminate 0 or 1)."""
    run = np.load(REF / (name + "_run.npz"))
    implied = bool(run["implied_angles"]) if "implied_angles" in run.files else False
    si = load(inp, implied_angles=implied)
    xyz = run["xyz"]
    text = F.format_state(si.box.env, si.box.molecules, step, (xyz[:, 0], xyz[:, 1], xyz[:, 2]))
    ref = (REF / ("%s_%d.state" % (name, step))).read_text()
    assert same_state(text, ref, resumed=inp.endswith(".state"))


@pytest.mark.parametrize("name,inp", [("wat", "wat.config"), ("watres", "ref/wat_300.state")])
def test_pdb_writer_reproduces_reference(name, inp):
    run = np.load(REF / (name + "_run.npz"))
    si = load(inp)
    xyz = run["xyz"]
    assert F.format_pdb(si.box.env, si.box.molecules, (xyz[:, 0], xyz[:, 1], xyz[:, 2])) == \
        (REF / (name + ".pdb")).read_text()


def test_state_read_write_roundtrip():
    """A reference-written .state read and written back is the same text
    (six significant digits survive the round trip through double)."""
    si = load("ref/wat_300.state", seed_from_file=True)
    r = si.rows
    box = F.read_state(str(REF / "wat_300.state"), seed_from_file=True)
    x = np.array([a.x for m in box.molecules for a in m.atoms])
    y = np.array([a.y for m in box.molecules for a in m.atoms])
    z = np.array([a.z for m in box.molecules for a in m.atoms])
    assert F.format_state(box.env, box.molecules, 300, (x, y, z)) == \
        (REF / "wat_300.state").read_text()
    assert r.n_atom == len(x)


def test_variable_geometry_markers():
    """handleZAdditions: the first data line after a Variable Bonds / Bond
    Angles header marks the FIRST template's entries whose first atom is in
    the range (here water bonds of atoms 2-3 and the angle of atom 3)."""
    si = load("mixv.config")
    wat = si.box.molecules[0]
    assert [b.variable for b in wat.bonds] == [True, True, False]
    assert [a.variable for a in wat.angles] == [True, False]
    amine = si.box.molecules[1]
    assert not any(b.variable for b in amine.bonds)
    text = F.format_state(si.box.env, si.box.molecules[:2], 0,
                          (si.rows.x, si.rows.y, si.rows.z))
    assert "\n1 0 0.9572 1\n2 0 0.9572 1\n3 0 1 0\n" in text


def test_primary_definitions():
    lists = []
    assert F.parse_primary_definitions("1,[1,2],3", lists) == 3
    assert lists[:3] == [[0], [0, 1], [2]] and all(v == [] for v in lists[3:])
    lists = []
    assert F.parse_primary_definitions("5", lists) == 1 and lists == [[4]]
    with pytest.raises(F.FileFormatError):
        F.parse_primary_definitions("[1,2", [])


def test_c_scalar_parsing():
    assert F.atof("  .957200abc") == 0.9572 and F.atof("x") == 0.0 and F.atof("-1e2") == -100.0
    assert F.atoi(" 12.7") == 12 and F.atoi("") == 0 and F.atoi("-3x") == -3
    s = F._Stream("12.5 ab")
    assert s.int() == 12 and s.float() == 0.5 and s.str() == "ab" and s.int() is None


def write(tmp_path, text, name="t.config"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


@pytest.mark.parametrize("text,msg", [
    ("x=1\ny 2\n", "not well formed"),
    ("x = 1\n", "Unexpected key encountered: x "),
    ("[section]\nx=1\n", "not well formed"),
    ("foo=1\n", "Unexpected key"),
    ("x=\n", "Missing environment X value"),
    ("cutoff=\n", "cutoff"),
    ("z-matrix=\nstate-input=\n", "Cannot safely continue"),
])
def test_config_errors(tmp_path, text, msg):
    with pytest.raises(F.FileFormatError, match=msg):
        F.read_config(write(tmp_path, text))


def test_config_values(tmp_path):
    cfg = F.read_config(write(tmp_path, "# c\n; c\n\n  x=10.5  \ny=11\nz=12\ntemp=300\n"
                                        "steps=7\nmolecules=8\nprimary-atom=1\n"
                                        "ensemble=npt\npressure=2e-5\nvolume-interval=50\n"
                                        "random-seed=\nstrategy=verlet\n"))
    e = cfg.env
    assert (e.x, e.y, e.z, e.temp, cfg.steps, e.n_molecules) == (10.5, 11.0, 12.0, 300.0, 7, 8)
    assert (cfg.ensemble, e.pressure, cfg.volume_interval, cfg.strategy) == \
        ("npt", 2e-5, 50, "verlet")
    assert e.random_seed != 0 and e.primary == [[0]]
    with pytest.raises(F.FileFormatError, match="Unable to open"):
        F.read_config(str(tmp_path / "missing.config"))


def test_missing_sb_file(tmp_path):
    for f in ("synth.par", "wat4.z", "wat.config"):
        (tmp_path / f).write_bytes((FILES / f).read_bytes())
    with cwd(tmp_path):
        with pytest.raises(F.FileFormatError, match="oplsaa.sb"):
            F.load("wat.config")


def test_fcc_needs_four_molecules(tmp_path):
    for f in ("synth.par", "oplsaa.sb", "wat4.z"):
        (tmp_path / f).write_bytes((FILES / f).read_bytes())
    (tmp_path / "w.config").write_text((FILES / "wat.config").read_text()
                                       .replace("molecules=108", "molecules=3"))
    with cwd(tmp_path):
        with pytest.raises(F.FileFormatError, match="FCC"):
            F.load("w.config")


def test_extension():
    assert F.extension("a/b.config") == "config" and F.extension("x.state") == "state"
    assert F.extension("dir.v1/file") == ""


def test_metrosim_cli():
    a = M.parse_args(["w.config", "-n", "10", "-I", "5", "-S", "verlet-list", "--form", "chain"])
    assert (a.steps, a.state_interval, a.strategy, a.form) == (10, 5, "verlet-list", "chain")
    assert M.parse_args(["w.config", "-l"]).neighbor == M.DEFAULT_NEIGHBORLIST_INTERVAL
    for bad, msg in ((["w.txt"], "config or state"), (["w.config", "-S", "x"], "strategy"),
                     (["w.config", "-s", "-p"], "both GPU and CPU"),
                     (["w.config", "-n", "0"], "greater than zero"), ([], "not specified")):
        with pytest.raises(F.FileFormatError, match=msg):
            M.parse_args(bad)


def test_metrosim_needs_the_gpu(tmp_path):
    """Without a GPU the driver fails at the CUDA library (no CPU path)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from mcgpu_gb300 import MCGPUError
    for f in ("synth.par", "oplsaa.sb", "wat4.z", "wat.config"):
        (tmp_path / f).write_bytes((FILES / f).read_bytes())
    with cwd(tmp_path):
        with pytest.raises((MCGPUError, OSError)):
            M.run(["wat.config", "-n", "5"], out=None)


def test_reference_loader_live(tmp_path):
    """Where the compiled reference is present, its loader is run directly
    (on a copy of the inputs: it writes a log file where it runs)."""
    import shutil
    from oracle.pyoracle import REF_SO, RefHarness
    if not REF_SO.exists():
        pytest.skip("compiled reference not present")
    for f in FILES.iterdir():
        if f.is_file():
            shutil.copy(f, tmp_path / f.name)
    R = RefHarness()
    for name in CONFIGS:
        ref = R.load_files(str(tmp_path / (name + ".config")))
        assert_rows(load(name + ".config"), ref)


@pytest.mark.parametrize("name", ["demo", "indole267", "meoh500"])
def test_reference_example_configs_live(tmp_path, name):
    """The reference's own example configurations (its z-matrices and OPLS
    table), where its sources and compiled loader are present: rows and LRC
    bit-identical."""
    import shutil
    from oracle.pyoracle import REF_SO, REFERENCE_SRC, RefHarness
    res = REFERENCE_SRC / "resources"
    if not REF_SO.exists() or not res.is_dir():
        pytest.skip("reference sources or compiled reference not present")
    shutil.copytree(res, tmp_path / "resources")
    src = res / (name + ".config")
    if not src.exists():
        src = res / "exampleFiles" / (name + ".config")
    shutil.copy(src, tmp_path / (name + ".config"))
    ref = RefHarness().load_files(str(tmp_path / (name + ".config")))
    with cwd(tmp_path):
        si = F.load(name + ".config")
    assert_rows(si, ref)
    assert F.energy_lrc(si.box.env, si.box.molecules) == ref["lrc"]
