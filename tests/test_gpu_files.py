"""The host driver (mcgpu_gb300.metrosim) on the GPU against the reference
program's own outputs, and bit-exact checkpoint/resume of device-resident
chains.

* plain form, FP64: the .state and .pdb files, final energy (with the
  long-range correction) and move counts equal the reference program's for
  a run from a .config and for a run resumed from the .state it wrote;
  mixtures (two templates, a two-primary molecule) reproduce the reference's
  coordinates and pair energy.
* chain form: a run interrupted by a checkpoint and resumed continues bit
  for bit (coordinates, energy, counters), with Verlet lists and NPT.
"""
import contextlib
import io
import os
import shutil
from pathlib import Path

import numpy as np
import pytest

from mcgpu_gb300 import ROT_AXIS, ChainBatch, Context, MCGPUError
from mcgpu_gb300 import files as F
from mcgpu_gb300 import metrosim as M
from mcgpu_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FILES = Path(__file__).resolve().parent / "golden" / "files"
REF = FILES / "ref"
INPUTS = ["synth.par", "oplsaa.sb", "wat4.z", "mix.z", "wat.config", "mix.config",
          "mixp.config", "flex.z", "flex.config"]


@contextlib.contextmanager
def workdir(tmp_path):
    for f in INPUTS:
        shutil.copy(FILES / f, tmp_path / f)
    old = os.getcwd()
    os.chdir(tmp_path)
    try:
        yield tmp_path
    finally:
        os.chdir(old)


def same_state(a: str, b: str, resumed: bool) -> bool:
    if not resumed:
        return a == b
    la, lb = a.split("\n", 1), b.split("\n", 1)
    return la[1] == lb[1] and la[0].split()[:-1] == lb[0].split()[:-1]


def atoms_of(text: str) -> np.ndarray:
    """x, y, z of every atom line of a .state text."""
    rows, sec = [], None
    for ln in text.split("\n")[3:]:
        if ln.startswith("= "):
            sec = ln
            continue
        if sec == "= Atoms" and ln and not ln.startswith("=="):
            t = ln.split()
            if len(t) >= 8:
                rows.append([float(t[1]), float(t[2]), float(t[3])])
        if ln.startswith("=="):
            sec = None
    return np.array(rows)


def test_plain_run_reproduces_reference_program(tmp_path):
    with workdir(tmp_path):
        out = io.StringIO()
        res = M.run(["wat.config", "-n", "300"], out=out)
        run = np.load(REF / "wat_run.npz")
        assert res.accepted == int(run["accepted"]) and res.rejected == 300 - res.accepted
        assert "Final Energy: %.3f" % float(run["final"]) in out.getvalue()
        assert "Energy Long-range Correction: %.3f" % float(run["lrc_printed"]) in out.getvalue()
        assert Path("wat_300.state").read_text() == (REF / "wat_300.state").read_text()
        assert Path("wat.pdb").read_text() == (REF / "wat.pdb").read_text()
        assert abs(res.energy - (float(run["e"]) + res.lrc)) <= 1e-9 * abs(res.energy)
        assert Path("wat.results").exists()


def test_plain_resume_reproduces_reference_program(tmp_path):
    with workdir(tmp_path):
        shutil.copy(REF / "wat_300.state", "wat_300.state")
        out = io.StringIO()
        res = M.run(["wat_300.state", "-n", "100", "--name", "watres"], out=out)
        run = np.load(REF / "watres_run.npz")
        assert res.start_step == 300 and res.accepted == int(run["accepted"])
        assert "Final Energy: %.3f" % float(run["final"]) in out.getvalue()
        assert same_state(Path("watres_400.state").read_text(),
                          (REF / "watres_400.state").read_text(), resumed=True)
        assert Path("watres.pdb").read_text() == (REF / "watres.pdb").read_text()


@pytest.mark.parametrize("name", ["mix", "mixp"])
def test_plain_mixture_reproduces_reference(tmp_path, name):
    """Two templates (water, methylamine), for mixp with two primary atoms
    on the amine; the reference's LRC is undefined for them (none added)."""
    with workdir(tmp_path):
        res = M.run([name + ".config", "-n", "200"], out=None)
        run = np.load(REF / (name + "_run.npz"))
        assert res.lrc == 0.0 and res.accepted == int(run["accepted"])
        assert abs(res.energy - float(run["e"])) <= 1e-9 * max(1.0, abs(float(run["e"])))
        ours = atoms_of(Path("%s_200.state" % name).read_text())
        ref = atoms_of((REF / ("%s_200.state" % name)).read_text())
        assert ours.shape == ref.shape and np.array_equal(ours, ref)


@pytest.mark.parametrize("form", ["plain", "device"])
def test_intra_run_reproduces_reference(tmp_path, form):
    """flex.config with the reference's intramolecular moves on (--intra,
    implied angles as the golden vectors were made): the reference's
    accepted count and final energy after the config's 2500 steps (its
    random-seed 4321), through the host loop and the device loop."""
    from helpers import load_intra_golden
    _, _, z = load_intra_golden()
    with workdir(tmp_path):
        res = M.run(["flex.config", "--intra", "--implied-angles", "--form", form], out=None)
    assert res.steps == int(z["traj_steps"][0]) and res.lrc == 0.0
    assert res.accepted == int(z["traj_accepted"][0])
    assert abs(res.energy - z["traj_energy"][0]) <= 1e-8 * max(1.0, abs(z["traj_e0"][0]))


def test_plain_state_interval(tmp_path):
    with workdir(tmp_path):
        res = M.run(["wat.config", "-n", "300", "-I", "100", "--name", "w"], out=None)
        for s in (100, 200, 300):
            assert Path("w_%d.state" % s).exists()
        assert "w_100.state" in " ".join(res.files)
        # the 300-step file equals the program's apart from the name
        assert Path("w_300.state").read_text() == (REF / "wat_300.state").read_text()


def test_chain_form_checkpoint_resume_exact(tmp_path):
    """--form chain, interrupted at step 600 and resumed from the .ckpt
    written there: the 1200-step files equal an uninterrupted run's."""
    with workdir(tmp_path):
        a = M.run(["wat.config", "--form", "chain", "-n", "1200", "--checkpoint-interval",
                   "600", "--name", "a"], out=None)
        assert Path("a_600.ckpt").exists() and Path("a_1200.ckpt").exists()
        b = M.run(["wat.config", "--form", "chain", "-n", "600", "--resume", "a_600.ckpt",
                   "--name", "b"], out=None)
        assert b.start_step == 600
        assert Path("b_1200.state").read_text().split("\n", 1)[1] == \
            Path("a_1200.state").read_text().split("\n", 1)[1]
        assert b.energy == a.energy
        assert a.accepted + a.rejected == 1200 and b.accepted + b.rejected == 600


def test_chain_form_npt_verlet(tmp_path):
    with workdir(tmp_path):
        cfg = Path("wat.config").read_text() + "ensemble=npt\npressure=1.4583972574259083e-05\n"
        Path("npt.config").write_text(cfg.replace("volume-interval=0", "volume-interval=50"))
        res = M.run(["npt.config", "--form", "chain", "-S", "verlet", "-n", "1000",
                     "--max-dlnv", "0.02", "--name", "n"], out=None)
        assert res.accepted > 0 and res.box[0] != 14.8
        st = F.read_state("n_1000.state", seed_from_file=True)
        assert st.env.x == float(F.fmt_g(res.box[0]))


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def _stats(bt):
    return [(s.energy, s.steps, s.accepted, s.ties, tuple(s.box), s.vol_accepted)
            for s in bt.stats()]


@pytest.mark.parametrize("verlet,npt", [(False, False), (True, False), (True, True)])
def test_batch_checkpoint_restore_bit_exact(ctx, verlet, npt):
    boxes, seeds = W.water_chains(6, n_min=100, n_max=900, seed=31)

    def make():
        bt = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
        bt.set_tile(128, 1, 16)
        if verlet:
            bt.set_verlet(1.2)
        if npt:
            bt.set_npt(40, 1.0, 0.02)
        return bt

    a = make()
    a.run(320)
    blob = a.checkpoint()
    a.run(240)
    b = make()
    b.run(16)                          # any state: the restore replaces it
    b.restore(blob)
    b.run(240)
    assert _stats(a) == _stats(b)
    for c in range(len(boxes)):
        xa, ya, za = a.download(c)
        xb, yb, zb = b.download(c)
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb) and np.array_equal(za, zb)
    a.close()
    b.close()


def test_batch_restore_rejects_other_layout(ctx):
    boxes, seeds = W.water_chains(3, n_min=100, n_max=300, seed=5)
    a = ChainBatch(ctx, boxes, seeds)
    blob = a.checkpoint()
    other = ChainBatch(ctx, boxes[:2], seeds[:2])
    with pytest.raises(MCGPUError):
        other.restore(blob)
    same = ChainBatch(ctx, boxes, seeds)
    same.set_verlet(1.0)
    with pytest.raises(MCGPUError):
        same.restore(blob)              # Verlet setting differs
    bad = bytearray(blob)
    bad[-1] ^= 0xFF
    with pytest.raises(MCGPUError):
        a.restore(bytes(bad))           # checksum
    for bt in (a, other, same):
        bt.close()


def test_batch_download_all_equals_per_chain(ctx):
    boxes, seeds = W.water_chains(5, n_min=64, n_max=300, seed=8)
    bt = ChainBatch(ctx, boxes, seeds)
    bt.run(64)
    allc = bt.download_all()
    for c in range(len(boxes)):
        x, y, z = bt.download(c)
        ax, ay, az = allc[c]
        assert np.array_equal(x, ax) and np.array_equal(y, ay) and np.array_equal(z, az)
    bt.close()


def test_batch_create_reports_lowest_failing_chain(ctx):
    """The pool is filled on several host threads; the error is still the
    one a chain-by-chain build meets first."""
    boxes, seeds = W.water_chains(40, n_min=600, n_max=1200, seed=12)
    boxes[17].x = boxes[17].x.copy()
    boxes[17].x[5] = np.nan
    boxes[31].mol_len = boxes[31].mol_len.copy()
    boxes[31].mol_len[0] = 0
    with pytest.raises(MCGPUError, match="chain 17: non-finite coordinate at atom 5"):
        ChainBatch(ctx, boxes, seeds)
    boxes[17].x[5] = 0.5
    with pytest.raises(MCGPUError, match="chain 31 molecule 0"):
        ChainBatch(ctx, boxes, seeds)
    boxes[3].pidx = np.zeros(0, np.int32)
    with pytest.raises(MCGPUError, match="chain 3: empty box"):
        ChainBatch(ctx, boxes, seeds)


def test_autotune_keeps_state(ctx):
    """The autotuner times tiles on saved copies of the rows: afterwards the
    batch is where it was and continues as a batch given the chosen tile."""
    boxes, seeds = W.water_chains(12, n_min=64, n_max=600, seed=44)
    a = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    t0 = a.tile
    a.run(32)
    before = _stats(a)
    tile = a.autotune(32)
    assert a.tile == tile and _stats(a) == before
    a.run(64)
    c = ChainBatch(ctx, boxes, seeds, rotation=ROT_AXIS)
    c.set_tile(*t0)
    c.run(32)
    c.set_tile(*tile)
    c.run(64)
    assert _stats(a) == _stats(c)
    for k in range(len(boxes)):
        assert all(np.array_equal(u, v) for u, v in zip(a.download(k), c.download(k)))
    a.close()
    c.close()
