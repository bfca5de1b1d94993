"""Host driver with the reference's command line: ``metrosim`` on the GPU.

    python -m mcgpu_gb300.metrosim <input.config|input.state> [options]

It reads the reference's files (``files.load``), runs the Metropolis loop of
Simulation::run (Simulation.cpp:64-300) through this package's GPU path and
writes the reference's outputs: ``<name>_<step>.state`` files at the state
interval and at the end, ``<name>.pdb`` and ``<name>.results``, and the same
summary lines on stdout (the final energy includes the long-range
correction, as the reference's does).

Options follow CommandParsing.cpp:40-190: ``-n/--steps``,
``-i/--status-interval``, ``-I/--state-interval``, ``--name``,
``-S/--strategy`` (brute, prox, nlc, verlet and their long names),
``-k/--verbose``, ``-l/--neighbor [interval]``, ``-s/--serial``,
``-p/--parallel``, ``-V/--version``.  ``-s`` is accepted for compatibility;
every form runs on the GPU.

Three forms of the loop:

* ``--form plain`` (default): the reference's loop step for step -- the C
  library's ``rand()`` seeded with the environment's seed, moves drawn in the
  reference's order, the decision on the host -- with the energies on the
  GPU (FP64 pairs, or FP32 pairs with ``--precision mixed``).  With FP64 it
  reproduces the reference's trajectory.
* ``--form device``: the same loop entirely on the GPU (one CTA, the C
  library's generator restated on the device and seeded with the
  environment's seed): the same draws and decisions, no intermediate states.
* ``--form chain``: one device-resident chain (Philox draws, the decision on
  the GPU, rotations as X->Y->Z Euler angles like the reference's) advanced in
  launches of many steps; ``ensemble=npt`` gives isobaric ln V moves every
  ``volume-interval`` steps at the configured pressure, ``-S verlet`` or
  ``-l`` Verlet lists.  ``--checkpoint-interval`` also writes
  ``<name>_<step>.ckpt`` (the exact device state) and ``--resume`` continues
  one bit for bit.

``--intra`` turns on the reference's intramolecular moves (its compile-time
ENABLE_INTRA, SimulationStep.h:15, false in its sources): bond stretches and
angle expansions of the molecules' variable bonds and angles, with their
energies, in the plain and device forms.  ``--implied-angles`` starts the
z-matrix scanner's implied-angle flag set (the reference leaves it
uninitialised; its program was seen to run with it clear).

Every strategy gives the exact in-range molecule set here, so ``-S`` only
chooses Verlet lists for the chain form; the reference's NLC and Verlet
strategies screen other sets (NLCStep.cpp:69, VerletStep.cpp:177) and its
NPT ensemble scales a fixed 10 % volume step and accepts every move with the
volume rule (Ensemble.cpp:9-23), so neither is imitated.
"""
from __future__ import annotations

import argparse
import sys
import time
from dataclasses import dataclass

from . import _abi
from . import files as F
from .batch import ChainBatch
from .step import Context, GpuBox, GpuSimulationStep, LibcRand

VERSION = "mcgpu_gb300 metrosim 0.1"
STRATEGIES = {"brute": "brute", "brute-force": "brute", "prox": "prox",
              "proximity-matrix": "prox", "nlc": "nlc", "neighbor-linked-cell": "nlc",
              "verlet": "verlet", "verlet-list": "verlet"}
DEFAULT_STATUS_INTERVAL = 1000       # CommandParsing.h:21
DEFAULT_NEIGHBORLIST_INTERVAL = 100  # CommandParsing.h:22


@dataclass
class RunResult:
    energy: float          # final energy including the long-range correction
    lrc: float
    accepted: int
    rejected: int
    start_step: int
    steps: int
    box: tuple
    run_time: float
    files: list


def parse_args(argv):
    p = argparse.ArgumentParser(prog="metrosim", add_help=True,
                                description="Metropolis Monte Carlo on the GPU (reference CLI)")
    p.add_argument("input", nargs="?")
    p.add_argument("-n", "--steps", type=int, default=0)
    p.add_argument("-i", "--status-interval", type=int, default=DEFAULT_STATUS_INTERVAL)
    p.add_argument("-I", "--state-interval", type=int, default=0)
    p.add_argument("--name", default="")
    p.add_argument("-S", "--strategy", default="")
    p.add_argument("-k", "--verbose", action="store_true")
    p.add_argument("-l", "--neighbor", nargs="?", const=DEFAULT_NEIGHBORLIST_INTERVAL, type=int,
                   default=None)
    p.add_argument("-s", "--serial", action="store_true")
    p.add_argument("-p", "--parallel", action="store_true")
    p.add_argument("-V", "--version", action="store_true")
    p.add_argument("--form", choices=("plain", "device", "chain"), default="plain")
    p.add_argument("--intra", action="store_true")
    p.add_argument("--implied-angles", action="store_true")
    p.add_argument("--precision", choices=("fp64", "mixed"), default="fp64")
    p.add_argument("--device", type=int, default=0)
    p.add_argument("--skin", type=float, default=1.5)
    p.add_argument("--max-dlnv", type=float, default=0.01)
    p.add_argument("--checkpoint-interval", type=int, default=0)
    p.add_argument("--resume", default="")
    a = p.parse_args(argv)
    if a.version:
        return a
    if not a.input:
        raise F.FileFormatError("metrosim: Input file not specified")
    if a.serial and a.parallel:
        raise F.FileFormatError("metrosim: Cannot specify both GPU and CPU modes")
    if a.steps < 0 or ("-n" in argv or "--steps" in argv) and a.steps <= 0:
        raise F.FileFormatError("metrosim:  --steps (-n): Step count must be greater than zero")
    if a.status_interval < 0:
        raise F.FileFormatError("metrosim:  --status_interval (-i): Status Interval must be "
                                "non-negative")
    if a.neighbor is not None and a.neighbor < 1:
        raise F.FileFormatError("metrosim:  --neighborlist_interval (-l): Neighborlist Interval "
                                "must be greater than 0")
    if a.strategy and a.strategy not in STRATEGIES:
        raise F.FileFormatError("metrosim: Unknown energy calculation strategy specified")
    if F.extension(a.input) not in ("config", "state"):
        raise F.FileFormatError("metrosim: Must specify a config or state file")
    return a


def _log(msg: str, out) -> None:
    if out is not None:
        out.write(msg)


def run(argv=None, out=sys.stdout) -> RunResult | None:
    """Runs one simulation as ``metrosim argv`` would; returns its result."""
    argv = list(sys.argv[1:] if argv is None else argv)
    a = parse_args(argv)
    if a.version:
        _log(VERSION + "\n", out)
        return None
    inp = F.load(a.input, implied_angles=a.implied_angles)
    if a.intra and a.form == "chain":
        raise F.FileFormatError("--intra runs in the plain or device form (the chain form moves "
                                "rigid molecules)")
    cfg = inp.config
    name = a.name or (cfg.sim_name if cfg else "")
    pdb_dir = cfg.pdb_output if cfg else ""
    state_dir = cfg.state_output if cfg else ""
    ensemble = cfg.ensemble if cfg else ""
    vol_interval = cfg.volume_interval if cfg else 0
    strategy = STRATEGIES.get(a.strategy or (cfg.strategy if cfg else ""), "brute")
    if cfg and cfg.strategy and not a.strategy and cfg.strategy not in STRATEGIES:
        raise F.FileFormatError("Error: Unknown energy calculation strategy specified in "
                                "config file")
    steps = a.steps if a.steps > 0 else inp.steps
    box = inp.box
    env = box.env
    seed = env.random_seed
    _log("Using seed: %d\n" % seed, out)
    try:
        lrc0 = F.energy_lrc(env, box.molecules)
    except F.FileFormatError as e:
        sys.stderr.write("note: no long-range correction: %s\n" % e)
        lrc0 = 0.0
    V0 = env.x * env.y * env.z
    base = name or "untitled"
    written = []

    def save_state(step: int, coords, edges) -> None:
        env.x, env.y, env.z = (float(v) for v in edges)
        p = F.state_path(base, step, state_dir)
        F.write_state(p, box, step, coords)
        written.append(p)

    if name:
        _log("Simulation Name: %s\n" % name, out)
    _log("Running %d time steps" % steps + (" starting from step %d" % inp.start_step
                                            if inp.start_step > 0 else "") + "\n", out)
    t0 = time.perf_counter()
    ctx = Context(a.device)
    try:
        if a.form == "plain":
            if ensemble == "npt":
                raise F.FileFormatError("ensemble=npt runs in the chain form (--form chain)")
            res = _run_plain(a, ctx, inp, steps, lrc0, save_state, out)
        elif a.form == "device":
            if ensemble == "npt":
                raise F.FileFormatError("ensemble=npt runs in the chain form (--form chain)")
            res = _run_device(a, ctx, inp, steps, lrc0)
        else:
            res = _run_chain(a, ctx, inp, steps, lrc0, ensemble, vol_interval, strategy, base,
                             state_dir, save_state, written, out)
    finally:
        ctx.close()
    energy, acc, rej, coords, edges, start = res
    run_time = time.perf_counter() - t0
    lrc = lrc0 * V0 / (edges[0] * edges[1] * edges[2])
    env.x, env.y, env.z = (float(v) for v in edges)
    pdb = F.pdb_path(name, pdb_dir)
    F.write_pdb(pdb, box, coords)
    written.append(pdb)
    end = start + steps
    if a.state_interval >= 0:
        save_state(end, coords, edges)
    _log("\nFinished running %d steps\n" % steps, out)
    _log("LJ-Energy Subtotal: %.3f\n" % 0.0, out)
    _log("Charge Energy Subtotal: %.3f\n" % 0.0, out)
    _log("Energy Long-range Correction: %.3f\n" % lrc, out)
    _log("Ewald Energy: %.3f\n" % 0.0, out)
    _log("Final Energy: %.3f\n" % energy, out)
    _log("Run Time: %.3f seconds\n" % run_time, out)
    _log("Accepted Moves: %d\n" % acc, out)
    _log("Rejected Moves: %d\n" % rej, out)
    _log("Acceptance Ratio: %.2f%%\n" % (100.0 * acc / max(1, acc + rej)), out)
    results = (name or "run") + ".results"
    with open(results, "w") as f:
        f.write(F.format_results(sim_name=name, mode="GPU", start_step=start,
                                 steps=steps, n_molecules=env.n_molecules, energy=energy,
                                 run_time=run_time, accepted=acc, rejected=rej))
    written.append(results)
    return RunResult(energy, lrc, acc, rej, start, steps, tuple(edges), run_time,
                     written)


def _box(a, ctx, inp):
    prec = _abi.PREC_FP64 if a.precision == "fp64" else _abi.PREC_MIXED
    g = GpuBox(ctx, inp.rows, prec)
    if a.intra:
        g.set_topology(inp.topology)
        g.set_intra(True)
    return g


def _run_device(a, ctx, inp, steps, lrc0):
    """The same loop entirely on the GPU (mcgpu_run_plain_device): the C
    library's generator restated on the device, seeded with the
    environment's seed; no intermediate states."""
    env = inp.box.env
    g = _box(a, ctx, inp)
    st = g.run_plain_device(env.random_seed, steps)
    coords = g.download()
    g.close()
    return st.energy + lrc0, st.accepted, st.rejected, coords, (env.x, env.y, env.z), \
        inp.start_step


def _run_plain(a, ctx, inp, steps, lrc0, save_state, out):
    """Simulation::run's loop (Simulation.cpp:219-264) on GpuSimulationStep.
    With --intra (the reference's ENABLE_INTRA): molecule energies with the
    intramolecular term, the intramolecular move after the rigid one (its
    draws taken by the library from the same rand()), the step counter the
    width tuning reads starting at 0 (SimBoxBuilder.cpp:37)."""
    env = inp.box.env
    edges = (env.x, env.y, env.z)
    g = _box(a, ctx, inp)
    rng = LibcRand(env.random_seed)
    step = GpuSimulationStep(g, rng)
    energy = step.calc_system_energy() + lrc0
    acc = rej = 0
    start = inp.start_step
    for move in range(start, start + steps):
        if a.verbose and a.status_interval > 0 and (move - start) % a.status_interval == 0:
            _log("Step %d:\n--Current Energy: %s\n\n" % (move, F.fmt_g(energy)), out)
        if a.state_interval > 0 and move > start and (move - start) % a.state_interval == 0:
            save_state(move, g.download(), edges)
        idx = step.choose_molecule()
        if a.intra:
            g.set_step(move - start)
            old = step.calc_molecule_energy(idx, 0)
            step.change_molecule(idx)
            new = step.calc_molecule_energy(idx, 0)
        else:
            mv = step.draw_move(idx)
            old, new = g.move_energies(idx, *mv)
        if step.accept_move(new - old):
            acc += 1
            energy += new - old
        else:
            rej += 1
            step.rollback(idx)
    coords = g.download()
    g.close()
    return energy, acc, rej, coords, edges, start


def _run_chain(a, ctx, inp, steps, lrc0, ensemble, vol_interval, strategy, base, state_dir,
               save_state, written, out):
    """The device-resident chain: launches of many steps between the state
    and checkpoint intervals."""
    env = inp.box.env
    V0 = env.x * env.y * env.z
    bt = ChainBatch(ctx, [inp.rows], [env.random_seed], rotation=_abi.ROT_EULER)
    if strategy == "verlet" or a.neighbor is not None:
        bt.set_verlet(a.skin)
    if ensemble == "npt":
        if vol_interval <= 0:
            raise F.FileFormatError("ensemble=npt needs volume-interval > 0")
        # the reference's pressure is in kcal/mol/A^3 (SimulationStep.cpp:476-488)
        bt.set_npt(vol_interval, env.pressure / 1.4583972574259083e-05, a.max_dlnv,
                   _abi.PREC_MIXED)
        # the tail correction follows the volume (E_LRC * V is constant)
        bt.set_lrc([lrc0 * V0])
    start = inp.start_step
    if a.resume:
        with open(a.resume, "rb") as f:
            bt.restore(f.read())
    # steps are labelled from the input's step (a .state file's, or the
    # checkpoint's); the chain's Philox counter runs on from its own count
    first = bt.stats()[0]
    if a.resume:
        start = int(first.steps)
    acc0, steps0 = int(first.accepted), int(first.steps)
    done = 0
    marks = sorted({s for s in range(1, steps) for iv in (a.state_interval,
                                                          a.checkpoint_interval)
                    if iv > 0 and s % iv == 0})
    for m in marks + [steps]:
        if m > done:
            bt.run(m - done)
            done = m
        if m == steps:
            break
        st = bt.stats()[0]
        if a.state_interval > 0 and m % a.state_interval == 0:
            save_state(start + m, bt.download(0), tuple(st.box))
        if a.checkpoint_interval > 0 and m % a.checkpoint_interval == 0:
            p = (state_dir + "/" if state_dir else "") + "%s_%d.ckpt" % (base, start + m)
            with open(p, "wb") as f:
                f.write(bt.checkpoint())
            written.append(p)
    st = bt.stats()[0]
    if st.error:
        bt.close()
        raise _abi.MCGPUError("device chain reported error %d" % st.error)
    edges = tuple(st.box)
    V = edges[0] * edges[1] * edges[2]
    energy = st.energy + lrc0 * V0 / V
    acc = int(st.accepted) - acc0
    rej = int(st.steps) - steps0 - acc
    if a.checkpoint_interval > 0:
        p = (state_dir + "/" if state_dir else "") + "%s_%d.ckpt" % (base, start + steps)
        with open(p, "wb") as f:
            f.write(bt.checkpoint())
        written.append(p)
    coords = bt.download(0)
    bt.close()
    return energy, acc, rej, coords, edges, start


def main(argv=None) -> int:
    try:
        res = run(argv)
    except F.FileFormatError as e:
        sys.stderr.write(str(e) + "\n")
        return 1
    if res is not None:
        _log("Finishing simulation...\n\n", sys.stdout)
    return 0


if __name__ == "__main__":
    sys.exit(main())
