"""Relaxed starting states for the measured workloads, made on the GPU by the
device-resident chain itself.

Random starts at liquid density carry close contacts and random orientations
(no hydrogen-bond network): their energies are positive and the first
thousands of moves relax them, so steps timed from them do not describe the
liquid.  The reference builds its starts on an FCC lattice and runs its loop
from there (FileUtilities.cpp:550-642, Simulation.cpp:219-264); here:

* ``relax``               a box advanced by the chain kernel (NVT, Philox
                          proposals, on-device accept) and downloaded.
* ``tile_box``            a periodic box replicated k x k x k: the images of
                          a periodic configuration fit without new contacts.
* ``relaxed_water_32768`` 512 waters relaxed at the density of the 32,768-
                          water system, replicated 4 x 4 x 4 into it.
"""
from __future__ import annotations

import numpy as np

from . import _abi
from .batch import ChainBatch
from .step import Context
from .workloads import BoxData, water_box


def relax(ctx: Context, box: BoxData, seed: int, steps: int,
          tile=(256, 1, 64, 0)) -> BoxData:
    """`box` after `steps` Metropolis steps of the device-resident chain
    (rotation about a random axis, Philox key `seed`)."""
    bt = ChainBatch(ctx, [box], [seed], rotation=_abi.ROT_AXIS)
    try:
        bt.set_tile(*tile)
        bt.run(int(steps))
        st = bt.stats()[0]
        if st.error:
            raise RuntimeError(f"relaxation run reported device error {st.error}")
        x, y, z = bt.download(0)
    finally:
        bt.close()
    out = box.copy()
    out.x, out.y, out.z = x, y, z
    return out.normalise()


def tile_box(box: BoxData, k: int) -> BoxData:
    """The box replicated k times along each edge (molecules of image
    (i, j, l) shifted by (i, j, l) times the edges, in that loop order);
    same cutoff, temperature and move sizes."""
    L = np.asarray(box.size, np.float64)
    shifts = np.array([(i, j, l) for i in range(k) for j in range(k) for l in range(k)],
                      np.float64) * L
    n_img = shifts.shape[0]
    na, nm, npi = box.n_atom, box.n_mol, box.n_pidx
    out = BoxData(
        x=(box.x[None, :] + shifts[:, 0, None]).ravel(),
        y=(box.y[None, :] + shifts[:, 1, None]).ravel(),
        z=(box.z[None, :] + shifts[:, 2, None]).ravel(),
        sigma=np.tile(box.sigma, n_img), epsilon=np.tile(box.epsilon, n_img),
        charge=np.tile(box.charge, n_img),
        mol_start=(box.mol_start[None, :] + na * np.arange(n_img)[:, None]).ravel(),
        mol_len=np.tile(box.mol_len, n_img),
        mol_pidx_start=(box.mol_pidx_start[None, :] + npi * np.arange(n_img)[:, None]).ravel(),
        mol_pidx_count=np.tile(box.mol_pidx_count, n_img),
        pidx=(box.pidx[None, :] + na * np.arange(n_img)[:, None]).ravel(),
        size=L * k, cutoff=box.cutoff, temperature=box.temperature,
        max_translate=box.max_translate, max_rotate=box.max_rotate,
        name=f"{box.name}x{k}")
    assert out.n_mol == nm * n_img
    return out.normalise()


def relaxed_water_32768(ctx: Context, sweeps: int = 400, seed: int = 0x4C49515549) -> BoxData:
    """The 32,768-water system (L = 99.3 A, rc 12 A, 298 K) from a liquid
    start: 512 waters in a box of a quarter of the edge (rc 9 A there)
    relaxed for `sweeps` x 512 steps, then replicated 4 x 4 x 4."""
    small = water_box(512, L=99.3 / 4, cutoff=9.0, temperature=298.0, seed=32768)
    small = relax(ctx, small, seed, sweeps * 512)
    big = tile_box(small, 4)
    big.cutoff = 12.0
    big.name = "water32768_relaxed"
    return big
