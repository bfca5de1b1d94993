"""Synthetic boxes have the configured shape (sizes, density, geometry)."""
import numpy as np

from mcgpu_gb300 import workloads as W


def test_water_box_c0_shape():
    b = W.water_box(256, L=19.71)
    assert b.n_mol == 256 and b.n_atom == 768 and b.n_pidx == 256
    assert np.allclose(b.size, 19.71)
    o = np.stack([b.x[b.pidx], b.y[b.pidx], b.z[b.pidx]], 1)
    assert o.min() >= 0 and o.max() <= 19.71
    d = o[:, None] - o[None]
    d -= 19.71 * np.rint(d / 19.71)
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, 99)
    assert r.min() >= 2.5
    # rigid geometry: r_OH and the HOH angle
    h1 = np.stack([b.x[1::3], b.y[1::3], b.z[1::3]], 1) - o
    h2 = np.stack([b.x[2::3], b.y[2::3], b.z[2::3]], 1) - o
    assert np.allclose(np.linalg.norm(h1, axis=1), 0.9572)
    ang = np.degrees(np.arccos((h1 * h2).sum(1) / 0.9572 ** 2))
    assert np.allclose(ang, 104.52)


def test_bicyclic_template():
    xyz, sig, eps, q, prim = W.bicyclic_template()
    assert xyz.shape == (16, 3) and abs(q.sum()) < 1e-12
    # drawn in [-0.3, 0.3], then shifted by the mean to make the molecule neutral
    assert (np.abs(q) <= 0.6).all() and np.ptp(q) <= 0.6
    assert sig[prim] == 3.25 and eps[prim] == 0.17
    heavy = xyz[:9]
    d = np.linalg.norm(heavy[:, None] - heavy[None], axis=-1)
    bonds = np.sort(d[np.triu_indices(9, 1)])[:10]   # 6 + 5 - 1 ring bonds
    assert np.allclose(bonds, 1.40, atol=1e-9)
    assert np.allclose(xyz[:, 2], 0.0)                # planar


def test_water_chains_distribution():
    boxes, seeds = W.water_chains(16, seed=3)
    assert len(boxes) == 16 and len(set(int(s) for s in seeds)) == 16
    for b in boxes:
        assert 64 <= b.n_mol <= 2048
        assert abs(b.n_mol / b.size[0] ** 3 - W.WATER_DENSITY) < 1e-9
        assert b.cutoff <= 9.0 and b.cutoff <= b.size[0] / 2 + 1e-12
        assert 280 <= b.temperature <= 360


def test_generators_are_seeded():
    a, b = W.water_box(100, seed=5), W.water_box(100, seed=5)
    assert np.array_equal(a.x, b.x)
    assert not np.array_equal(a.x, W.water_box(100, seed=6).x)


def test_fcc_lattice_start():
    """FCC centres: 4000 molecules fill 10^3 cells exactly at L = 86.1 A,
    nearest centres a/sqrt(2) apart; one common orientation keeps the 16-atom
    molecules' atoms apart, so the start energy is finite and small."""
    from oracle.pyoracle import OracleBox
    c = W.fcc_centres(1, 4000, 86.1)
    assert c.shape == (4000, 3)
    d = c[:200, None, :] - c[None, :, :]
    d -= 86.1 * np.rint(d / 86.1)
    r = np.sqrt((d ** 2).sum(-1))
    r[np.arange(200), np.arange(200)] = np.inf
    assert abs(r.min() - 8.61 / np.sqrt(2)) < 1e-9
    box = W.bicyclic_box(500, seed=3, lattice=True)
    e = OracleBox(box).system_energy()
    assert np.isfinite(e) and e / box.n_mol < 1e3


def test_oracle_centre_builder_places_the_same_points():
    """The CPU baseline builds its workload with the oracle's centre builder
    (so it never loads the product library); it must give the product
    builder's points, hence bit-identical boxes."""
    from oracle.pyoracle import build_centres
    for n, L, dmin, seed in [(100, 15.0, 2.5, 5), (2048, 39.4, 2.5, 7), (300, 10.0, 0.0, 3),
                             (64, 12.3, 2.5, 2024 * 100003)]:
        assert np.array_equal(build_centres(seed, n, L, dmin), W.rsa_centres(seed, n, L, dmin))
    a, _ = W.water_chains(6, seed=11)
    b, _ = W.water_chains(6, seed=11, centres=build_centres)
    for x, y in zip(a, b):
        assert np.array_equal(x.x, y.x) and np.array_equal(x.z, y.z)


def test_tile_box_images_fit():
    """A periodic box replicated k x k x k: with the cutoff below half the
    small edge every molecule sees the same neighbours, so the system
    energy is k^3 times the small box's (oracle, FP64; the cutoff plus two
    molecule radii stays below half the small edge, so no atom pair of the
    small box takes a wrong single image)."""
    from mcgpu_gb300.prepare import tile_box
    from oracle.pyoracle import OracleBox
    small = W.water_box(40, L=13.0, cutoff=4.0, seed=9)
    big = tile_box(small, 2)
    assert big.n_mol == 320 and np.allclose(big.size, 26.0)
    assert np.array_equal(big.pidx[:40], small.pidx) and big.pidx[40] == small.n_atom
    e_small = OracleBox(small).system_energy()
    e_big = OracleBox(big).system_energy()
    assert abs(e_big - 8 * e_small) <= 1e-9 * abs(8 * e_small)
