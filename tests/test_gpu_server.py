"""The serving loop: continuous batching of jobs with admission by slots
and HBM footprint.  A job's result is the same alone and in any mix (its
trajectory depends on its own seed, chain id and ensemble only), and equals
the oracle's run of the same chain."""
import numpy as np
import pytest

from helpers import load_golden
from mcgpu_gb300 import PREC_FP64, PREC_MIXED, JobServer, MCGPUError, ROT_AXIS
from mcgpu_gb300 import workloads as W
from oracle.pyoracle import OracleChain

pytestmark = pytest.mark.gpu

MB = 1 << 20


@pytest.fixture(scope="module")
def ctx():
    from mcgpu_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def mixed_jobs(n, seed):
    """Water chains of uneven sizes and a few bicyclic (16-atom) boxes."""
    boxes, seeds = W.water_chains(n, n_min=64, n_max=400, seed=seed)
    jobs = []
    rng = np.random.default_rng(seed)
    for i, (b, s) in enumerate(zip(boxes, seeds)):
        jobs.append(dict(box=b, seed=int(s), n_steps=int(rng.integers(1, 6)) * 50,
                         chain_id=i, npt=bool(i % 2), pressure_atm=1.0, max_dlnv=0.02,
                         vol_precision=PREC_MIXED if i % 4 == 1 else PREC_FP64))
    bic = load_golden("bicyclic100")[0]
    jobs.insert(3, dict(box=bic, seed=4242, n_steps=150, chain_id=77, npt=True,
                        pressure_atm=1.0, max_dlnv=0.02))
    return jobs


def run_server(ctx, jobs, **kw):
    srv = JobServer(ctx, **kw)
    ids = [srv.submit(**j) for j in jobs]
    srv.drain()
    res = srv.results()
    srv.close()
    return [res[i] for i in ids]


def same(a, b):
    ra, rb = a.result, b.result
    assert ra.energy == rb.energy and ra.accepted == rb.accepted and ra.steps == rb.steps
    assert ra.vol_tried == rb.vol_tried and ra.vol_accepted == rb.vol_accepted
    assert tuple(ra.box) == tuple(rb.box)
    assert np.array_equal(a.coords, b.coords)


def test_server_alone_equals_mixed(ctx):
    jobs = mixed_jobs(12, seed=5)
    mixed = run_server(ctx, jobs, hbm_budget_bytes=64 * MB, max_slots=4, round_steps=50)
    for k in (0, 3, 7, 12):
        alone = run_server(ctx, [jobs[k]], hbm_budget_bytes=64 * MB, max_slots=4, round_steps=50)
        same(alone[0], mixed[k])
    for j, out in zip(jobs, mixed):
        assert out.result.steps == j["n_steps"] and out.result.error == 0
        assert out.result.t_submit <= out.result.t_admit <= out.result.t_done


def test_server_matches_oracle(ctx):
    """Served jobs (NVT and NPT) replayed by the oracle: same coordinates bit
    for bit, same volume decisions, energies within the FP32-pair rule."""
    jobs = mixed_jobs(4, seed=9)[:4]
    for j in jobs:
        if j["npt"]:   # a tail correction in the volume criterion (E_LRC * V)
            b = j["box"]
            j["lrc_v"] = -2.0 * b.n_mol * float(b.size[0] * b.size[1] * b.size[2])
    outs = run_server(ctx, jobs, hbm_budget_bytes=64 * MB, max_slots=8, round_steps=50)
    for j, out in zip(jobs, outs):
        oc = OracleChain(j["box"], ROT_AXIS)
        e = oc.system_energy()
        done, vacc = 0, 0
        while done < j["n_steps"]:
            k = min(50, j["n_steps"] - done)
            e, _, _ = oc.run(j["seed"], j["chain_id"], k, e, step0=done)
            done += k
            if j["npt"] and done % 50 == 0:
                r = oc.volume_move(j["seed"], j["chain_id"], done, j["pressure_atm"],
                                   j["max_dlnv"], e, j.get("lrc_v", 0.0))
                e = r["energy"]
                vacc += r["status"] == 1
        assert np.array_equal(out.coords, oc.coords())
        assert out.result.vol_accepted == vacc
        assert tuple(out.result.box) == tuple(oc.ob.s.size)
        b = j["box"]
        scale = sum(oc.ob.mol_energy_abs(m, m) for m in range(b.n_mol))
        assert abs(out.result.energy - e) <= 1e-5 * max(abs(e), 1e-3 * scale) + 50 * 1e-9 * scale


def test_server_admission_by_footprint(ctx):
    """A budget that holds about two jobs: never more resident bytes than the
    budget, jobs wait in the queue and all complete; a job larger than the
    budget is refused at submit."""
    boxes, seeds = W.water_chains(6, n_min=300, n_max=400, seed=3)
    big = max(b.n_atom * 108 + b.n_mol * 88 + b.n_pidx * 20 for b in boxes) + 4096
    srv = JobServer(ctx, hbm_budget_bytes=2 * big + 1024, max_slots=16, round_steps=40)
    for i, (b, s) in enumerate(zip(boxes, seeds)):
        srv.submit(b, int(s), 120, chain_id=i)
    peak_bytes, peak_run = 0, 0
    while True:
        st = srv.status()
        peak_bytes = max(peak_bytes, st["bytes_in_use"])
        peak_run = max(peak_run, st["running"])
        if st["finished"] == len(boxes):
            break
        srv.step()
    assert peak_bytes <= 2 * big + 1024 and 1 <= peak_run <= 2
    res = srv.results()
    assert len(res) == len(boxes) and all(r.result.steps == 120 for r in res.values())
    huge = W.water_box(4000, seed=1)
    with pytest.raises(MCGPUError):
        srv.submit(huge, 1, 10)
    srv.close()


def test_server_overlapping_arrivals(ctx):
    """Jobs submitted while others run are admitted between rounds and their
    work overlaps on the device (several resident at once)."""
    jobs = mixed_jobs(10, seed=21)
    srv = JobServer(ctx, hbm_budget_bytes=256 * MB, max_slots=6, round_steps=50)
    ids, max_running = [], 0
    for j in jobs:
        ids.append(srv.submit(**j))
        srv.step()
        max_running = max(max_running, srv.status()["running"])
    srv.drain()
    res = srv.results()
    assert max_running >= 3
    alone = run_server(ctx, [jobs[5]], hbm_budget_bytes=64 * MB, max_slots=6, round_steps=50)
    same(alone[0], res[ids[5]])
    srv.close()


@pytest.mark.parametrize("tile", [(512, 1, 0), (512, 2, 0)])
def test_server_wide_tiles_agree(ctx, tile):
    """Rounds with 512-thread CTAs (the wide chain kernel) give the same jobs."""
    jobs = mixed_jobs(4, seed=21)[:5]
    base = run_server(ctx, jobs, hbm_budget_bytes=64 * MB, max_slots=8, round_steps=50)
    wide = run_server(ctx, jobs, hbm_budget_bytes=64 * MB, max_slots=8, round_steps=50,
                      tile=tile)
    for a, b in zip(base, wide):
        assert a.result.accepted == b.result.accepted
        assert np.array_equal(a.coords, b.coords)
        assert abs(a.result.energy - b.result.energy) <= 1e-9 * max(1.0, abs(a.result.energy))
