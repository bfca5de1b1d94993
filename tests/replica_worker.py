"""One rank of the two-rank CPU check of bench.py's replica path (launched by
test_replicas.py under torch.distributed.run; gloo): the max and sum
reductions behind `value` and `ms_per_step`, and distinct seeded replicas
per rank."""
import importlib.util
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
bench = importlib.util.module_from_spec(spec)
spec.loader.exec_module(bench)

import torch  # noqa: E402

ws, rank, local = bench.dist_info()
dist = bench.dist_init(ws)
assert ws == 2 and dist is not None
# max over ranks of the timed region, sum of the units processed
assert bench.dist_max(dist, 1.0 + rank) == 2.0
assert bench.dist_sum(dist, 1.0 + rank) == 3.0
# every rank runs its own replica: the seeds bench.py gives each rank make
# different chains
from mcgpu_gb300 import workloads as W  # noqa: E402

boxes, seeds = W.water_chains(4, n_min=64, n_max=128, seed=2024 + 7919 * rank)
mine = float(np.sum(boxes[0].x)) + float(np.sum(seeds))
t = torch.zeros(2, dtype=torch.float64)
t[rank] = mine
dist.all_reduce(t)
assert t[rank].item() == mine and t[0].item() != t[1].item()
dist.barrier()
dist.destroy_process_group()
print(f"rank {rank} ok", flush=True)
