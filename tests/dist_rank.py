"""One rank of the bench's multi-GPU form, on the CPU (gloo): started by
tests/test_distributed.py through bench.spawn_ranks, as bench.py --gpus N
starts its ranks.  The library's device selection is faked (no GPU here)."""
from __future__ import annotations

import json
import os
import pathlib
import sys

sys.path.insert(0, str(pathlib.Path(__file__).resolve().parents[1]))

import bench  # noqa: E402


class FakeLibrary:
    """Stands in for the package's device selection: records the ordinal."""

    def __init__(self):
        self.ordinal = -1

    def set_device(self, k: int) -> None:
        self.ordinal = k

    def device_ordinal(self) -> int:
        return self.ordinal


def main(out_dir: str, n: int) -> None:
    lib = FakeLibrary()
    rank, world, local = bench.dist_setup(n, lib)
    specs = bench.workload_sizes("batch256", 256, 20261203)
    mine = [i for i in range(len(specs)) if i % world == rank]
    atoms = sum(10 * c * r for c, r, _ in (specs[i] for i in mine))
    bench.barrier(world)
    t_max = bench.max_over_ranks(float(rank + 1), world)
    total = bench.sum_over_ranks(float(atoms), world)
    rec = {"rank": rank, "world": world, "local": local, "device": lib.device_ordinal(), "mine": mine,
           "atoms": atoms, "t_max": t_max, "total": total}
    pathlib.Path(out_dir, f"rank{rank}.json").write_text(json.dumps(rec))
    import torch.distributed as dist

    dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1], int(sys.argv[2]))
