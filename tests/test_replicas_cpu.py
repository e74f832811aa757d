"""World-size-2 `gloo` test of the multi-GPU path: independent decks sharded
round robin over two ranks (CPU processes here), solved with no exchange, the
results gathered back into deck order and the time taken as the maximum over
ranks.  The per-deck solver is the CPU oracle, so the test needs no GPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
N_DECKS = 5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _solve_deck(k):
    sys.path.insert(0, str(ROOT / "oracle"))
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle as O
    from parity_util import random_deck
    ch = O.OracleChunk(O.parse_deck(random_deck(24, 200 + k, steps=2, eps=1e-12)), O.make_opts(mode=1))
    ch.initialise()
    steps, sums = ch.diffuse()
    return [r.iters for r in steps], sums[-1][3]


def _worker(rank, world, port, out_dir):
    import time
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT / "tests"))
    import importlib
    from conftest import load_package
    load_package()
    replicas = importlib.import_module("tealeaf_gb300.replicas")
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    mine = replicas.deck_shard(N_DECKS, rank, world)
    t0 = time.perf_counter()
    res = [_solve_deck(k) for k in mine]
    t = time.perf_counter() - t0
    tmax = replicas.max_over_ranks(t, dist)
    merged = replicas.gather_by_deck(res, N_DECKS, dist)
    if rank == 0:
        import json
        Path(out_dir, "merged.json").write_text(json.dumps({"merged": merged, "tmax": tmax, "t0": t}))
    dist.barrier()
    dist.destroy_process_group()


def test_deck_shard():
    from conftest import load_package
    load_package()
    import importlib
    rep = importlib.import_module("tealeaf_gb300.replicas")
    assert rep.deck_shard(5, 0, 2) == [0, 2, 4] and rep.deck_shard(5, 1, 2) == [1, 3]
    assert sorted(sum((rep.deck_shard(7, r, 3) for r in range(3)), [])) == list(range(7))
    with pytest.raises(ValueError):
        rep.deck_shard(4, 2, 2)


def test_two_rank_gloo(tmp_path):
    import json
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = json.loads((tmp_path / "merged.json").read_text())
    serial = [_solve_deck(k) for k in range(N_DECKS)]
    assert [tuple((tuple(a), b)) for a, b in got["merged"]] == [tuple((tuple(a), b)) for a, b in serial]
    assert got["tmax"] >= got["t0"]
