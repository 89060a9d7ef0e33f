"""Shots of one job split over ranks (one process per GPU): the host-side
partition and gather, run here as world_size-2 gloo processes on CPU with the
CPU oracle standing in for each rank's GPU state.  A rank simulating shots
[first, first + count) with its shot offset set draws exactly what one state
holding all shots draws for that range, so the gathered records equal the
single-process records bit for bit."""
import os
import socket

import numpy as np
import pytest


def test_shard_range_covers_exactly():
    from plaquette_simulator.shard import shard_range, weak_range
    for total in (0, 1, 63, 64, 65, 256, 1000, 16384, 16385):
        for world in (1, 2, 3, 4, 8):
            parts = [shard_range(total, world, r) for r in range(world)]
            pos = 0
            for first, count in parts:
                assert first == pos or count == 0
                assert first % 64 == 0
                pos = first + count if count else pos
            assert sum(c for _, c in parts) == total
            words = [(c + 63) // 64 for _, c in parts]
            assert max(words) - min(words) <= 1
    assert weak_range(16384, 3) == (49152, 16384)
    with pytest.raises(ValueError):
        weak_range(100, 0)
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, total, out_path):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    sys.path.insert(0, os.path.join(root, "plaquette-simulator_gb300", "python"))
    import torch.distributed as dist
    import oracle
    from plaquette_simulator import circuits as C
    from plaquette_simulator.shard import gather_records, shard_range
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    circ = C.surface_code_memory(3, 3, p=0.02)
    first, count = shard_range(total, world, rank)
    o = oracle.Oracle(circ.num_qubits, count, seed=2024, shot_base=first)
    o.run(circ.op_array(), circ.param_array())
    nm = circ.num_measurements()
    bits = np.stack([o.record(k)[0] for k in range(nm)]).astype(np.uint8)
    det = np.stack([o.record(k)[1] for k in range(nm)]).astype(np.uint8)
    allbits = gather_records(bits)
    alldet = gather_records(det)
    if rank == 0:
        np.savez(out_path, res=allbits, det=alldet)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_reproduce_one_state(O, tmp_path):
    import torch.multiprocessing as mp
    from plaquette_simulator import circuits as C
    total, world = 320, 2  # 5 words: ranks hold 192 and 128 shots
    out = str(tmp_path / "gathered.npz")
    mp.spawn(_worker, args=(world, _free_port(), total, out), nprocs=world, join=True)
    got = np.load(out)
    circ = C.surface_code_memory(3, 3, p=0.02)
    o = O.Oracle(circ.num_qubits, total, seed=2024)
    o.run(circ.op_array(), circ.param_array())
    for k in range(circ.num_measurements()):
        res, det = o.record(k)
        assert np.array_equal(got["res"][k], res), f"record {k} results differ"
        assert np.array_equal(got["det"][k], det), f"record {k} determined differ"
