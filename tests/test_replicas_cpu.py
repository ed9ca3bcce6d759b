"""Two-rank (gloo, CPU) check of the frame row split: each rank renders its band of rows with
the CPU oracle, the bands are all-gathered, and the result equals the single-process frame."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_path):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "atom-3d-engine_gb300"))
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle_py
    from mm3e_cuda import scenes
    from mm3e_cuda.replicas import row_band

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    scene, cam = scenes.demo_scene()
    y0, y1 = row_band(rank, world, scene.height)
    band = oracle_py.render_rows(scene.desc(), cam, y0, y1, threads=1)
    rows = torch.zeros((scene.height, scene.width, 3), dtype=torch.float32)
    rows[y0:y1] = torch.from_numpy(band)
    dist.all_reduce(rows)  # bands are disjoint: the sum is the gather
    if rank == 0:
        np.save(out_path, rows.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_row_bands_reassemble_the_frame(tmp_path):
    import oracle_py
    from mm3e_cuda import scenes

    out = str(tmp_path / "frame.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    gathered = np.load(out)
    scene, cam = scenes.demo_scene()
    full = oracle_py.render_rows(scene.desc(), cam, 0, scene.height, threads=2)
    assert np.array_equal(gathered, full)
