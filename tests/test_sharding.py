"""One frame split over ranks by rows (lighthouse2_gb300.sharding): each of two gloo ranks renders its band of a
small frame with the oracle, one all-gather puts the bands together, and the result equals the frame rendered
whole, bit for bit (every path keeps the seeds it has in the whole frame). Also the band arithmetic."""
import os

import numpy as np
import pytest

from lighthouse2_gb300 import sharding


def test_row_bands():
    for H in (1, 7, 32, 1080):
        for world in (1, 2, 3, 8):
            b = sharding.row_bands(H, world)
            assert len(b) == world and b[0][0] == 0 and sum(c for _, c in b) == H
            assert all(b[i][0] + b[i][1] == b[i + 1][0] for i in range(world - 1))
            assert max(c for _, c in b) - min(c for _, c in b) <= 1


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"], os.environ["MASTER_PORT"] = "127.0.0.1", str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from lighthouse2_gb300 import scenes as S
        from oracle import bind
        sc = S.cornell_sphere(subdiv=3)
        o = bind.Oracle()
        o.set_scene(sc)
        for W, H, spp in ((40, 31, 1), (24, 17, 3)):
            view = S.cornell_view(W, H)
            p = bind.make_params(W, H, spp, max_depth=5, rr_start=2, camera_r0=bind.camera_r0(1), flags=bind.RP_NEE | bind.RP_DEPTH_W)
            band = o.render(view, sharding.band_params(p, rank, world))["accum"]
            frame = sharding.gather_frame(dist, band, p, rank, world)
            if rank == 0:
                np.save(os.path.join(out_dir, f"split_{W}x{H}x{spp}.npy"), frame)
                np.save(os.path.join(out_dir, f"whole_{W}x{H}x{spp}.npy"), o.render(view, p)["accum"])
    finally:
        dist.destroy_process_group()


def test_split_frame_equals_whole_frame(tmp_path, oracle_lib):
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for W, H, spp in ((40, 31, 1), (24, 17, 3)):
        split = np.load(tmp_path / f"split_{W}x{H}x{spp}.npy")
        whole = np.load(tmp_path / f"whole_{W}x{H}x{spp}.npy")
        assert split.shape == whole.shape
        assert np.array_equal(split.view(np.uint32), whole.view(np.uint32))
        assert whole[:, :3].sum() > 0
