"""One frame over several GPUs: the frame's pixel rows split into contiguous bands, one per rank, each rendered by
that rank's core with the seeds its paths have in the whole frame (lh2g_render_params rowBegin / rowCount), then
one gather of the bands. Paths are independent, so no data crosses ranks before the gather, and the gathered frame
equals the frame rendered on one GPU bit for bit. The scene and its BVH are replicated: every rank builds them
from the same inputs.

Lighthouse 2 has no multi-GPU path of its own (its cores render on one device); this follows the sharding its
wavefront layout allows: a path's pixel and sample come from its index alone.
"""
from __future__ import annotations

import numpy as np


def row_bands(height: int, world: int):
    """Contiguous bands of rows, as even as possible: [(rowBegin, rowCount)] for ranks 0..world-1 (a band may be
    empty when world > height)."""
    base, extra = divmod(height, world)
    bands, row = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        bands.append((row, n))
        row += n
    return bands


def band_params(params, rank: int, world: int):
    """A copy of the frame's render parameters restricted to this rank's band."""
    p = params.copy()
    begin, count = row_bands(int(params["height"]), world)[rank]
    p["rowBegin"], p["rowCount"] = begin, count
    return p


def render_band(core, view, params, rank: int, world: int, accumulate=False):
    """Renders this rank's band with a core whose target is the band (width x rowCount x spp) and returns its
    accumulator (rowCount * width float4). The core's target is set here when it does not match."""
    p = band_params(params, rank, world)
    W, spp, count = int(p["width"]), int(p["spp"]), int(p["rowCount"])
    if count == 0:
        return np.zeros((0, 4), np.float32)
    if (core.W, core.H, core.spp) != (W, count, spp):
        core.SetTarget(W, count, spp)
    core.render_ex(view, p, accumulate=accumulate, counters=False)
    return core.read_accumulator()


def gather_frame(dist, band: np.ndarray, params, rank: int, world: int, device="cpu"):
    """One gather of every rank's band into the whole frame (H * W float4, rows in order), returned on every rank.
    Bands differ in size by at most one row: each is padded to the largest for the collective."""
    import torch
    W, H = int(params["width"]), int(params["height"])
    bands = row_bands(H, world)
    rows = max(c for _, c in bands)
    buf = torch.zeros((rows * W, 4), dtype=torch.float32, device=device)
    if len(band):
        buf[:len(band)] = torch.from_numpy(np.ascontiguousarray(band, np.float32)).to(device)
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    out = np.zeros((H * W, 4), np.float32)
    for (begin, count), part in zip(bands, parts):
        out[begin * W:(begin + count) * W] = part[:count * W].cpu().numpy()
    return out
