"""Multi-GPU layout of the render path: replicas, and the row split for sharding one frame.

The render path shards without any exchange: frames (or scenes, or requests) are independent,
so N GPUs run N replicas. Sharding a single frame splits its rows into contiguous bands with the
reference's rule (lib.rs:917-938: the first `h % n` bands take one extra row); the bands of the
HDR frame are then gathered before the post pass (bloom reads a 2*radius row halo).
"""


def row_band(rank, world, height):
    """Rows [y0, y1) of band `rank` of `world` (render_linear_unchecked's split)."""
    world = max(1, min(world, max(1, height)))
    if rank >= world:
        return 0, 0
    band, extra = divmod(height, world)
    y0 = rank * band + min(rank, extra)
    return y0, y0 + band + (1 if rank < extra else 0)


def bands(world, height):
    """The non-empty bands (a frame with fewer rows than ranks uses one rank per row)."""
    world = max(1, min(world, max(1, height)))
    return [row_band(r, world, height) for r in range(world)]
