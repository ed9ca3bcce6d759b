"""Parity metrics between the CUDA path and the CPU oracle (the spec acceptance bars)."""
import numpy as np

NIL = 0xFFFFFFFF


def image_metrics(gpu_rgb8, ref_rgb8):
    """(iii): RGB8 within 1 LSB on >= 99.9% of pixels, PSNR >= 50 dB."""
    a = np.asarray(gpu_rgb8)[..., :3].astype(np.int32)
    b = np.asarray(ref_rgb8)[..., :3].astype(np.int32)
    d = np.abs(a - b)
    px = d.max(-1)
    mse = float((d.astype(np.float64) ** 2).mean())
    psnr = float("inf") if mse == 0 else 10.0 * np.log10(255.0 ** 2 / mse)
    return {"psnr": psnr, "within1_px": float((px <= 1).mean()), "exact_px": float((px == 0).mean()),
            "max": int(d.max()), "mean_abs": float(d.mean())}


def silhouette_mask(mat):
    """Pixels whose 4-neighbourhood holds a different hit/miss or material id."""
    m = np.asarray(mat)
    edge = np.zeros(m.shape, bool)
    edge[1:, :] |= m[1:, :] != m[:-1, :]
    edge[:-1, :] |= m[:-1, :] != m[1:, :]
    edge[:, 1:] |= m[:, 1:] != m[:, :-1]
    edge[:, :-1] |= m[:, :-1] != m[:, 1:]
    return edge


def hit_metrics(gpu, ref):
    """(i) hit/miss mask and matId identical except silhouette pixels (<= 0.1% counted);
    (ii) hit distance within 1e-4 relative on agreed hits."""
    gm, rm = gpu["mat"], ref["mat"]
    diff = gm != rm
    sil = silhouette_mask(rm) | silhouette_mask(gm)
    n = gm.size
    agreed = (~diff) & (rm != NIL)
    rel = np.abs(gpu["t"][agreed].astype(np.float64) - ref["t"][agreed]) / np.maximum(np.abs(ref["t"][agreed]), 1e-12)
    return {"mismatch": int(diff.sum()), "mismatch_frac": float(diff.sum()) / n,
            "mismatch_off_silhouette": int((diff & ~sil).sum()), "agreed_hits": int(agreed.sum()),
            "t_rel_max": float(rel.max()) if rel.size else 0.0,
            "t_within_1e-4": float((rel <= 1e-4).mean()) if rel.size else 1.0}
