"""Seeded synthetic inputs for the tensor-voting benchmarks.

No public dataset is involved: the workloads are defined by their recipe.
  tube_volume   3D: random tubes (piecewise-linear centrelines) + Gaussian noise,
                optionally planar sheets (the 3D voting workloads)
  tube_volume_device  the same geometry rasterised on a torch device (for
                volumes too large to build quickly on the host); its noise
                comes from the device generator
  curve_image   2D: random cubic Bezier curves + Gaussian noise (the 2D workload)
  eigen_batch   Q diag(l) Q^T tensors with Haar Q and log-uniform spectra,
                with near-degenerate and fully degenerate fractions
Everything is NumPy on the host (PCG64), so every process and machine that
uses the same seed gets the same arrays.
"""
import numpy as np


def _raster_segment(vol, p, q, r):
    """Set voxels whose centre lies within distance r of segment p-q to 1."""
    n0, n1, n2 = vol.shape
    lo = np.maximum(np.floor(np.minimum(p, q) - r - 1).astype(int), 0)
    hi = np.minimum(np.ceil(np.maximum(p, q) + r + 1).astype(int), [n0 - 1, n1 - 1, n2 - 1])
    if np.any(hi < lo):
        return
    z, y, x = np.meshgrid(np.arange(lo[0], hi[0] + 1), np.arange(lo[1], hi[1] + 1), np.arange(lo[2], hi[2] + 1),
                          indexing="ij")
    pts = np.stack([z, y, x], axis=-1).astype(np.float32)
    d = (q - p).astype(np.float32)
    dd = float(d @ d)
    t = np.clip(((pts - p) @ d) / dd, 0.0, 1.0) if dd > 0 else np.zeros(pts.shape[:3], np.float32)
    dist2 = ((pts - (p + t[..., None] * d)) ** 2).sum(-1)
    sub = vol[lo[0]:hi[0] + 1, lo[1]:hi[1] + 1, lo[2]:hi[2] + 1]
    sub[dist2 <= r * r] = 1.0


def tube_volume(n, n_tubes=64, r_range=(1.0, 3.0), segments=8, noise_sd=0.05, seed=2, n_sheets=0, sheet_thickness=2.0):
    """(n, n, n) float32 volume: n_tubes tubes of radius U(r_range) along
    `segments`-segment piecewise-linear random walks (segment length
    U(n/16, n/6)), intensity 1, plus n_sheets planar discs of the given
    thickness, plus N(0, noise_sd) noise."""
    segs, sheets = _geometry(n, n_tubes, r_range, segments, seed, n_sheets)
    vol = np.zeros((n, n, n), np.float32)
    for p, q, r in segs:
        _raster_segment(vol, p, q, r)
    for nrm, c, rad in sheets:
        lo = np.maximum(np.floor(c - rad).astype(int), 0)
        hi = np.minimum(np.ceil(c + rad).astype(int), n - 1)
        z, y, x = np.meshgrid(np.arange(lo[0], hi[0] + 1), np.arange(lo[1], hi[1] + 1), np.arange(lo[2], hi[2] + 1),
                              indexing="ij")
        rel = np.stack([z, y, x], axis=-1) - c
        h = rel @ nrm
        inplane = (rel ** 2).sum(-1) - h * h
        m = (np.abs(h) <= sheet_thickness / 2) & (inplane <= rad * rad)
        vol[lo[0]:hi[0] + 1, lo[1]:hi[1] + 1, lo[2]:hi[2] + 1][m] = 1.0
    # the noise continues the geometry's generator stream
    rng = np.random.default_rng(seed)
    _geometry_draws(rng, n, n_tubes, r_range, segments, n_sheets)
    vol += rng.standard_normal(vol.shape, dtype=np.float32) * np.float32(noise_sd)
    return vol


def curve_image(n=512, n_curves=32, width=1.5, noise_sd=0.05, seed=1):
    """(n, n) float32 image of n_curves random cubic Bezier curves of the
    given width (intensity 1) plus N(0, noise_sd) noise."""
    rng = np.random.default_rng(seed)
    img = np.zeros((n, n), np.float32)
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float32)
    ts = np.linspace(0, 1, 400, dtype=np.float32)
    for _ in range(n_curves):
        P = rng.uniform(0, n, (4, 2)).astype(np.float32)
        B = ((1 - ts) ** 3)[:, None] * P[0] + (3 * (1 - ts) ** 2 * ts)[:, None] * P[1] + \
            (3 * (1 - ts) * ts ** 2)[:, None] * P[2] + (ts ** 3)[:, None] * P[3]
        for (py, px) in B[::2]:
            y0, y1 = int(max(py - 3, 0)), int(min(py + 4, n))
            x0, x1 = int(max(px - 3, 0)), int(min(px + 4, n))
            if y0 >= y1 or x0 >= x1:
                continue
            d2 = (yy[y0:y1, x0:x1] - py) ** 2 + (xx[y0:y1, x0:x1] - px) ** 2
            img[y0:y1, x0:x1][d2 <= (width / 2) ** 2 + 0.25] = 1.0
    img += rng.standard_normal(img.shape, dtype=np.float32) * np.float32(noise_sd)
    return img


def eigen_batch(n, seed=3, log_range=(-6.0, 3.0), pair_frac=0.10, full_frac=0.01, pair_rel=1e-6, chunk=1 << 22):
    """(n, 9) float32 tensors Q diag(l) Q^T: Q Haar-random (QR of a Gaussian
    with the sign fix), l log-uniform in 10**log_range; pair_frac of them
    with a pair within pair_rel relative, full_frac fully degenerate."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, 9), np.float32)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        G = rng.standard_normal((m, 3, 3))
        Q, R = np.linalg.qr(G)
        Q *= np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
        lam = 10.0 ** rng.uniform(log_range[0], log_range[1], (m, 3))
        k = rng.uniform(size=m)
        pair = k < pair_frac
        lam[pair, 1] = lam[pair, 0] * (1 + rng.uniform(-pair_rel, pair_rel, int(pair.sum())))
        full = k >= 1.0 - full_frac
        lam[full, 1] = lam[full, 0]
        lam[full, 2] = lam[full, 0]
        out[s:s + m] = ((Q * lam[:, None, :]) @ np.swapaxes(Q, 1, 2)).reshape(m, 9)
    return out


def _geometry_draws(rng, n, n_tubes, r_range, segments, n_sheets):
    """The random draws of the tube/sheet recipe, in order, from `rng`:
    tube segments (p, q, r) and sheets (normal, centre, radius)."""
    segs, sheets = [], []
    for _ in range(n_tubes):
        r = rng.uniform(*r_range)
        p = rng.uniform(0, n, 3).astype(np.float32)
        for _ in range(segments):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            q = np.clip(p + d * rng.uniform(n / 16, n / 6), 0, n - 1).astype(np.float32)
            segs.append((p, q, r))
            p = q
    for _ in range(n_sheets):
        nrm = rng.normal(size=3)
        nrm /= np.linalg.norm(nrm)
        sheets.append((nrm, rng.uniform(0, n, 3), rng.uniform(n / 8, n / 3)))
    return segs, sheets


def _geometry(n, n_tubes, r_range, segments, seed, n_sheets):
    return _geometry_draws(np.random.default_rng(seed), n, n_tubes, r_range, segments, n_sheets)


def tube_volume_device(n, device, n_tubes=64, r_range=(1.0, 3.0), segments=8, noise_sd=0.05, seed=2, n_sheets=0,
                       sheet_thickness=2.0):
    """tube_volume's recipe rasterised with torch on `device`: the same tubes
    and sheets (same NumPy draws), N(0, noise_sd) noise from torch's
    generator on `device` seeded with `seed`."""
    import torch
    segs, sheets = _geometry(n, n_tubes, r_range, segments, seed, n_sheets)
    vol = torch.zeros((n, n, n), dtype=torch.float32, device=device)

    def grid(lo, hi):
        ax = [torch.arange(int(lo[k]), int(hi[k]) + 1, device=device, dtype=torch.float32) for k in range(3)]
        z, y, x = torch.meshgrid(*ax, indexing="ij")
        return torch.stack([z, y, x], dim=-1)

    for p, q, r in segs:
        lo = np.maximum(np.floor(np.minimum(p, q) - r - 1).astype(int), 0)
        hi = np.minimum(np.ceil(np.maximum(p, q) + r + 1).astype(int), [n - 1, n - 1, n - 1])
        if np.any(hi < lo):
            continue
        pts = grid(lo, hi)
        pt = torch.as_tensor(p, device=device)
        d = torch.as_tensor(q - p, device=device)
        dd = float((q - p) @ (q - p))
        t = ((pts - pt) @ d / dd).clamp(0.0, 1.0) if dd > 0 else torch.zeros(pts.shape[:3], device=device)
        dist2 = ((pts - (pt + t[..., None] * d)) ** 2).sum(-1)
        sub = vol[lo[0]:hi[0] + 1, lo[1]:hi[1] + 1, lo[2]:hi[2] + 1]
        sub[dist2 <= r * r] = 1.0
    for nrm, c, rad in sheets:
        lo = np.maximum(np.floor(c - rad).astype(int), 0)
        hi = np.minimum(np.ceil(c + rad).astype(int), n - 1)
        rel = grid(lo, hi).double() - torch.as_tensor(c, device=device)
        h = rel @ torch.as_tensor(nrm, device=device)
        inplane = (rel ** 2).sum(-1) - h * h
        m = (h.abs() <= sheet_thickness / 2) & (inplane <= rad * rad)
        vol[lo[0]:hi[0] + 1, lo[1]:hi[1] + 1, lo[2]:hi[2] + 1][m] = 1.0
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    vol += torch.randn(vol.shape, generator=g, device=device, dtype=torch.float32) * noise_sd
    return vol
