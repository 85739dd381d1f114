"""Seeded synthetic phantoms for the NLM workloads.

The reference denoises BMP test images (3DNLM/nlm.cpp:31); the workloads here use
seeded synthetic phantoms of the stated shapes instead:

* 3D: axis-aligned ellipsoids (seeded centres, radii U[4, 20] voxels, constant
  intensities U[0, 1]) painted in order on a 0.1 background, plus i.i.d.
  Gaussian noise N(0, sigma^2).
* 2D: discs and rectangles (intensities U[0, 1]) on a 0.1 background plus noise.
* Batch: 64 volumes with each dimension drawn from {32, 48, ..., 192}, their own
  phantom and sigma ~ U[0.02, 0.1], h = sigma, search radius 3 for the first
  half and 5 for the second half, patch radius 1.

All randomness comes from numpy's PCG64 generator seeded explicitly.
"""
import numpy as np


def ellipsoid_phantom(shape, n_ellipsoids=8, sigma=0.05, seed=0, radii=(4.0, 20.0),
                      background=0.1, dtype=np.float32):
    """Return (noisy, clean) volumes of shape (Z, Y, X)."""
    rng = np.random.default_rng(seed)
    Z, Y, X = shape
    clean = np.full(shape, background, np.float32)
    for _ in range(n_ellipsoids):
        c = rng.uniform(0, 1, 3) * np.array([Z, Y, X])
        r = rng.uniform(radii[0], radii[1], 3)
        val = np.float32(rng.uniform(0, 1))
        lo = np.maximum(np.floor(c - r).astype(int), 0)
        hi = np.minimum(np.ceil(c + r).astype(int) + 1, [Z, Y, X])
        if np.any(hi <= lo):
            continue
        zz = (np.arange(lo[0], hi[0]) - c[0]) / r[0]
        yy = (np.arange(lo[1], hi[1]) - c[1]) / r[1]
        xx = (np.arange(lo[2], hi[2]) - c[2]) / r[2]
        mask = zz[:, None, None] ** 2 + yy[None, :, None] ** 2 + xx[None, None, :] ** 2 <= 1.0
        sub = clean[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        sub[mask] = val
    noise = rng.standard_normal(shape, dtype=np.float32) * np.float32(sigma)
    noisy = (clean + noise).astype(dtype)
    return noisy, clean.astype(dtype)


def disc_rect_phantom(shape, n_shapes=32, sigma=0.08, seed=0, background=0.1,
                      dtype=np.float32):
    """Return (noisy, clean) images of shape (Y, X): discs and rectangles."""
    rng = np.random.default_rng(seed)
    Y, X = shape
    clean = np.full(shape, background, np.float32)
    yy = np.arange(Y)[:, None]
    xx = np.arange(X)[None, :]
    scale = min(X, Y)
    for i in range(n_shapes):
        val = np.float32(rng.uniform(0, 1))
        cy, cx = rng.uniform(0, Y), rng.uniform(0, X)
        if i % 2 == 0:
            r = rng.uniform(0.02, 0.12) * scale
            mask = (yy - cy) ** 2 + (xx - cx) ** 2 <= r * r
        else:
            hy, hx = rng.uniform(0.02, 0.12, 2) * scale
            mask = (np.abs(yy - cy) <= hy) & (np.abs(xx - cx) <= hx)
        clean[mask] = val
    noise = rng.standard_normal(shape, dtype=np.float32) * np.float32(sigma)
    return (clean + noise).astype(dtype), clean.astype(dtype)


BATCH_DIMS = tuple(range(32, 193, 16))  # {32, 48, ..., 192}: 11 values


def batch_specs(n_volumes=64, seed=1234):
    """Per-volume (shape, sigma, h, search_radius, patch_radius, phantom_seed)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_volumes):
        Z, Y, X = (int(d) for d in rng.choice(BATCH_DIMS, 3))
        sigma = float(rng.uniform(0.02, 0.1))
        sr = 3 if i < n_volumes // 2 else 5
        specs.append(dict(shape=(Z, Y, X), sigma=sigma, h=sigma, sr=sr, pr=1,
                          seed=int(rng.integers(0, 2**31 - 1))))
    return specs


def batch_volumes(specs, dtype=np.float32):
    """Noisy volumes for batch_specs(); ellipsoid count scales with volume size."""
    vols = []
    for s in specs:
        Z, Y, X = s["shape"]
        n_ell = max(4, int(8 * (Z * Y * X) / 64 ** 3) // 4 + 4)
        noisy, _ = ellipsoid_phantom(s["shape"], n_ellipsoids=n_ell, sigma=s["sigma"],
                                     seed=s["seed"], dtype=dtype)
        vols.append(noisy)
    return vols
