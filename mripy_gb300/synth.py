"""Seeded synthetic MRI workloads: trajectories, phantoms and coil maps.

Trajectories are returned in cycles (k in [-0.5, 0.5)); multiply by 2*pi for the
radian coordinates the NUFFT takes.  The phantoms and coil maps follow their own
parameterisations (no published phantom table is reproduced).

Workloads (sizes of the benchmark configurations):
  c1  2-D 128^2 image, uniform radial 128 spokes x 256 samples, 1 coil
  c2  2-D 256^2 ellipse phantom x 8 coils, golden-angle radial 402 x 512, 30 dB noise
  c3  64 frames x 12 coils of 192^2, golden-angle spokes U{5..34} per frame x 384
  c4  3-D 128^3 ellipsoid phantom x 8 coils, 20,000 centre-out spokes x 128 (Fibonacci sphere)
  c5  2-D 256^2 x 16 coils, variable-density spiral 24 x 2048, coords + N(0, 1e-3)
"""
import math

import numpy as np

GOLDEN_ANGLE = math.pi * (math.sqrt(5.0) - 1.0) / 2.0  # 111.246 degrees


def radial_2d(n_spokes, n_read, angles=None):
    """Radial spokes through the centre; angles default to pi*s/n_spokes."""
    if angles is None:
        angles = math.pi * np.arange(n_spokes) / n_spokes
    r = (np.arange(n_read) - n_read / 2.0) / n_read          # [-0.5, 0.5)
    kx = np.cos(angles)[:, None] * r[None, :]
    ky = np.sin(angles)[:, None] * r[None, :]
    return kx.reshape(-1), ky.reshape(-1)


def golden_radial_2d(n_spokes, n_read, start=0):
    return radial_2d(n_spokes, n_read, angles=GOLDEN_ANGLE * (start + np.arange(n_spokes)))


def fibonacci_sphere(n):
    i = np.arange(n) + 0.5
    z = 1.0 - 2.0 * i / n
    phi = math.pi * (3.0 - math.sqrt(5.0)) * i
    r = np.sqrt(1.0 - z * z)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=0)  # (3, n)


def centre_out_radial_3d(n_spokes, n_read):
    d = fibonacci_sphere(n_spokes)                            # (3, S)
    r = 0.5 * np.arange(n_read) / n_read                      # [0, 0.5)
    k = d[:, :, None] * r[None, None, :]
    return k[0].reshape(-1), k[1].reshape(-1), k[2].reshape(-1)


def vd_spiral_2d(n_interleaves, n_read, turns=16, alpha=2.0):
    """Variable-density Archimedean-type spiral: radius grows as (t^alpha) so the
    centre is sampled densely; k_max 0.5 (just inside)."""
    t = np.arange(n_read) / n_read
    r = 0.4999 * t ** alpha
    theta = 2.0 * math.pi * turns * t
    out_x, out_y = [], []
    for i in range(n_interleaves):
        a = theta + 2.0 * math.pi * i / n_interleaves
        out_x.append(r * np.cos(a))
        out_y.append(r * np.sin(a))
    return np.concatenate(out_x), np.concatenate(out_y)


def ellipse_phantom(n, rng=None, n_ellipses=10):
    """Sum of seeded ellipses with smooth-ish edges; complex with a mild phase."""
    rng = np.random.default_rng(0) if rng is None else rng
    y, x = np.mgrid[-1:1:complex(0, n), -1:1:complex(0, n)]
    img = np.zeros((n, n))
    img += 1.0 * (((x / 0.72) ** 2 + (y / 0.92) ** 2) <= 1.0)
    img -= 0.7 * (((x / 0.66) ** 2 + (y / 0.86) ** 2) <= 1.0)
    for _ in range(n_ellipses):
        cx, cy = rng.uniform(-0.45, 0.45, 2)
        a, b = rng.uniform(0.05, 0.3, 2)
        th = rng.uniform(0, math.pi)
        xr = (x - cx) * math.cos(th) + (y - cy) * math.sin(th)
        yr = -(x - cx) * math.sin(th) + (y - cy) * math.cos(th)
        img += rng.uniform(-0.2, 0.3) * ((xr / a) ** 2 + (yr / b) ** 2 <= 1.0)
    phase = np.exp(1j * 0.3 * math.pi * (x + 0.5 * y))
    return (img * phase).astype(np.complex64)


def ellipsoid_phantom(n, rng=None, n_ellipsoids=8):
    rng = np.random.default_rng(0) if rng is None else rng
    z, y, x = np.mgrid[-1:1:complex(0, n), -1:1:complex(0, n), -1:1:complex(0, n)]
    img = 1.0 * (((x / 0.7) ** 2 + (y / 0.9) ** 2 + (z / 0.8) ** 2) <= 1.0)
    img -= 0.6 * (((x / 0.64) ** 2 + (y / 0.84) ** 2 + (z / 0.74) ** 2) <= 1.0)
    for _ in range(n_ellipsoids):
        c = rng.uniform(-0.4, 0.4, 3)
        ax = rng.uniform(0.06, 0.3, 3)
        img += rng.uniform(-0.2, 0.3) * ((((x - c[0]) / ax[0]) ** 2 + ((y - c[1]) / ax[1]) ** 2 +
                                           ((z - c[2]) / ax[2]) ** 2) <= 1.0)
    return img.astype(np.complex64)


def coil_maps(shape, n_coil, rng=None):
    """Gaussian-windowed complex exponentials around a ring of coil centres, normalised so
    that sum_c |S_c|^2 = 1 at every pixel.  Returns (*shape, n_coil) complex64."""
    rng = np.random.default_rng(1) if rng is None else rng
    dim = len(shape)
    axes = np.meshgrid(*[np.linspace(-1, 1, s) for s in shape], indexing="ij")
    maps = []
    for c in range(n_coil):
        ang = 2 * math.pi * c / n_coil
        centre = np.zeros(dim)
        centre[0], centre[1] = 1.2 * math.cos(ang), 1.2 * math.sin(ang)
        if dim == 3:
            centre[2] = 0.6 * ((c % 2) * 2 - 1)
        d2 = sum((a - centre[i]) ** 2 for i, a in enumerate(axes))
        win = np.exp(-d2 / 1.5)
        freq = rng.normal(0, 1.0, dim)
        ph = np.exp(1j * sum(freq[i] * a for i, a in enumerate(axes)))
        maps.append(win * ph)
    S = np.stack(maps, axis=-1)
    S /= np.sqrt(np.sum(np.abs(S) ** 2, axis=-1, keepdims=True))
    return S.astype(np.complex64)


def radial_dcf_2d(kx, ky):
    """Ram-Lak density compensation |k| (with a floor at the centre)."""
    r = np.sqrt(kx ** 2 + ky ** 2)
    return np.maximum(r, 0.5 / len(kx) ** 0.5).astype(np.float32)


# ---------------------------------------------------------------- configurations

def config1(seed=0):
    rng = np.random.default_rng(seed)
    img = (rng.standard_normal((128, 128)) + 1j * rng.standard_normal((128, 128))).astype(np.complex64)
    kx, ky = radial_2d(128, 256)
    return {"image": img, "k": (kx, ky), "shape": (128, 128), "eps": 5e-6}


def config2(seed=0, n_coil=8, snr_db=30.0):
    rng = np.random.default_rng(seed)
    x = ellipse_phantom(256, rng)
    S = coil_maps((256, 256), n_coil, rng)
    kx, ky = golden_radial_2d(402, 512)
    return {"image": x, "sens": S, "k": (kx, ky), "shape": (256, 256), "eps": 5e-6, "snr_db": snr_db,
            "rng": rng}


def config3(seed=0, n_frames=64, n_coil=12, n_read=384):
    rng = np.random.default_rng(seed)
    spokes = rng.integers(5, 35, size=n_frames)                 # U{5..34}
    kxs, kys, offsets = [], [], [0]
    start = 0
    for f in range(n_frames):
        kx, ky = golden_radial_2d(int(spokes[f]), n_read, start=start)
        start += int(spokes[f])
        kxs.append(kx)
        kys.append(ky)
        offsets.append(offsets[-1] + len(kx))
    img = (rng.standard_normal((n_frames, 192, 192, n_coil)) +
           1j * rng.standard_normal((n_frames, 192, 192, n_coil))).astype(np.complex64)
    return {"image": img, "k": (np.concatenate(kxs), np.concatenate(kys)), "offsets": offsets,
            "shape": (192, 192), "eps": 5e-6, "spokes": spokes}


def config4(seed=0, n=128, n_coil=8, n_spokes=20000, n_read=128):
    rng = np.random.default_rng(seed)
    x = ellipsoid_phantom(n, rng)
    S = coil_maps((n, n, n), n_coil, rng)
    k = centre_out_radial_3d(n_spokes, n_read)
    return {"image": x, "sens": S, "k": k, "shape": (n, n, n), "eps": 5e-6}


def config5(seed=0, n_coil=16):
    rng = np.random.default_rng(seed)
    img = (rng.standard_normal((256, 256, n_coil)) + 1j * rng.standard_normal((256, 256, n_coil))).astype(
        np.complex64)
    kx, ky = vd_spiral_2d(24, 2048)
    dkx = rng.normal(0, 1e-3, kx.shape)
    dky = rng.normal(0, 1e-3, ky.shape)
    return {"image": img, "k": (kx, ky), "k_perturbed": (kx + dkx, ky + dky), "shape": (256, 256), "eps": 5e-6}
