"""Meshes, microphone arrays and seeded synthetic problems for the five
workloads of the inverse pipeline.

Layout follows the reference's C arrays: coordinates are structure-of-arrays,
``r[i], r[i+n], r[i+2n]`` (CUDA/esm.cuh:9, CUDA/ibem.cuh:10), connectivity is
``e_n[i + j*n]`` with 0-based node indices (CUDA/ibem.cuh:10).  Here those
arrays are numpy ``(3, n)`` float64 / int32 arrays whose C-order ravel() is the
reference layout.

Sign convention: the reference's outgoing wave is exp(+ikr)
(CUDA/esm.cuh:16, CUDA/ibem.cuh:27) with h_n = j_n + i y_n
(CUDA/hels.cuh:109).  All synthetic fields here use that convention.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

C_DEFAULT = 343.0
RHO_DEFAULT = 1.21


# ---------------------------------------------------------------------------
# meshes
# ---------------------------------------------------------------------------
def icosphere(subdiv: int, radius: float = 1.0):
    """Icosahedron refined ``subdiv`` times by edge midpoints projected to the
    sphere.  Returns ``(nodes (3, m) float64, elems (3, n) int32)`` with every
    triangle ordered so the reference's element normal
    ``(v0 - v2) x (v1 - v2)`` (CUDA/ibem.cuh:502-510) points outward.
    Node counts: 12, 42, 162, 642, 2562 for subdiv 0..4."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                p = verts[a] + verts[b]
                verts.append(p / np.linalg.norm(p))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for (a, b, c) in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts).T * radius
    F = np.array(faces, dtype=np.int64)
    # orient outward for the reference normal (v0 - v2) x (v1 - v2)
    p0, p1, p2 = V[:, F[:, 0]], V[:, F[:, 1]], V[:, F[:, 2]]
    nrm = np.cross((p0 - p2).T, (p1 - p2).T).T
    cen = (p0 + p1 + p2) / 3.0
    flip = np.einsum("ij,ij->j", nrm, cen) < 0
    F[flip, 0], F[flip, 1] = F[flip, 1].copy(), F[flip, 0].copy()
    return np.ascontiguousarray(V), np.ascontiguousarray(F.T.astype(np.int32))


def plate_grid(lx: float, ly: float, nx: int, ny: int):
    """Centres (3, nx*ny) and the common area of a baffled rectangular plate
    cut into nx x ny equal rectangles, plate centred on the origin in z=0."""
    dx, dy = lx / nx, ly / ny
    xs = -lx / 2 + dx * (np.arange(nx) + 0.5)
    ys = -ly / 2 + dy * (np.arange(ny) + 0.5)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    P = np.stack([X.ravel(), Y.ravel(), np.zeros(nx * ny)])
    return np.ascontiguousarray(P), dx * dy


def rayleigh_pressure(P, centres, area, k, vel, c=C_DEFAULT, rho=RHO_DEFAULT):
    """Pressure at points P (3, l) radiated by a baffled plate of elements of
    equal area at centres (3, n) with normal velocity vel (n,), by the
    midpoint-rule Rayleigh integral p = -i omega rho/(2 pi) sum A v e^{ikR}/R.
    In the monopole form p = G q, G = e^{ikR}/(4 pi R), the equivalent source
    strengths are q = -2 i omega rho A v."""
    R = np.sqrt(((P.T[:, None, :] - centres.T[None, :, :]) ** 2).sum(-1))
    G = np.exp(1j * k * R) / (4 * np.pi * R)
    return G @ (-2j * k * c * rho * area * np.asarray(vel))


def planar_array(nx: int, ny: int, pitch: float, z: float):
    """nx x ny microphones on a grid of the given pitch, centred on the z axis."""
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.ascontiguousarray(np.stack([X.ravel(), Y.ravel(), np.full(nx * ny, z)]))


def hemisphere_array(rng: np.random.Generator, count: int, radius: float):
    """``count`` microphones at uniform-random directions on the upper
    hemisphere (z >= 0) of the given radius."""
    v = rng.normal(size=(3, count))
    v /= np.linalg.norm(v, axis=0)
    v[2] = np.abs(v[2])
    return np.ascontiguousarray(v * radius)


def cartesian_to_spherical(P: np.ndarray) -> np.ndarray:
    """(az, el, r) rows as in the reference's cartesian_2_spherical
    (CUDA/utils.cuh:414-427): az in [0, 2pi), el = atan2(rho_xy, z) with the
    reference's -2pi shift where x < 0 (only cos(el) and sin^2(el) are used
    downstream, so the shift does not change any matrix)."""
    x, y, z = P
    xy = x * x + y * y
    r = np.sqrt(xy + z * z)
    az = np.arctan2(y, x)
    az = np.where(y < 0, az + 2 * np.pi, az)
    el = np.arctan2(np.sqrt(xy), z)
    el = np.where(x < 0, el - 2 * np.pi, el)
    return np.ascontiguousarray(np.stack([az, el, r]))


# ---------------------------------------------------------------------------
# analytic fields (exp(+ikr) convention, velocity u_r = dp/dr / (i rho c k))
# ---------------------------------------------------------------------------
def _h0(x):
    return -1j * np.exp(1j * x) / x


def _h1(x):
    return -np.exp(1j * x) * (x + 1j) / (x * x)


def _dh1(x):
    return _h0(x) - 2.0 * _h1(x) / x


def pulsating_sphere_pressure(P, k, a, u, c=C_DEFAULT, rho=RHO_DEFAULT):
    """Pressure of a sphere of radius a pulsating with normal velocity u, at
    points P (3, n) -- the reference's analytic KAT (CUDA/utils.cuh:384-412)."""
    r = np.linalg.norm(P, axis=0)
    return (a / r) * rho * c * u * ((1j * k * a) / ((1j * k * a) - 1)) * np.exp(1j * k * (r - a))


def oscillating_sphere_pressure(P, k, a, u, c=C_DEFAULT, rho=RHO_DEFAULT):
    """Pressure of a rigid sphere of radius a oscillating along z with normal
    velocity u*cos(theta): p = i rho c u h1(kr)/h1'(ka) cos(theta)."""
    r = np.linalg.norm(P, axis=0)
    cos_t = P[2] / r
    return 1j * rho * c * u * _h1(k * r) / _dh1(k * a) * cos_t


def add_noise(rng, p, snr_db):
    """Complex white Gaussian noise at the given SNR (per-vector power)."""
    p = np.asarray(p)
    sig = np.sqrt(np.mean(np.abs(p) ** 2, axis=-1, keepdims=True))
    sigma = sig * 10.0 ** (-snr_db / 20.0)
    nz = (rng.normal(size=p.shape) + 1j * rng.normal(size=p.shape)) / np.sqrt(2.0)
    return p + sigma * nz


def complex_normal(rng, shape):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)) / np.sqrt(2.0)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
@dataclass
class Workload:
    name: str
    kind: str                    # "esm" | "ibem" | "hels" | "sinc" | "esm_design"
    k: np.ndarray                # wavenumbers (F,)
    c: float = C_DEFAULT
    rho: float = RHO_DEFAULT
    arrays: dict = field(default_factory=dict)
    params: dict = field(default_factory=dict)


def esm_single(seed: int = 0) -> Workload:
    """ESM, single frequency: 8x8 mics (0.03 m pitch) at z=0.10 m, 162
    monopoles on an icosphere of radius 0.05 m, f=1000 Hz, 30 dB SNR,
    Tikhonov-GCV over 200 log-spaced lambda in [1e-8, 1e2]."""
    rng = np.random.default_rng(seed)
    mics = planar_array(8, 8, 0.03, 0.10)
    src, _ = icosphere(2, 0.05)
    f = np.array([1000.0])
    k = 2 * np.pi * f / C_DEFAULT
    return Workload("esm_162x64_f1", "esm", k, arrays=dict(mics=mics, sources=src),
                    params=dict(snr_db=30.0, lam_grid=(1e-8, 1e2, 200), rng=rng))


def ibem_sphere(seed: int = 1, n_freq: int = 64, subdiv: int = 3) -> Workload:
    """IBEM on a sphere of radius 0.10 m (icosphere subdiv 3: 642 nodes, 1280
    triangles), 120 mics at uniform-random directions on a hemisphere of
    radius 0.30 m, n_freq frequencies 100-2000 Hz, pulsating + oscillating
    sphere with seeded complex amplitudes, 30 dB SNR."""
    rng = np.random.default_rng(seed)
    nodes, elems = icosphere(subdiv, 0.10)
    mics = hemisphere_array(rng, 120, 0.30)
    f = np.linspace(100.0, 2000.0, n_freq)
    k = 2 * np.pi * f / C_DEFAULT
    amp = complex_normal(rng, (n_freq, 2))
    return Workload(f"ibem_sphere_{nodes.shape[1]}n_{elems.shape[1]}e_120mic_F{n_freq}", "ibem", k,
                    arrays=dict(nodes=nodes, elems=elems, mics=mics),
                    params=dict(radius=0.10, amp=amp, snr_db=30.0, rng=rng))


def ibem_sphere_pressures(w: Workload) -> np.ndarray:
    """Measured pressures (F, 1, 120) of the sphere workload: pulsating plus
    oscillating sphere fields with the workload's seeded complex amplitudes,
    plus noise at its SNR.  Draws the noise from the workload's generator, so
    call it once per workload object."""
    mics, amp, rng = w.arrays["mics"], w.params["amp"], w.params["rng"]
    a, snr = w.params["radius"], w.params["snr_db"]
    return np.stack([
        add_noise(rng, amp[f, 0] * pulsating_sphere_pressure(mics, w.k[f], a, 1.0) +
                  amp[f, 1] * oscillating_sphere_pressure(mics, w.k[f], a, 1.0), snr)[None, :]
        for f in range(len(w.k))])


def hels_plane(seed: int = 2, n_freq: int = 512, order: int = 15) -> Workload:
    """HELS, order 15 (256 terms), 16x16 mics (0.025 m pitch) at z=0.15 m, 40
    seeded monopoles inside r < 0.08 m, n_freq frequencies 50-3000 Hz, 25 dB."""
    rng = np.random.default_rng(seed)
    mics = planar_array(16, 16, 0.025, 0.15)
    d = rng.normal(size=(3, 40))
    d /= np.linalg.norm(d, axis=0)
    srcs = d * 0.08 * rng.uniform(0, 1, size=40) ** (1 / 3)
    f = np.linspace(50.0, 3000.0, n_freq)
    k = 2 * np.pi * f / C_DEFAULT
    q = complex_normal(rng, (n_freq, 40))
    return Workload(f"hels_N{order}_256mic_F{n_freq}", "hels", k,
                    arrays=dict(mics=mics, monopoles=np.ascontiguousarray(srcs)),
                    params=dict(order=order, q=q, snr_db=25.0, rng=rng))


def monopole_field(P, src, k, q):
    """Free-field pressure exp(ikr)/(4 pi r) (the reference's sign) at points P
    (3, l) of monopoles at src (3, s) with complex strengths q (s,)."""
    r = np.linalg.norm(P[:, :, None] - src[:, None, :], axis=0)
    return (np.exp(1j * k * r) / (4 * np.pi * r)) @ q


def hels_plane_pressures(w: Workload) -> np.ndarray:
    """Measured pressures (F, 1, 256) of the HELS workload: the 40 monopoles
    with their seeded strengths, plus noise at the workload's SNR.  Draws the
    noise from the workload's generator, so call it once per workload object."""
    mics, srcs, q, rng = w.arrays["mics"], w.arrays["monopoles"], w.params["q"], w.params["rng"]
    return np.stack([add_noise(rng, monopole_field(mics, srcs, w.k[f], q[f]), w.params["snr_db"])[None, :]
                     for f in range(len(w.k))])


def radiation_plate(seed: int = 3, n_freq: int = 256) -> Workload:
    """Baffled 0.5 x 0.4 m plate cut 40 x 32 (1280 elements), sinc resistance
    matrix, 256 frequencies 20-2000 Hz, first 20 simply-supported modes with
    seeded complex amplitudes, 192 mics at 0.05 m standoff."""
    rng = np.random.default_rng(seed)
    centres, area = plate_grid(0.5, 0.4, 40, 32)
    mics = planar_array(16, 12, 0.5 / 16, 0.05)
    f = np.linspace(20.0, 2000.0, n_freq)
    k = 2 * np.pi * f / C_DEFAULT
    modes = []
    for mx in range(1, 8):
        for my in range(1, 8):
            modes.append((mx, my, (mx / 0.5) ** 2 + (my / 0.4) ** 2))
    modes = sorted(modes, key=lambda t: t[2])[:20]
    x = centres[0] + 0.25
    y = centres[1] + 0.20
    shapes = np.stack([np.sin(mx * np.pi * x / 0.5) * np.sin(my * np.pi * y / 0.4) for mx, my, _ in modes])
    amp = complex_normal(rng, (n_freq, 20))
    vel = amp @ shapes
    return Workload(f"sinc_plate_1280el_F{n_freq}", "sinc", k, arrays=dict(centres=centres, mics=mics),
                    params=dict(area=area, vel=vel, rng=rng))


def esm_design(seed: int = 4, n_freq: int = 128) -> Workload:
    """Differentiable ESM design: 128 mics seeded on a 0.4 x 0.4 m plane at
    z=0.12 m, 642 sources on an icosphere (radius 0.10 m) retreated by 0.04 m,
    128 frequencies 200-4000 Hz, 16 seeded complex source fields."""
    rng = np.random.default_rng(seed)
    mics = np.stack([rng.uniform(-0.2, 0.2, 128), rng.uniform(-0.2, 0.2, 128), np.full(128, 0.12)])
    surf, _ = icosphere(3, 0.10)
    f = np.linspace(200.0, 4000.0, n_freq)
    k = 2 * np.pi * f / C_DEFAULT
    q = complex_normal(rng, (n_freq, 642, 16))
    return Workload(f"esm_design_128mic_642src_F{n_freq}", "esm_design", k,
                    arrays=dict(mics=np.ascontiguousarray(mics), surface=surf),
                    params=dict(retreat=0.04, q=q, rng=rng))
