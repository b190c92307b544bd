"""Run one of the benchmark workloads a fixed number of times, for profilers
(ncu launch lists and kernel captures); prints nothing but a checksum.  Same
workloads and code paths as bench.py's timed steps.

    python -m inverseacoustics_gb300.profile_step [--workload ibem|radiation|design|bemmodes|admm|hels]
        [--precision mixed|fp64] [--reps 2] [--freqs 64] [--subdiv 3] [--admm-iters 50]
        [--complex-modes]

ibem: the IBEM sphere pipeline (642 nodes / 1280 triangles / 120 mics).
radiation: the baffled plate (1280 elements, 192 mics): sinc R, 32 radiation
modes, ESM TSVD reconstruction (k = 36), sound power.
design: ESM array design (128 mics, 642 sources, 16 fields), forward + adjoint.
bemmodes: BEM radiation modes of the IBEM sphere, 32 modes of Re(G Z), or
with --complex-modes of G Z itself (the C++ invr()).
admm: L1 ADMM on the sphere's monopole transfer matrices (120 mics, 642
sources), epsilon = 0: all 14 continuation stages of --admm-iters iterations.
hels: the order-15 spherical-harmonic expansion on the 16 x 16 plane (256
mics), expansion matrices and Tikhonov-GCV.
"""
from __future__ import annotations

import argparse
import math

import numpy as np


def _ibem(a, dev, api, g):
    import torch
    w = g.ibem_sphere(n_freq=a.freqs, subdiv=a.subdiv)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    rng = np.random.default_rng(5)
    p = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in w.k])
    ctx = api.Context(0)
    mesh = api.Mesh(ctx, nodes, elems)
    md, kd, pd = (torch.as_tensor(np.ascontiguousarray(x), device=dev) for x in (mics, w.k, p))
    cfg = api.default_config(precision=1 if a.precision == "mixed" else 0)
    out = None
    for _ in range(a.reps):
        out = api.ibem_solve_batch(ctx, mesh, md, kd, pd, cfg)
    torch.cuda.synchronize()
    return float(out[0].abs().sum()), int(out[3].abs().sum())


def _radiation(a, dev, api, g):
    import torch
    w = g.radiation_plate(n_freq=a.freqs)
    x, area, mics = w.arrays["centres"], w.params["area"], w.arrays["mics"]
    rng = np.random.default_rng(3)
    p = np.stack([g.add_noise(rng, g.rayleigh_pressure(mics, x, area, k, w.params["vel"][f]), 30.0)[None, :]
                  for f, k in enumerate(w.k)])
    ctx = api.Context(0)
    xd, md, kd, pd = (torch.as_tensor(np.ascontiguousarray(v), device=dev) for v in (x, mics, w.k, p))
    prec = 1 if a.precision == "mixed" else 0
    cm, cs = api.default_config(precision=prec), api.default_config(method=1, tsvd_k=36, precision=prec)
    chk, info = 0.0, 0
    for _ in range(a.reps):
        R = api.sinc_resistance_batch(ctx, xd, kd, area)
        lam, modes, i1 = api.radiation_modes_batch(ctx, R, 32, cm)
        q, _, _, i2 = api.esm_solve_batch(ctx, md, xd, kd, pd, cs)
        W = api.sound_power_batch(ctx, R, q)
        torch.cuda.synchronize()
        chk = float(lam.sum() + W.sum())
        info = int(i1.abs().sum() + i2.abs().sum())
    return chk, info


def _design(a, dev, api, g):
    import torch
    w = g.esm_design(n_freq=a.freqs)
    mics, surf, q = w.arrays["mics"], w.arrays["surface"], w.params["q"]
    rng = np.random.default_rng(41)
    F, R = len(w.k), q.shape[2]
    noise = 10 ** (-30 / 20) * g.complex_normal(rng, (F, R, mics.shape[1])) * 0.05
    args = [torch.as_tensor(np.ascontiguousarray(v), device=dev) for v in
            (mics, surf, np.array([w.params["retreat"]]), w.k, np.full(F, math.log(0.05)),
             np.transpose(q, (0, 2, 1)), noise)]
    ctx = api.Context(0)
    out = None
    for _ in range(a.reps):
        out = api.esm_design_batch(ctx, *args)
    torch.cuda.synchronize()
    return float(out[0].sum()), int(out[4].abs().sum())


def _bemmodes(a, dev, api, g):
    import torch
    w = g.ibem_sphere(n_freq=a.freqs, subdiv=a.subdiv)
    ctx = api.Context(0)
    mesh = api.Mesh(ctx, w.arrays["nodes"], w.arrays["elems"])
    md, kd = (torch.as_tensor(np.ascontiguousarray(x), device=dev) for x in (w.arrays["mics"], w.k))
    cfg = api.default_config(precision=1 if a.precision == "mixed" else 0)
    out = None
    for _ in range(a.reps):
        out = api.bem_modes_batch(ctx, mesh, md, kd, 32, cfg, complex_modes=a.complex_modes)
    torch.cuda.synchronize()
    return float(out[0].sum()), int(out[4].abs().sum())


def _admm(a, dev, api, g):
    import torch
    w = g.ibem_sphere(n_freq=a.freqs, subdiv=a.subdiv)
    mics, src = w.arrays["mics"], w.arrays["nodes"] * 0.7
    ctx = api.Context(0)
    l, m, F = mics.shape[1], src.shape[1], a.freqs
    H = api.monopole_batch(ctx, torch.as_tensor(mics, device=dev), torch.as_tensor(src, device=dev),
                           torch.as_tensor(w.k, device=dev))
    H /= torch.linalg.vector_norm(H, dim=(1, 2), keepdim=True) / math.sqrt(l)
    x = torch.zeros((F, m, 1), dtype=torch.complex128, device=dev)
    x[:, [5, 77, 140, 400], 0] = torch.tensor([1.0, 0.7j, -0.5, 0.3 + 0.3j], dtype=torch.complex128, device=dev)
    p = torch.matmul(H.transpose(1, 2), x).transpose(1, 2).contiguous()
    lam = torch.full((F, 1), 0.01, dtype=torch.float64, device=dev)
    acfg = api.default_admm_config(norm=1, max_iters=a.admm_iters, rho=2.0, epsilon=0.0,
                                   precision=1 if a.precision == "mixed" else 0)
    out = None
    for _ in range(a.reps):
        out = api.admm_batch(ctx, H, p, lam, acfg)
    torch.cuda.synchronize()
    return float(out[0].abs().sum()), int(out[1].sum())


def _hels(a, dev, api, g):
    import torch
    w = g.hels_plane(n_freq=a.freqs)
    p = torch.as_tensor(g.hels_plane_pressures(w), device=dev)
    pts = torch.as_tensor(np.ascontiguousarray(g.cartesian_to_spherical(w.arrays["mics"])), device=dev)
    k = torch.as_tensor(w.k, device=dev)
    ctx = api.Context(0)
    cfg = api.default_config(precision=1 if a.precision == "mixed" else 0)
    out = None
    for _ in range(a.reps):
        out = api.hels_solve_batch(ctx, pts, w.params["order"], k, p, cfg)
    torch.cuda.synchronize()
    return float(out[0].abs().sum()), int(out[3].abs().sum())


def main():
    import torch

    from . import api
    from . import geometry as g

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="ibem", choices=["ibem", "radiation", "design", "bemmodes", "admm", "hels"])
    ap.add_argument("--admm-iters", type=int, default=50, help="ADMM: Nm (iterations per continuation stage)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--freqs", type=int, default=None)
    ap.add_argument("--subdiv", type=int, default=3)
    ap.add_argument("--complex-modes", action="store_true", help="bemmodes: modes of G Z instead of Re(G Z)")
    a = ap.parse_args()
    if a.freqs is None:
        a.freqs = {"ibem": 64, "radiation": 256, "design": 128, "bemmodes": 16, "admm": 64, "hels": 512}[a.workload]
    dev = torch.device("cuda:0")
    fn = {"ibem": _ibem, "radiation": _radiation, "design": _design, "bemmodes": _bemmodes,
          "admm": _admm, "hels": _hels}[a.workload]
    chk, info = fn(a, dev, api, g)
    print("checksum", chk, "info", info)


if __name__ == "__main__":
    main()
