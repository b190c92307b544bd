"""Run the IBEM pipeline of the bench workload a fixed number of times, for
profilers (ncu launch lists and kernel captures); prints nothing but a
checksum.  Same workload and code path as bench.py's timed step.

    python -m inverseacoustics_gb300.profile_step [--precision mixed|fp64] [--reps 2]
        [--freqs 64] [--subdiv 3]
"""
from __future__ import annotations

import argparse

import numpy as np


def main():
    import torch

    from . import api
    from . import geometry as g

    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--freqs", type=int, default=64)
    ap.add_argument("--subdiv", type=int, default=3)
    a = ap.parse_args()
    w = g.ibem_sphere(n_freq=a.freqs, subdiv=a.subdiv)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    rng = np.random.default_rng(5)
    p = np.stack([g.add_noise(rng, g.pulsating_sphere_pressure(mics, k, 0.1, 1.0), 30.0)[None, :] for k in w.k])
    dev = torch.device("cuda:0")
    ctx = api.Context(0)
    mesh = api.Mesh(ctx, nodes, elems)
    md, kd, pd = (torch.as_tensor(np.ascontiguousarray(x), device=dev) for x in (mics, w.k, p))
    cfg = api.default_config(precision=1 if a.precision == "mixed" else 0)
    out = None
    for _ in range(a.reps):
        out = api.ibem_solve_batch(ctx, mesh, md, kd, pd, cfg)
    torch.cuda.synchronize()
    print("checksum", float(out[0].abs().sum()), "info", int(out[3].abs().sum()))


if __name__ == "__main__":
    main()
