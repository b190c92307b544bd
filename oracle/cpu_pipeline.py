"""Timed CPU run of the reference's IBEM inverse path (the oracle port).

ORACLE / TEST INFRASTRUCTURE ONLY: bench.py runs this as its CPU-baseline leg
and as its reference arm.  Per frequency it does what the reference's CPU
code does -- ibem() assembly and zgels solve Z = A \\ B, H = A_hs Z - B_hs
(CUDA/ibem.cuh:424-770) -- followed by csvd, GCV and Tikhonov
(MATLAB/regtools csvdG/gcvG/tikhonovG).  Frequencies run concurrently on a
thread pool (the C assembly and LAPACK release the GIL), one BLAS thread per
worker.

    python -m oracle.cpu_pipeline --freqs 16 --threads 0 [--repeat R]
prints one JSON line with the freq-solves/s of each repeat.
"""
from __future__ import annotations

import os

if "OPENBLAS_NUM_THREADS" not in os.environ:
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"

import argparse  # noqa: E402
import concurrent.futures as cf  # noqa: E402
import json  # noqa: E402
import sys  # noqa: E402
import time  # noqa: E402

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from inverseacoustics_gb300 import geometry as g  # noqa: E402
from inverseacoustics_gb300 import quadrature as Q  # noqa: E402
from oracle import ia_oracle as O  # noqa: E402


def one_frequency(nodes, elems, mics, k, p, reg, sing):
    _, H = O.ibem(nodes, elems, mics, k, reg, sing, 343.0, 1.21)
    x, lam, s = O.solve_tikhonov_gcv(H, p)
    return x, lam


def run(n_freq_sample=16, threads=0, repeat=1, n_freq_total=64):
    w = g.ibem_sphere(n_freq=n_freq_total)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    reg, sing = Q.builtin()
    rng = np.random.default_rng(99)
    idx = np.linspace(0, n_freq_total - 1, n_freq_sample).round().astype(int)
    ps = [g.add_noise(rng, g.pulsating_sphere_pressure(mics, w.k[i], 0.1, 1.0), 30.0) for i in idx]
    threads = threads or os.cpu_count() or 1
    O.clib()
    rates = []
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for _ in range(repeat):
            t0 = time.perf_counter()
            futs = [ex.submit(one_frequency, nodes, elems, mics, w.k[i], p, reg, sing) for i, p in zip(idx, ps)]
            for fu in futs:
                fu.result()
            dt = time.perf_counter() - t0
            rates.append(n_freq_sample / dt)
    return dict(rates=rates, threads=threads, sample=f"{n_freq_sample} of {n_freq_total} frequencies "
                f"(642 nodes, 1280 triangles, 120 mics), {threads} threads, 1 BLAS thread each",
                cpu=_cpu_model())


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--freqs", type=int, default=16)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--repeat", type=int, default=1)
    a = ap.parse_args()
    print(json.dumps(run(a.freqs, a.threads, a.repeat)))


if __name__ == "__main__":
    main()
