"""Timed CPU run of the reference's IBEM inverse path (the oracle port).

ORACLE / TEST INFRASTRUCTURE ONLY: bench.py runs this as its CPU-baseline leg
and as its reference arm.  Per frequency it does what the reference's CPU
code does -- ibem() assembly and zgels solve Z = A \\ B, H = A_hs Z - B_hs
(CUDA/ibem.cuh:424-770) -- followed by csvd, GCV and Tikhonov
(MATLAB/regtools csvdG/gcvG/tikhonovG).  Frequencies run concurrently on a
thread pool (the C assembly and LAPACK release the GIL), one BLAS thread per
worker.

    python -m oracle.cpu_pipeline --freqs 16 --threads 0 [--repeat R] [--warmup W]
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


def oracle_ibem_bin(args):
    """One bin of the IBEM path in the oracle: transfer matrix (C assembly,
    zgels-equivalent solve, H GEMM) and the Tikhonov-GCV solve; (x, lam, s)."""
    nodes, elems, mics, k, p = args
    reg, sing = Q.builtin()
    H = O.ibem_transfer(nodes, elems, mics, k, reg, sing, 343.0, 1.21)
    return O.solve_tikhonov_gcv(H, p)


def oracle_hels_bin(args):
    """One bin of the HELS path in the oracle: h_n Y_n^m at the points, then the
    Tikhonov-GCV solve; (x, lam, s)."""
    pts, k, order, p = args
    _, He, _ = O.hels(pts, pts, k, order, 343.0, 1.21)
    return O.solve_tikhonov_gcv(He, p)


def map_bins(fn, items, workers=0):
    """fn over items on a spawn process pool, one BLAS thread per worker (the
    children read the environment set here when they import numpy)."""
    import multiprocessing as mp
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    workers = workers or os.cpu_count() or 1
    with mp.get_context("spawn").Pool(min(workers, len(items))) as pool:
        return pool.map(fn, items, chunksize=1)


def run(n_freq_sample=16, threads=0, repeat=1, n_freq_total=64, warmup=0):
    w = g.ibem_sphere(n_freq=n_freq_total)
    nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
    reg, sing = Q.builtin()
    p_all = g.ibem_sphere_pressures(w)          # the GPU arm's inputs, bit for bit
    idx = np.linspace(0, n_freq_total - 1, n_freq_sample).round().astype(int)
    ps = [p_all[i, 0] for i in idx]
    threads = threads or os.cpu_count() or 1
    O.clib()
    rates = []
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for _ in range(warmup):
            for fu in [ex.submit(one_frequency, nodes, elems, mics, w.k[i], p, reg, sing) for i, p in zip(idx, ps)]:
                fu.result()
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
    ap.add_argument("--warmup", type=int, default=0)
    a = ap.parse_args()
    print(json.dumps(run(a.freqs, a.threads, a.repeat, warmup=a.warmup)))


if __name__ == "__main__":
    main()
