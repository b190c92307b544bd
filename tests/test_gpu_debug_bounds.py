"""GPU suite: the bounds-checked debug build.  libia_debug.so (compiled with
IA_DEBUG_BOUNDS) tests the main kernels' global-memory indexes against their
buffers' extents, skips a failing access and records it; run through the
mixed pipeline at small and full size (cluster QR and Jacobi, one-CTA
kernels, fused FP32 solves, tensor-core slicing, assembly) and the FP64
pipeline, it must record no failure.  The run is a child process that loads
the debug library (IA_LIBRARY) instead of libia.so."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import ctypes as C, json
import numpy as np, torch
from inverseacoustics_gb300 import api, _lib, geometry as g
dev = torch.device("cuda:0")
ctx = api.Context(0)
w = g.ibem_sphere(n_freq=64)
nodes, elems, mics = w.arrays["nodes"], w.arrays["elems"], w.arrays["mics"]
p = g.ibem_sphere_pressures(w)
mesh = api.Mesh(ctx, nodes, elems)
md = torch.as_tensor(mics, device=dev)
infos = []
for F, prec in ((4, 1), (64, 1), (4, 0)):
    kd = torch.as_tensor(np.ascontiguousarray(w.k[:F]), device=dev)
    pd = torch.as_tensor(np.ascontiguousarray(p[:F]), device=dev)
    x, lam, s, info = api.ibem_solve_batch(ctx, mesh, md, kd, pd, api.default_config(precision=prec))
    torch.cuda.synchronize()
    infos.append(int(info.abs().sum()))
en, cnt, fil, line, idx, ext = C.c_int(), C.c_ulonglong(), C.c_char_p(), C.c_int(), C.c_longlong(), C.c_longlong()
_lib.check(_lib.lib().ia_bounds_report(C.byref(en), C.byref(cnt), C.byref(fil), C.byref(line), C.byref(idx),
                                       C.byref(ext)), "ia_bounds_report")
print(json.dumps({"enabled": en.value, "count": cnt.value, "file": fil.value.decode() if fil.value else None,
                  "line": line.value, "index": idx.value, "extent": ext.value, "infos": infos,
                  "library": _lib.LIB_PATH}))
"""


def test_debug_build_reports_no_bounds_failure(cuda):
    lib = os.path.join(ROOT, "inverseacoustics_gb300", "libia_debug.so")
    assert os.path.exists(lib), "libia_debug.so not built (inverseacoustics_gb300._build.build(debug_bounds=True))"
    env = dict(os.environ, IA_LIBRARY=lib)
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    rep = json.loads(r.stdout.strip().splitlines()[-1])
    assert rep["library"] == lib
    assert rep["enabled"] == 1, rep
    assert rep["count"] == 0, rep
    assert rep["infos"] == [0, 0, 0], rep
