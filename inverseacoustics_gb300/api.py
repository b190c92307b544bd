"""Python mirror of the reference's call surface, over libia.so.

Host functions (numpy in, numpy out) keep the reference's names and argument
order: ``esm`` (CUDA/esm.cuh:112), ``ibem`` (CUDA/ibem.cuh:424), ``hels``
(CUDA/hels.cuh:222), ``csvd`` / ``tsvd`` (CUDA/tsvd.cuh:10,122),
``to_pressure`` / ``to_velocity`` / ``sound_power`` (CUDA/utils.cuh:199-289).
Point sets are (3, n) arrays whose C-order ravel is the reference's SoA
layout; matrices come back as 2-D column-major-equivalent numpy arrays.

Batched functions take torch CUDA tensors (complex128 / float64 / int32,
contiguous) and run on a :class:`Context` stream; they are the GB300 path.
Every call goes through the CUDA library; a failing status raises IAError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import IA_OK, IAError, check, default_admm_config, default_config  # noqa: F401

_P = C.c_void_p


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _c128(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def _take(ptr: C.c_void_p, count: int, dtype=np.complex128):
    L = _lib.lib()
    item = np.dtype(dtype).itemsize
    buf = (C.c_char * (max(count, 1) * item)).from_address(ptr.value)
    out = np.frombuffer(buf, dtype=dtype, count=count).copy()
    L.ia_free(ptr)
    return out


def _cfg(cfg, c, rho):
    if cfg is None:
        cfg = default_config()
    if c is not None:
        cfg.c = c
    if rho is not None:
        cfg.rho = rho
    return cfg


# ---------------------------------------------------------------- host layer
def esm(r_ms, r_lh, k, r_i, c=None, rho=None, cfg=None):
    """(Me m x m, He l x m) -- esm() CUDA/esm.cuh:112."""
    L = _lib.lib()
    r_ms, r_lh = _f64(r_ms).ravel(), _f64(r_lh).ravel()
    m, l = r_ms.size // 3, r_lh.size // 3
    cfg = _cfg(cfg, c, rho)
    me, h = _P(), _P()
    check(L.ia_esm(m, l, r_ms.ctypes.data, r_lh.ctypes.data, C.byref(me), C.byref(h), float(k), float(r_i),
                   C.byref(cfg)), "ia_esm")
    return _take(me, m * m).reshape(m, m, order="F"), _take(h, l * m).reshape(l, m, order="F")


def rules_struct(regular, singular):
    """ia_rules from (nq, 3) regular and (3, nqs, 3) singular (xi1, xi2, w) rows.
    Returns (struct, keepalive)."""
    reg = np.ascontiguousarray(np.asarray(regular, dtype=np.float64).T).ravel()
    sg = np.asarray(singular, dtype=np.float64)
    sing = np.ascontiguousarray(np.concatenate([sg[p].T.ravel() for p in range(3)]))
    r = _lib.Rules(reg.size // 3, reg.ctypes.data, sing.size // 9, sing.ctypes.data)
    return r, (reg, sing)


def ibem(r_ms, e_n, r_lh, k, n_ch=0, cp=None, rules=None, c=None, rho=None, cfg=None):
    """(Z m x m, H l x m) -- ibem() CUDA/ibem.cuh:424.  ``rules`` is
    (regular (nq,3), singular (3,nqs,3)) or None for the built-in rules."""
    L = _lib.lib()
    r_ms, r_lh = _f64(r_ms).ravel(), _f64(r_lh).ravel()
    e = np.ascontiguousarray(np.asarray(e_n, dtype=np.int32)).ravel()
    m, l, n = r_ms.size // 3, r_lh.size // 3, e.size // 3
    cpa = _f64(cp).ravel() if n_ch else np.zeros(3)
    cfg = _cfg(cfg, c, rho)
    keep = None
    rp = None
    if rules is not None:
        rs, keep = rules_struct(*rules)
        rp = C.byref(rs)
    me, h = _P(), _P()
    check(L.ia_ibem(m, l, n, r_ms.ctypes.data, e.ctypes.data, r_lh.ctypes.data, C.byref(me), C.byref(h), float(k),
                    int(n_ch), cpa.ctypes.data, rp, C.byref(cfg)), "ia_ibem")
    del keep
    return _take(me, m * m).reshape(m, m, order="F"), _take(h, l * m).reshape(l, m, order="F")


def invr(r_ms, e_n, r_lh, k, n_am, n_ch=0, cp=None, rules=None, c=None, rho=None, cfg=None):
    """(m_e = Z q_e m x n_am, h = H q_e l x n_am, q_e m x n_am) -- invr()
    CUDA/invr.cuh:457; q_e the leading left singular vectors of G Z."""
    L = _lib.lib()
    r_ms, r_lh = _f64(r_ms).ravel(), _f64(r_lh).ravel()
    e = np.ascontiguousarray(np.asarray(e_n, dtype=np.int32)).ravel()
    m, l, n = r_ms.size // 3, r_lh.size // 3, e.size // 3
    cpa = _f64(cp).ravel() if n_ch else np.zeros(3)
    cfg = _cfg(cfg, c, rho)
    keep = None
    rp = None
    if rules is not None:
        rs, keep = rules_struct(*rules)
        rp = C.byref(rs)
    me, h, qe = _P(), _P(), _P()
    check(L.ia_invr(m, l, n, r_ms.ctypes.data, e.ctypes.data, r_lh.ctypes.data, C.byref(me), C.byref(h),
                    C.byref(qe), float(k), int(n_ch), cpa.ctypes.data, int(n_am), rp, C.byref(cfg)), "ia_invr")
    del keep
    return (_take(me, m * n_am).reshape(m, n_am, order="F"), _take(h, l * n_am).reshape(l, n_am, order="F"),
            _take(qe, m * n_am).reshape(m, n_am, order="F"))


def hels(r_ms_s, r_lh_s, k, n_sh, c=None, rho=None, cfg=None):
    """(Me m x nt, He l x nt, Qe m x nt) -- hels() CUDA/hels.cuh:222."""
    L = _lib.lib()
    a, b = _f64(r_ms_s).ravel(), _f64(r_lh_s).ravel()
    m, l = a.size // 3, b.size // 3
    nt = (n_sh + 1) ** 2
    cfg = _cfg(cfg, c, rho)
    me, h, qe = _P(), _P(), _P()
    check(L.ia_hels(m, l, a.ctypes.data, b.ctypes.data, C.byref(me), C.byref(h), C.byref(qe), float(k), int(n_sh),
                    C.byref(cfg)), "ia_hels")
    return (_take(me, m * nt).reshape(m, nt, order="F"), _take(h, l * nt).reshape(l, nt, order="F"),
            _take(qe, m * nt).reshape(m, nt, order="F"))


def csvd(A):
    """(U m x p, s p, V n x p) -- csvd() CUDA/tsvd.cuh:10."""
    L = _lib.lib()
    A = np.asarray(A, dtype=np.complex128)
    m, n = A.shape
    p = min(m, n)
    a = np.asfortranarray(A)
    u, s, v = _P(), _P(), _P()
    check(L.ia_csvd(m, n, a.ctypes.data, C.byref(u), C.byref(s), C.byref(v)), "ia_csvd")
    return (_take(u, m * p).reshape(m, p, order="F"), _take(s, p, np.float64),
            _take(v, n * p).reshape(n, p, order="F"))


def tsvd(U, s, V, b, k):
    """x_k -- tsvd() CUDA/tsvd.cuh:122; raises IAError for k outside [1, p]."""
    L = _lib.lib()
    U = np.asfortranarray(np.asarray(U, dtype=np.complex128))
    V = np.asfortranarray(np.asarray(V, dtype=np.complex128))
    s = _f64(s)
    b = _c128(b)
    m, p = U.shape
    n = V.shape[0]
    x = _P()
    check(L.ia_tsvd(m, n, p, int(k), U.ctypes.data, s.ctypes.data, V.ctypes.data, b.ctypes.data, C.byref(x)),
          "ia_tsvd")
    return _take(x, n)


def to_pressure(Me, x):
    L = _lib.lib()
    Me = np.asfortranarray(np.asarray(Me, dtype=np.complex128))
    x = _c128(x)
    m, n = Me.shape
    out = _P()
    check(L.ia_to_pressure(m, n, Me.ctypes.data, x.ctypes.data, C.byref(out)), "ia_to_pressure")
    return _take(out, m)


def to_velocity(Qe, x):
    L = _lib.lib()
    Qe = np.asfortranarray(np.asarray(Qe, dtype=np.complex128))
    x = _c128(x)
    m, n = Qe.shape
    out = _P()
    check(L.ia_to_velocity(m, n, Qe.ctypes.data, x.ctypes.data, C.byref(out)), "ia_to_velocity")
    return _take(out, m)


def sound_power(p, v, s):
    L = _lib.lib()
    p, v = _c128(p), _c128(v)
    w = C.c_double()
    check(L.ia_sound_power(p.size, p.ctypes.data, v.ctypes.data, C.byref(w), float(s)), "ia_sound_power")
    return w.value


def read_msh(path, k, t=0.0):
    """gmsh v2.2 mesh -- geometry() CUDA/utils.cuh:291.  Returns (nodes (3, m),
    field points (3, m) = nodes (1 + 2 pi t / k), triangles (3, n) int32)."""
    L = _lib.lib()
    rm, rl, en = _P(), _P(), _P()
    m, l, n = C.c_int(), C.c_int(), C.c_int()
    check(L.ia_read_msh(str(path).encode(), float(k), float(t), C.byref(rm), C.byref(rl), C.byref(en), C.byref(m),
                        C.byref(l), C.byref(n)), "ia_read_msh")
    nodes = _take(rm, 3 * m.value, np.float64).reshape(3, m.value)
    field = _take(rl, 3 * l.value, np.float64).reshape(3, l.value)
    elems = _take(en, 3 * n.value, np.int32).reshape(3, n.value)
    return nodes, field, elems


# ------------------------------------------------------------- device layer
def _dptr(t, dtype=None):
    import torch
    if t is None:
        return None
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("device entry points take CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {t.dtype}")
    return t.data_ptr()


class Context:
    """An ia_context bound to a CUDA stream (default: torch's current stream)."""

    def __init__(self, device: int = 0, stream=None):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(device)
        self.stream = stream
        self._h = _P()
        check(_lib.lib().ia_create(C.byref(self._h), int(device), _P(stream.cuda_stream)), "ia_create")

    @property
    def handle(self):
        return self._h

    def launches(self) -> int:
        return int(_lib.lib().ia_launch_count(self._h))

    def synchronize(self):
        check(_lib.lib().ia_synchronize(self._h), "ia_synchronize")

    def capture(self, fn):
        """Record fn() (batched calls on this context) into a CUDA graph.
        Run fn once uncaptured first so the workspace is sized; the stream
        must be a created stream, e.g. torch.cuda.Stream()."""
        L = _lib.lib()
        check(L.ia_capture_begin(self._h), "ia_capture_begin")
        g = _P()
        try:
            fn()
        except BaseException:
            if L.ia_capture_end(self._h, C.byref(g)) == IA_OK:
                L.ia_graph_destroy(g)
            raise
        check(L.ia_capture_end(self._h, C.byref(g)), "ia_capture_end")
        return Graph(g)

    def close(self):
        if self._h:
            _lib.lib().ia_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Graph:
    """A captured sequence of batched calls (ia_graph)."""

    def __init__(self, h):
        self._h = h

    def launch(self):
        check(_lib.lib().ia_graph_launch(self._h), "ia_graph_launch")

    def kernel_count(self) -> int:
        return int(_lib.lib().ia_graph_kernel_count(self._h))

    def close(self):
        if self._h:
            _lib.lib().ia_graph_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mesh:
    """A triangle mesh uploaded with its quadrature rules (ia_mesh_create)."""

    def __init__(self, ctx: Context, nodes, elems, rules=None):
        self.ctx = ctx
        nodes = _f64(nodes).ravel()
        elems = np.ascontiguousarray(np.asarray(elems, dtype=np.int32)).ravel()
        self.m, self.n = nodes.size // 3, elems.size // 3
        rp = None
        keep = None
        if rules is not None:
            rs, keep = rules_struct(*rules)
            rp = C.byref(rs)
        self._h = _P()
        check(_lib.lib().ia_mesh_create(ctx.handle, self.m, self.n, nodes.ctypes.data, elems.ctypes.data, rp,
                                        C.byref(self._h)), "ia_mesh_create")
        del keep

    def close(self):
        if self._h:
            _lib.lib().ia_mesh_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def monopole_batch(ctx, mics, src, k, out=None):
    import torch
    l, m, F = mics.shape[-1], src.shape[-1], k.numel()
    if out is None:
        out = torch.empty((F, m, l), dtype=torch.complex128, device=mics.device)
    check(_lib.lib().ia_monopole_batch(ctx.handle, l, m, F, _dptr(mics, torch.float64), _dptr(src, torch.float64),
                                       _dptr(k, torch.float64), _dptr(out)), "ia_monopole_batch")
    return out  # [f, j, i] = G_f(i, j) (column-major l x m per frequency)


def ibem_assemble_batch(ctx, mesh, mics, k, cfg=None, cp=None):
    """Row-major IBEM rows: (At (F, mt, m), Bt, Ahs_t (F, l, m), Bhs_t); row i of
    each output is row i of A, B, A_hs, B_hs."""
    import torch
    cfg = cfg or default_config()
    l = mics.shape[-1]
    n_ch = 0 if cp is None else cp.shape[-1]
    F = k.numel()
    m = mesh.m
    dev = k.device
    At = torch.empty((F, m + n_ch, m), dtype=torch.complex128, device=dev)
    Bt = torch.empty_like(At)
    Ah = torch.empty((F, l, m), dtype=torch.complex128, device=dev)
    Bh = torch.empty_like(Ah)
    check(_lib.lib().ia_ibem_assemble_batch(ctx.handle, mesh._h, l, _dptr(mics, torch.float64), n_ch,
                                            _dptr(cp, torch.float64) if cp is not None else None, F,
                                            _dptr(k, torch.float64), C.byref(cfg), _dptr(At), _dptr(Bt), _dptr(Ah),
                                            _dptr(Bh)), "ia_ibem_assemble_batch")
    return At, Bt, Ah, Bh


def ibem_transfer_batch(ctx, mesh, mics, k, cfg=None):
    """H (F, m, l): H[f].T is the l x m transfer matrix (column-major storage)."""
    import torch
    cfg = cfg or default_config()
    l, F = mics.shape[-1], k.numel()
    H = torch.empty((F, mesh.m, l), dtype=torch.complex128, device=k.device)
    info = torch.zeros(F, dtype=torch.int32, device=k.device)
    check(_lib.lib().ia_ibem_transfer_batch(ctx.handle, mesh._h, l, _dptr(mics, torch.float64), F,
                                            _dptr(k, torch.float64), C.byref(cfg), _dptr(H), _dptr(info)),
          "ia_ibem_transfer_batch")
    return H, info


def hels_batch(ctx, pts, n_sh, k):
    import torch
    l, F = pts.shape[-1], k.numel()
    nt = (n_sh + 1) ** 2
    H = torch.empty((F, nt, l), dtype=torch.complex128, device=k.device)
    check(_lib.lib().ia_hels_batch(ctx.handle, l, _dptr(pts, torch.float64), int(n_sh), F, _dptr(k, torch.float64),
                                   _dptr(H)), "ia_hels_batch")
    return H


def svd_batch(ctx, A_colmajor, m, n):
    """A_colmajor: (F, n, m) tensor holding F column-major m x n matrices.
    Returns U (F, p, m), s (F, p), V (F, p, n) in the same storage convention
    (U[f].T is m x p), and info (F,)."""
    import torch
    F = A_colmajor.shape[0]
    p = min(m, n)
    dev = A_colmajor.device
    U = torch.empty((F, p, m), dtype=torch.complex128, device=dev)
    V = torch.empty((F, p, n), dtype=torch.complex128, device=dev)
    s = torch.empty((F, p), dtype=torch.float64, device=dev)
    info = torch.zeros(F, dtype=torch.int32, device=dev)
    check(_lib.lib().ia_svd_batch(ctx.handle, m, n, F, _dptr(A_colmajor), _dptr(U), _dptr(s), _dptr(V), _dptr(info)),
          "ia_svd_batch")
    return U, s, V, info


def zgemm_batch(ctx, opa, opb, M, N, K, A, B, C, alpha=1.0, beta=0.0, precision=1, slices=0, info=None):
    """C = alpha op(A) op(B) + beta C for a batch of complex FP64 matrices in
    column-major storage: A (F, cols, rows) with rows = M (op 'N') or K, B
    likewise, C (F, N, M).  op in 'N', 'T', 'C'.  precision 0: FP64 CUDA-core
    GEMM; 1: tensor-core GEMM on BF16 slices (Ozaki scheme)."""
    ops = {"N": 0, "T": 1, "C": 2}
    F = C.shape[0]
    lda, ldb, ldc = A.shape[-1], B.shape[-1], C.shape[-1]
    check(_lib.lib().ia_zgemm_batch(ctx.handle, ops[opa], ops[opb], M, N, K, float(alpha), _dptr(A), lda,
                                    A[0].numel(), _dptr(B), ldb, B[0].numel(), float(beta), _dptr(C), ldc,
                                    C[0].numel(), F, int(precision), int(slices), _dptr(info)), "ia_zgemm_batch")
    return C


def solve_batch(ctx, H_colmajor, m, n, b, cfg=None):
    """Tikhonov-GCV (or cfg.method) solves of F problems H_f x = b_f.
    H_colmajor (F, n, m); b (F, nrhs, m); returns x (F, nrhs, n), lambda
    (F, nrhs), s (F, p), info (F,)."""
    import torch
    cfg = cfg or default_config()
    F, nrhs = b.shape[0], b.shape[1]
    p = min(m, n)
    dev = b.device
    x = torch.empty((F, nrhs, n), dtype=torch.complex128, device=dev)
    lam = torch.empty((F, nrhs), dtype=torch.float64, device=dev)
    s = torch.empty((F, p), dtype=torch.float64, device=dev)
    info = torch.zeros(F, dtype=torch.int32, device=dev)
    check(_lib.lib().ia_solve_batch(ctx.handle, m, n, F, _dptr(H_colmajor), nrhs, _dptr(b), C.byref(cfg), _dptr(x),
                                    _dptr(lam), _dptr(s), _dptr(info)), "ia_solve_batch")
    return x, lam, s, info


def ibem_solve_outputs(mesh, mics, k, p):
    """Output tensors (x, lambda, s, info) for ibem_solve_batch."""
    import torch
    l, F, nrhs, m, dev = mics.shape[-1], k.numel(), p.shape[1], mesh.m, k.device
    return (torch.empty((F, nrhs, m), dtype=torch.complex128, device=dev),
            torch.empty((F, nrhs), dtype=torch.float64, device=dev),
            torch.empty((F, min(l, m)), dtype=torch.float64, device=dev),
            torch.zeros(F, dtype=torch.int32, device=dev))


def ibem_solve_batch(ctx, mesh, mics, k, p, cfg=None, out=None):
    """The IBEM pipeline: p (F, nrhs, l) measured pressures -> surface
    velocity x (F, nrhs, m), lambda (F, nrhs), s (F, min(l, m)), info (F,).
    out: preallocated outputs (ibem_solve_outputs), e.g. for graph capture."""
    import torch
    cfg = cfg or default_config()
    l, F, nrhs = mics.shape[-1], k.numel(), p.shape[1]
    x, lam, s, info = out if out is not None else ibem_solve_outputs(mesh, mics, k, p)
    check(_lib.lib().ia_ibem_solve_batch(ctx.handle, mesh._h, l, _dptr(mics, torch.float64), F,
                                         _dptr(k, torch.float64), nrhs, _dptr(p), C.byref(cfg), _dptr(x), _dptr(lam),
                                         _dptr(s), _dptr(info)), "ia_ibem_solve_batch")
    return x, lam, s, info


def esm_solve_batch(ctx, mics, src, k, p, cfg=None, out=None):
    """The ESM pipeline: p (F, nrhs, l) -> source strengths x (F, nrhs, m),
    lambda (F, nrhs), s (F, min(l, m)), info (F,); out: preallocated outputs."""
    import torch
    cfg = cfg or default_config()
    l, m, F, nrhs = mics.shape[-1], src.shape[-1], k.numel(), p.shape[1]
    dev = k.device
    if out is not None:
        x, lam, s, info = out
    else:
        x = torch.empty((F, nrhs, m), dtype=torch.complex128, device=dev)
        lam = torch.empty((F, nrhs), dtype=torch.float64, device=dev)
        s = torch.empty((F, min(l, m)), dtype=torch.float64, device=dev)
        info = torch.zeros(F, dtype=torch.int32, device=dev)
    check(_lib.lib().ia_esm_solve_batch(ctx.handle, l, m, _dptr(mics, torch.float64), _dptr(src, torch.float64), F,
                                        _dptr(k, torch.float64), nrhs, _dptr(p), C.byref(cfg), _dptr(x), _dptr(lam),
                                        _dptr(s), _dptr(info)), "ia_esm_solve_batch")
    return x, lam, s, info


def hels_solve_batch(ctx, pts, n_sh, k, p, cfg=None):
    import torch
    cfg = cfg or default_config()
    l, F, nrhs = pts.shape[-1], k.numel(), p.shape[1]
    nt = (n_sh + 1) ** 2
    dev = k.device
    x = torch.empty((F, nrhs, nt), dtype=torch.complex128, device=dev)
    lam = torch.empty((F, nrhs), dtype=torch.float64, device=dev)
    s = torch.empty((F, min(l, nt)), dtype=torch.float64, device=dev)
    info = torch.zeros(F, dtype=torch.int32, device=dev)
    check(_lib.lib().ia_hels_solve_batch(ctx.handle, l, _dptr(pts, torch.float64), int(n_sh), F,
                                         _dptr(k, torch.float64), nrhs, _dptr(p), C.byref(cfg), _dptr(x), _dptr(lam),
                                         _dptr(s), _dptr(info)), "ia_hels_solve_batch")
    return x, lam, s, info


def sinc_resistance_batch(ctx, x, k, area, cfg=None, out=None):
    """R (F, n, n) float64: omega^2 rho A^2/(4 pi c) sinc(k r_ij) for radiators
    at x (3 x n SoA, device) and wavenumbers k (F, device).  Symmetric, so the
    row-major tensor equals the column-major matrix."""
    import torch
    n, F = x.shape[-1], k.numel()
    R = out if out is not None else torch.empty((F, n, n), dtype=torch.float64, device=k.device)
    check(_lib.lib().ia_sinc_resistance_batch(ctx.handle, n, _dptr(x, torch.float64), F, _dptr(k, torch.float64),
                                              float(area), C.byref(cfg) if cfg is not None else None, _dptr(R)),
          "ia_sinc_resistance_batch")
    return R


def radiation_modes_batch(ctx, R, nmodes, cfg=None):
    """Leading nmodes eigenpairs of each R[f]: (lambda (F, nmodes) descending,
    modes (F, nmodes, n) -- mode j of frequency f is modes[f, j], info (F))."""
    import torch
    cfg = cfg or default_config()
    F, n = R.shape[0], R.shape[-1]
    lam = torch.empty((F, nmodes), dtype=torch.float64, device=R.device)
    modes = torch.empty((F, nmodes, n), dtype=torch.float64, device=R.device)
    info = torch.zeros(F, dtype=torch.int32, device=R.device)
    check(_lib.lib().ia_radiation_modes_batch(ctx.handle, n, F, _dptr(R, torch.float64), int(nmodes), C.byref(cfg),
                                              _dptr(lam), _dptr(modes), _dptr(info)), "ia_radiation_modes_batch")
    return lam, modes, info


def bem_modes_batch(ctx, mesh, mics, k, nmodes, cfg=None, pressures=True, cp=None, complex_modes=False):
    """BEM radiation modes of mesh at wavenumbers k (F,): (s (F, nmodes)
    descending singular values, Ur (F, nmodes, m) left singular vectors -- mode
    j of frequency f is Ur[f, j] --, Hr (F, nmodes, l) modal transfer columns
    at mics (3, l), Pr (F, nmodes, m) modal surface pressures or None, info
    (F,)).  Modes of the resistance Re(G Z) (real Ur, MATLAB invrS.m), or with
    complex_modes of G Z itself (complex Ur, the C++ invr()).  cp (3, n_ch):
    CHIEF points."""
    import torch
    cfg = cfg or default_config()
    l, F, m = mics.shape[-1], k.numel(), mesh.m
    n_ch = 0 if cp is None else cp.shape[-1]
    dev = k.device
    s = torch.empty((F, nmodes), dtype=torch.float64, device=dev)
    Ur = torch.empty((F, nmodes, m), dtype=torch.complex128 if complex_modes else torch.float64, device=dev)
    Hr = torch.empty((F, nmodes, l), dtype=torch.complex128, device=dev)
    Pr = torch.empty((F, nmodes, m), dtype=torch.complex128, device=dev) if pressures else None
    info = torch.zeros(F, dtype=torch.int32, device=dev)
    fn = _lib.lib().ia_bem_modes_complex_batch if complex_modes else _lib.lib().ia_bem_modes_batch
    check(fn(ctx.handle, mesh._h, l, _dptr(mics, torch.float64), n_ch, _dptr(cp, torch.float64) if n_ch else None, F,
             _dptr(k, torch.float64), int(nmodes), C.byref(cfg), _dptr(Ur), _dptr(s), _dptr(Hr),
             _dptr(Pr) if Pr is not None else None, _dptr(info)),
          "ia_bem_modes_complex_batch" if complex_modes else "ia_bem_modes_batch")
    return s, Ur, Hr, Pr, info


def admm_batch(ctx, H, p, lambda0, acfg=None, x0=None, out=None):
    """ADMM inversion (MATLAB/ADMMG.m): H (F, m, l) complex128 -- torch's
    row-major view of F column-major l x m matrices, as elsewhere here -- p
    (F, nrhs, l), lambda0 (F, nrhs) float64, x0 (F, nrhs, m) or None.  Returns
    (c (F, nrhs, m), iters (F, nrhs), info (F,))."""
    import torch
    acfg = acfg or default_admm_config()
    F, m, l = H.shape
    nrhs = p.shape[1]
    dev = H.device
    if out is not None:
        c, its, info = out
    else:
        c = torch.empty((F, nrhs, m), dtype=torch.complex128, device=dev)
        its = torch.empty((F, nrhs), dtype=torch.int32, device=dev)
        info = torch.zeros(F, dtype=torch.int32, device=dev)
    check(_lib.lib().ia_admm_batch(ctx.handle, l, m, F, _dptr(H), nrhs, _dptr(p), _dptr(lambda0, torch.float64),
                                   C.byref(acfg), _dptr(x0) if x0 is not None else None, _dptr(c), _dptr(its),
                                   _dptr(info)), "ia_admm_batch")
    return c, its, info


def sound_power_batch(ctx, R, v):
    """W (F, nrhs) = 1/2 Re(v^H R v) for velocity fields v (F, nrhs, n) complex128."""
    import torch
    F, n = R.shape[0], R.shape[-1]
    nrhs = v.shape[1]
    W = torch.empty((F, nrhs), dtype=torch.float64, device=R.device)
    check(_lib.lib().ia_sound_power_batch(ctx.handle, n, F, _dptr(R, torch.float64), nrhs, _dptr(v), _dptr(W)),
          "ia_sound_power_batch")
    return W


def esm_design_batch(ctx, mics, surface, retreat, k, loglam, q, noise=None, grad=True):
    """Differentiable ESM design objective on the device.

    mics (3, l), surface (3, m), retreat (1,), k (F,), loglam (F,) float64 and
    q (F, nrhs, m), noise (F, nrhs, l) complex128 CUDA tensors.  Returns
    (err (F, nrhs), grad_mics (3, l), grad_retreat (1,), grad_loglam (F,),
    info (F,)); the gradients are those of err.mean() and are None when
    grad is False."""
    import torch
    l, m, F, nrhs = mics.shape[-1], surface.shape[-1], k.numel(), q.shape[1]
    dev = k.device
    err = torch.empty((F, nrhs), dtype=torch.float64, device=dev)
    info = torch.zeros(F, dtype=torch.int32, device=dev)
    gm = gd = gl = None
    if grad:
        gm = torch.empty((3, l), dtype=torch.float64, device=dev)
        gd = torch.empty(1, dtype=torch.float64, device=dev)
        gl = torch.empty(F, dtype=torch.float64, device=dev)
    check(_lib.lib().ia_esm_design_batch(ctx.handle, l, m, F, nrhs, _dptr(mics, torch.float64),
                                         _dptr(surface, torch.float64), _dptr(retreat, torch.float64),
                                         _dptr(k, torch.float64), _dptr(loglam, torch.float64), _dptr(q),
                                         _dptr(noise), _dptr(err), _dptr(gm), _dptr(gd), _dptr(gl), _dptr(info)),
          "ia_esm_design_batch")
    return err, gm, gd, gl, info
