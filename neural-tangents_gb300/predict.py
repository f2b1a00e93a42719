"""nt_gb300.predict -- closed-form kernel regression (neural_tangents/_src/predict.py).

``gp_inference`` and ``gradient_descent_mse_ensemble`` (predict.py:566-1005) give the
NNGP / NTK / NTKGP posterior and the infinite-ensemble predictions on the same kernels.

``gradient_descent_mse(k_train_train, y_train, ...)`` keeps the reference
signature (predict.py:71-278) and returns ``predict_fn(t=None, fx_train_0=0.,
fx_test_0=None, k_test_train=None)``. ``t=None`` (infinite time) and a scalar
``t=inf`` take the Cholesky path: an FP32 Cholesky of K + lambda I on the GPU (128-wide panels,
the panel solves and trailing updates on the tcgen05 tensor cores), solves by the
explicit inverse factors and a refinement whose products with K are accumulated in
double-float (preconditioned conjugate gradients for up to 16 right-hand sides, plain
refinement steps for more; `refine_iters` overrides the default, 0 gives the plain FP32
solve), all in libntgb300.so. The mean predictions multiply k_test_train by the FP64
solution in double-float (ntg_gemm_df). The factorisation is computed once and cached,
as the reference caches it (predict.py:163). Finite ``t`` uses the eigenbasis of
predict.py:185-229 with this library's own eigensolver (two-sided block Jacobi in FP32
with double-float refinement, ntg_eigh), its spectral-weight kernel and FP32 GEMMs.
Only 2-D ``k_train_train`` with ``trace_axes=(-1,)`` is supported.
"""
from __future__ import annotations

import collections
import math
import warnings
from typing import Optional

import numpy as np
import torch

from . import _lib as L


def _dev(x, dtype=torch.float32) -> torch.Tensor:
    dev = L.require_cuda()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=dtype).contiguous()
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=dev).contiguous()


def _gemm(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    out = torch.empty((a.shape[0], b.shape[1]), device=a.device, dtype=torch.float32)
    L.call('ntg_gemm', L.stream(), L.ptr(a), L.ptr(b), L.ptr(out), a.shape[0], b.shape[1],
           a.shape[1], 0)
    return out


def _gemm_df(a: torch.Tensor, x64: torch.Tensor, out64: bool = False):
    """a @ x64 for a [rows, n] float32 and x64 [n, m] float64, accumulated in double-float
    and rounded to float32 (ntg_gemm_df): the mean predictions k_test_train A^{-1} y, whose
    products cancel when A is ill-conditioned, keep the digits of the FP64 solution.
    out64: return (float32, float64) results."""
    a = a.contiguous()
    x64 = x64.contiguous()
    rows, n = a.shape
    m = x64.shape[1]
    out = torch.empty((rows, m), device=a.device, dtype=torch.float32)
    o64 = torch.empty((rows, m), device=a.device, dtype=torch.float64) if out64 else None
    ws_bytes = int(L.load().ntg_gemm_df_workspace_bytes(rows, n, m))
    ws = torch.empty((ws_bytes,), device=a.device, dtype=torch.uint8)
    L.call('ntg_gemm_df', L.stream(), L.ptr(a), n, rows, n, x64.data_ptr(), m, None,
           out.data_ptr(), None if o64 is None else o64.data_ptr(), ws.data_ptr(), ws_bytes)
    return (out, o64) if out64 else out


def _gemm_tn(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """a^T @ b for a [k, m], b [k, n] on the library's FP32 GEMM."""
    out = torch.empty((a.shape[1], b.shape[1]), device=a.device, dtype=torch.float32)
    L.call('ntg_gemm_ex', L.stream(), L.ptr(a), L.ptr(b), L.ptr(out), a.shape[1], b.shape[1],
           a.shape[0], 1, 1., 0)
    return out


def _eigh(k: torch.Tensor, shift: float, max_sweeps: int = 20, tol: float = 1e-5,
          refine_steps: int = 2):
    """Eigenpairs of k + shift I on this library's block-Jacobi kernels (FP32) with
    `refine_steps` double-float refinement steps: (evals [n], evecs [n, n], column j
    for evals[j]), evals not sorted. The Jacobi sweeps stop at an off-diagonal norm of
    `tol` (relative); the refinement steps take the pairs from there to FP32 accuracy."""
    n = k.shape[0]
    lib = L.load()
    nbytes = int(lib.ntg_eigh_workspace_bytes(n))
    ws = torch.empty((nbytes,), device=k.device, dtype=torch.uint8)
    evals = torch.empty((n,), device=k.device, dtype=torch.float32)
    evecs = torch.empty((n, n), device=k.device, dtype=torch.float32)
    L.call('ntg_eigh', L.stream(), L.ptr(k.contiguous()), n, float(shift), L.ptr(evals),
           L.ptr(evecs), int(max_sweeps), float(tol), int(refine_steps), ws.data_ptr(), nbytes,
           None)
    return evals, evecs


# spectral functions of ntg_spectral_scale (predict.py:1277-1294 and the ensemble's)
_EXPM1, _INV_EXPM1, _POS_EXP2, _EXP, _NEG_INV_EXPM1_2, _NEG_EXPM1, _NEG_INV_EXPM1 = range(7)


def _spectral(evals: torch.Tensor, ts: torch.Tensor, kind: int, norm: float,
              x: torch.Tensor) -> torch.Tensor:
    """out [n, T, m] = w_kind(lambda_i, t) x[i, :] for x [n, m] and the times ts [T]."""
    n, m = x.shape
    out = torch.empty((n, ts.numel(), m), device=x.device, dtype=torch.float32)
    L.call('ntg_spectral_scale', L.stream(), L.ptr(evals), ts.data_ptr(), ts.numel(), kind,
           float(norm), L.ptr(x.contiguous()), n, m, L.ptr(out))
    return out


def _spectral_apply(evecs, evals, ts, kind, norm, x):
    """sum_i evecs[:, i] w_kind(lambda_i, t) x[i, :] for every t: [T, n, m]."""
    w = _spectral(evals, ts, kind, norm, x)                    # [n, T, m]
    n, nt, m = w.shape
    return _gemm(evecs, w.reshape(n, nt * m)).reshape(evecs.shape[0], nt, m).permute(1, 0, 2)


def _times(t, learning_rate, dev):
    tt = np.asarray(t, np.float64) * learning_rate
    return tt.shape, torch.as_tensor(tt.reshape(-1), dtype=torch.float64, device=dev)


class CholeskySolver:
    """Cached factorisation of K + lambda I (predict.py:1224-1258) on the tensor-core
    Cholesky kernels: L lives in a [n, ldl] buffer (ldl = n rounded up to 32, the row
    pitch the TMA loads of the trailing updates need); the factor workspace keeps the
    inverses of the 128-wide diagonal blocks and L^T for the solves."""

    # refinement per solve when the caller gives none: at most 8 preconditioned CG
    # iterations for up to 16 right-hand sides (they stop once converged, typically after
    # two; the rest of the launches return at once), 2 plain refinement steps for more
    REFINE_FEW, REFINE_MANY, FEW = 8, 2, 16

    def __init__(self, k: torch.Tensor, diag_reg: float, absolute: bool,
                 refine_iters: Optional[int] = None):
        n = k.shape[0]
        if k.ndim != 2 or k.shape[1] != n:
            raise NotImplementedError('nt_gb300 supports a 2-D square k_train_train')
        lib = L.load()
        self.k, self.n = k, n
        self.refine = None if refine_iters is None else int(refine_iters)
        self.ldl = (n + 31) // 32 * 32
        self.Lbuf = torch.empty((n, self.ldl), device=k.device, dtype=torch.float32)
        fws = int(lib.ntg_chol_factor_tc_workspace_bytes(n, self.ldl))
        self.fws = torch.empty((fws,), device=k.device, dtype=torch.uint8)
        self.lam = torch.zeros((2,), device=k.device, dtype=torch.float64)
        info = torch.zeros((1,), device=k.device, dtype=torch.int32)
        L.call('ntg_chol_factor_tc', L.stream(), L.ptr(k), n, float(diag_reg),
               int(bool(absolute)), self.Lbuf.data_ptr(), self.ldl, self.lam.data_ptr(),
               info.data_ptr(), self.fws.data_ptr(), fws)
        self.info = int(info.item())
        if self.info:
            warnings.warn(f'k_train_train + diag_reg * I is not positive definite (pivot '
                          f'{self.info}); the solution is NaN, as jax.scipy.linalg.cho_solve '
                          f'would return.')
        self.residual = None

    @property
    def L(self) -> torch.Tensor:
        """The lower factor as an [n, n] view of its padded buffer."""
        return self.Lbuf[:, :self.n]

    def logdet(self) -> torch.Tensor:
        """log det(K + lambda I) = 2 sum log L_ii (device float64, shape [1])."""
        out = torch.zeros(1, device=self.k.device, dtype=torch.float64)
        L.call('ntg_chol_logdet_tc', L.stream(), self.Lbuf.data_ptr(), self.n, self.ldl,
               out.data_ptr())
        return out

    COLS = 4096  # right-hand sides per ntg_chol_solve_tc call (bounds its workspace)

    def solve(self, b: torch.Tensor, refine_iters: Optional[int] = None,
              residual: bool = True, want_x64: bool = False,
              b64: Optional[torch.Tensor] = None):
        """A^{-1} b; refine_iters overrides the solver's refinement steps; residual=False
        skips the final residual kept in self.residual. want_x64: also return the FP64
        solution before its rounding to float32, as (x, x64). b64: the right-hand side in
        FP64 (b its float32 rounding), which the refinement then solves for."""
        b = b.reshape(self.n, -1).contiguous()
        if b64 is not None:
            b64 = b64.reshape(self.n, -1).contiguous()
        refine = self.refine if refine_iters is None else int(refine_iters)
        if refine is None:
            refine = self.REFINE_FEW if b.shape[1] <= self.FEW else self.REFINE_MANY
        if self.info:
            nan = torch.full_like(b, float('nan'))
            return (nan, nan.double()) if want_x64 else nan
        out = torch.empty_like(b)
        x64 = torch.empty(b.shape, device=b.device, dtype=torch.float64) if want_x64 else None
        cols = min(b.shape[1], self.COLS)
        lib = L.load()
        ws_bytes = int(lib.ntg_chol_solve_tc_workspace_bytes(self.n, cols, self.ldl))
        ws = torch.empty((ws_bytes,), device=b.device, dtype=torch.uint8)
        res = torch.zeros((1,), device=b.device, dtype=torch.float64) if residual else None
        single = b.shape[1] <= cols
        for c0 in range(0, b.shape[1], cols):
            bc = b if single else b[:, c0:c0 + cols].contiguous()
            b64c = b64 if (single or b64 is None) else b64[:, c0:c0 + cols].contiguous()
            xc = out if single else torch.empty_like(bc)
            x64c = x64 if (single or x64 is None) else torch.empty(bc.shape, device=b.device,
                                                                     dtype=torch.float64)
            L.call('ntg_chol_solve_tc', L.stream(), L.ptr(self.k), self.Lbuf.data_ptr(), self.ldl,
                   self.fws.data_ptr(), self.lam.data_ptr(), self.n, L.ptr(bc), bc.shape[1],
                   L.ptr(xc), refine, ws.data_ptr(), ws_bytes,
                   None if res is None else res.data_ptr(),
                   None if x64c is None else x64c.data_ptr(),
                   None if b64c is None else b64c.data_ptr())
            if not single:
                out[:, c0:c0 + cols] = xc
                if x64 is not None:
                    x64[:, c0:c0 + cols] = x64c
        if res is not None:
            self.residual = res
        return (out, x64) if want_x64 else out


def gradient_descent_mse(k_train_train, y_train, learning_rate: float = 1.,
                         diag_reg: float = 0., diag_reg_absolute_scale: bool = False,
                         trace_axes=(-1,), refine_iters: Optional[int] = None):
    """predict.py:71-278."""
    if tuple(trace_axes) not in ((-1,), (1,)):
        raise NotImplementedError('nt_gb300 supports trace_axes=(-1,)')
    k = _dev(k_train_train)
    y = _dev(y_train)
    if y.ndim == 1:
        raise ValueError('y_train must have a trailing output axis')
    state = {}

    def solver() -> CholeskySolver:
        if 'chol' not in state:
            state['chol'] = CholeskySolver(k, diag_reg, diag_reg_absolute_scale, refine_iters)
        return state['chol']

    def eig():
        if 'eig' not in state:
            n = k.shape[0]
            reg = diag_reg if diag_reg_absolute_scale else \
                diag_reg * float(k.diagonal().double().sum()) / n
            state['eig'] = _eigh(k, reg)
        return state['eig']

    def predict_fn(t=None, fx_train_0=0., fx_test_0=None, k_test_train=None):
        if fx_test_0 is not None and k_test_train is None:
            raise ValueError('`k_test_train` must be specified when `fx_test_0` is not `None`.')
        # A scalar t = inf is the limit t=None computes (predict.py:236-239, pinned by
        # predict_test.py:396-428): it takes the Cholesky path too, unless the regularised
        # kernel is not positive definite, where the eigenbasis path's |lambda| applies.
        if _is_inf(t) and solver().info == 0:
            t = None
        if t is None:
            fx_train_t = y
            if fx_test_0 is None:
                return fx_train_t
            rhs = y if fx_train_0 is None else y - _as_like(fx_train_0, y)
            # differentiable in k_train_train, k_test_train, y and the initial outputs
            fx_test_t = _as_like(fx_test_0, None) + _RidgePredict.apply(
                k, _dev(k_test_train), rhs, float(diag_reg), bool(diag_reg_absolute_scale),
                refine_iters, solver())
            if fx_train_0 is None:
                return fx_test_t
            return fx_train_t, fx_test_t
        # eigenbasis path (predict.py:185-229): own block-Jacobi eigenpairs, spectral
        # weights and products on this library's kernels, FP32
        evals, evecs = eig()
        tshape, ts = _times(t, learning_rate, k.device)
        rhs = -y if fx_train_0 is None else _as_tensor(fx_train_0, y) - y
        proj = _gemm_tn(evecs, rhs.contiguous())                    # [n, m]
        norm = y.numel()
        outs = []
        if fx_train_0 is not None:
            dfx = _spectral_apply(evecs, evals, ts, _EXPM1, norm, proj)   # [T, n, m]
            outs.append((_as_tensor(fx_train_0, y) + dfx).reshape(tshape + tuple(y.shape)))
        if fx_test_0 is not None:
            dfx = _spectral_apply(evecs, evals, ts, _INV_EXPM1, norm, proj)
            kt = _dev(k_test_train)
            nt_, n, m = dfx.shape
            flat = dfx.permute(1, 0, 2).reshape(n, nt_ * m).contiguous()
            test = _gemm(kt, flat).reshape(kt.shape[0], nt_, m).permute(1, 0, 2)
            test = _as_tensor(fx_test_0, y) + test
            outs.append(test.reshape(tshape + (kt.shape[0], y.shape[1])))
        if len(outs) == 2:
            return tuple(outs)
        return outs[0] if outs else y

    return predict_fn


def _is_inf(t) -> bool:
    """Whether t is the scalar +inf (a Python number or a 0-d array)."""
    if t is None:
        return False
    a = np.asarray(t.cpu() if isinstance(t, torch.Tensor) else t)
    return a.ndim == 0 and bool(np.isposinf(a))


def _as_like(v, like: Optional[torch.Tensor]):
    if isinstance(v, (int, float)):
        return v
    return _dev(v)


def _as_tensor(v, like: torch.Tensor):
    """A scalar stays a Python number; arrays become float32 device tensors."""
    if isinstance(v, (int, float)):
        return v
    return _dev(v)


class _NLL(torch.autograd.Function):
    """1/2 tr(Y^T A^{-1} Y) + m/2 log det A + n m/2 log 2 pi, A = K + lambda I."""

    @staticmethod
    def forward(ctx, k, y, diag_reg, absolute, refine_iters):
        k = k.contiguous()
        n, m = y.shape
        solver = CholeskySolver(k, diag_reg, absolute, refine_iters)
        alpha = solver.solve(y)
        ld = solver.logdet()
        quad = (y.double() * alpha.double()).sum()
        nll = 0.5 * quad + 0.5 * m * ld[0] + 0.5 * n * m * math.log(2 * math.pi)
        ctx.solver, ctx.alpha, ctx.meta = solver, alpha, (diag_reg, absolute, n, m)
        return nll.float()

    @staticmethod
    def backward(ctx, g):
        diag_reg, absolute, n, m = ctx.meta
        solver, alpha = ctx.solver, ctx.alpha
        eye = torch.zeros((n, n), device=alpha.device)
        eye.view(-1)[::n + 1] = 1.
        # A^{-1} for the log-determinant term, with one refinement step (double-float
        # residual): on the ill-conditioned kernels of wide, deep FCNs the plain FP32
        # inverse moves this gradient term by tens of percent, one step squares that error
        kinv = solver.solve(eye, refine_iters=1, residual=False)
        out = torch.empty((n, n), device=alpha.device)
        tr = torch.zeros(1, device=alpha.device, dtype=torch.float64)
        L.call('ntg_nll_grad', L.stream(), L.ptr(kinv), L.ptr(alpha.contiguous()), n, m,
               float(g.item()), 0. if absolute else diag_reg / n, L.ptr(out), tr.data_ptr())
        return out, alpha * g, None, None, None


def negative_log_likelihood(k_train_train, y_train, diag_reg: float = 0.,
                            diag_reg_absolute_scale: bool = False,
                            refine_iters: Optional[int] = None):
    """NNGP negative log marginal likelihood, differentiable with respect to the kernel.

    A helper for hyper-parameter learning (not part of the reference's predict
    module): 1/2 tr(Y^T A^{-1} Y) + m/2 log det A + n m/2 log(2 pi) with
    A = K + diag_reg * trace(K) / n * I (or diag_reg * I when absolute), on the
    Cholesky kernels of this module; its backward is the Cholesky adjoint
    g (-1/2 alpha alpha^T + m/2 A^{-1}).
    """
    k = k_train_train if isinstance(k_train_train, torch.Tensor) else _dev(k_train_train)
    y = _dev(y_train)
    return _NLL.apply(k, y, float(diag_reg), bool(diag_reg_absolute_scale), refine_iters)


class _RidgeSolve(torch.autograd.Function):
    """alpha = A^{-1} Y, A = K + lambda I; backward: gY = A^{-1} g,
    gK = -gY alpha^T - [relative lambda] (r / n) <gY, alpha> I."""

    @staticmethod
    def forward(ctx, k, y, diag_reg, absolute, refine_iters):
        k = k.contiguous()
        y2 = y.reshape(y.shape[0], -1).contiguous()
        solver = CholeskySolver(k, diag_reg, absolute, refine_iters)
        alpha = solver.solve(y2)
        ctx.solver, ctx.alpha, ctx.meta = solver, alpha, (diag_reg, absolute, tuple(y.shape))
        return alpha.reshape(y.shape)

    @staticmethod
    def backward(ctx, g):
        diag_reg, absolute, yshape = ctx.meta
        solver, alpha = ctx.solver, ctx.alpha
        n = alpha.shape[0]
        gy = solver.solve(g.reshape(n, -1).contiguous(), residual=False)
        gk = torch.empty((n, n), device=alpha.device)
        L.call('ntg_gemm_ex', L.stream(), L.ptr(gy), L.ptr(alpha.t().contiguous()), L.ptr(gk), n,
               n, alpha.shape[1], 0, -1., 0)
        if not absolute and diag_reg:
            gk.diagonal().sub_((diag_reg / n) * (gy.double() * alpha.double()).sum().float())
        return gk, gy.reshape(yshape), None, None, None


def kernel_ridge_solve(k_train_train, y_train, diag_reg: float = 0.,
                       diag_reg_absolute_scale: bool = False,
                       refine_iters: Optional[int] = None):
    """(K + diag_reg * trace(K) / n * I)^{-1} y on this module's Cholesky kernels,
    differentiable with respect to K and y (a helper for kernel-ridge losses such
    as the support-set objective of dataset distillation; the reference computes
    the same solve inside gradient_descent_mse, predict.py:1235-1258). The
    backward reuses the cached factorisation: gY = A^{-1} g, gK = -gY alpha^T
    (minus the trace term of a relative diag_reg)."""
    k = k_train_train if isinstance(k_train_train, torch.Tensor) else _dev(k_train_train)
    y = y_train if isinstance(y_train, torch.Tensor) else _dev(y_train)
    return _RidgeSolve.apply(k, y, float(diag_reg), bool(diag_reg_absolute_scale),
                             refine_iters)


class _RidgePredict(torch.autograd.Function):
    """k_test_train A^{-1} y, A = K + lambda I, from the FP64 solution and a double-float
    product (ntg_gemm_df): with an ill-conditioned A the product cancels, and an FP32
    product of the rounded solution would lose cond(A)-many of its digits. Backward,
    with alpha = A^{-1} y and the cotangent g: gK_td = g alpha^T, gY = A^{-1} K_td^T g
    (the right-hand side in double-float, solved for in FP64),
    gK = -gY alpha^T - [relative lambda] (r / n) <gY, alpha> I."""

    @staticmethod
    def forward(ctx, k, k_td, y, diag_reg, absolute, refine_iters, solver):
        n = k.shape[0]
        y2 = y.reshape(n, -1).contiguous()
        if solver is None:
            solver = CholeskySolver(k.contiguous(), diag_reg, absolute, refine_iters)
        alpha, alpha64 = solver.solve(y2, want_x64=True)
        k_td = k_td.contiguous()
        out = _gemm_df(k_td, alpha64)
        ctx.solver, ctx.alpha, ctx.meta = solver, alpha, (diag_reg, absolute, tuple(y.shape))
        ctx.save_for_backward(k_td)
        return out.reshape((k_td.shape[0],) + tuple(y.shape[1:]))

    @staticmethod
    def backward(ctx, g):
        diag_reg, absolute, yshape = ctx.meta
        solver, alpha = ctx.solver, ctx.alpha
        (k_td,) = ctx.saved_tensors
        n = alpha.shape[0]
        g2 = g.reshape(k_td.shape[0], -1).contiguous()
        gk = gk_td = gy = None
        if ctx.needs_input_grad[1]:
            gk_td = _gemm(g2, alpha.t().contiguous())
        if ctx.needs_input_grad[0] or ctx.needs_input_grad[2]:
            # K_td^T g in double-float and solved for in FP64: its float32 rounding alone
            # would move gY by cond(A) u
            r32, r64 = _gemm_df(k_td.t().contiguous(), g2.double(), out64=True)
            gy = solver.solve(r32, residual=False, b64=r64)
            if ctx.needs_input_grad[0]:
                gk = torch.empty((n, n), device=alpha.device)
                L.call('ntg_gemm_ex', L.stream(), L.ptr(gy), L.ptr(alpha.t().contiguous()),
                       L.ptr(gk), n, n, alpha.shape[1], 0, -1., 0)
                if not absolute and diag_reg:
                    gk.diagonal().sub_((diag_reg / n) *
                                       (gy.double() * alpha.double()).sum().float())
            gy = gy.reshape(yshape)
        return gk, gk_td, gy, None, None, None, None


def kernel_ridge_predict(k_test_train, k_train_train, y_train, diag_reg: float = 0.,
                         diag_reg_absolute_scale: bool = False,
                         refine_iters: Optional[int] = None):
    """k_test_train (K + diag_reg * trace(K) / n * I)^{-1} y, differentiable with respect to
    both kernels and y: the mean prediction of gradient_descent_mse at t = None
    (predict.py:236-276), and the prediction of kernel-ridge losses such as
    ||y_t - K_ts (K_ss + lambda I)^{-1} y_s||^2 (dataset distillation). The product
    is formed from the FP64 solution in double-float, so an ill-conditioned K costs
    no digits beyond those of the kernels themselves; the backward reuses the
    factorisation (see _RidgePredict)."""
    k = k_train_train if isinstance(k_train_train, torch.Tensor) else _dev(k_train_train)
    kt = k_test_train if isinstance(k_test_train, torch.Tensor) else _dev(k_test_train)
    y = y_train if isinstance(y_train, torch.Tensor) else _dev(y_train)
    return _RidgePredict.apply(k, kt, y, float(diag_reg), bool(diag_reg_absolute_scale),
                               refine_iters, None)


class _MatMul(torch.autograd.Function):
    """a @ b on the library's FP32 GEMM, with its two adjoint GEMMs."""

    @staticmethod
    def forward(ctx, a, b):
        a, b = a.contiguous(), b.contiguous()
        ctx.save_for_backward(a, b)
        return _gemm(a, b)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        g = g.contiguous()
        ga = _gemm(g, b.t().contiguous())
        gb = torch.empty_like(b)
        L.call('ntg_gemm_ex', L.stream(), L.ptr(a), L.ptr(g), L.ptr(gb), b.shape[0], b.shape[1],
               a.shape[0], 1, 1., 0)
        return ga, gb


def matmul(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Differentiable a @ b for float32 CUDA matrices on the library's GEMM kernels."""
    return _MatMul.apply(a, b)


# ---------------------------------------------------------------------------
# Posterior of the NNGP / NTK / NTKGP and the infinite ensemble
# (predict.py:566-745, 753-1005)
# ---------------------------------------------------------------------------

Gaussian = collections.namedtuple('Gaussian', 'mean covariance')


def _kattr(k, g):
    """A field of a kernel container (Kernel, AnalyticKernel, dict) or the array itself."""
    if isinstance(k, dict):
        return k[g]
    if hasattr(k, g):
        return getattr(k, g)
    return k


def _has(k, g) -> bool:
    return (g in k) if isinstance(k, dict) else hasattr(k, g)


def _names(get):
    if get is None:
        return ('nngp', 'ntk')
    if isinstance(get, str):
        return (get.lower(),)
    return tuple(g.lower() for g in get)


def _gaussians(get, names, out):
    if isinstance(get, str):
        return out[names[0]]
    return collections.namedtuple('Gaussians', names)(*[out[g] for g in names])


def gp_inference(k_train_train, y_train, diag_reg: float = 0.,
                 diag_reg_absolute_scale: bool = False, trace_axes=(-1,),
                 refine_iters: Optional[int] = None):
    """predict.py:566-745: ``predict_fn(get, k_test_train, k_test_test)`` with the
    NNGP / NTK / NTKGP posterior mean and, given ``k_test_test``, covariance.

    Every solve runs on this module's Cholesky kernels (FP32 factorisation cached per
    kernel, solves refined in double-float), the means on the double-float product with
    the FP64 solution and every other product on its GEMM kernel; 2-D kernels with
    ``trace_axes=(-1,)``."""
    if tuple(trace_axes) not in ((-1,), (1,)):
        raise NotImplementedError('nt_gb300 supports trace_axes=(-1,)')
    y = _dev(y_train)
    solvers = {}

    def solve(g: str):
        if g not in solvers:
            solvers[g] = CholeskySolver(_dev(_kattr(k_train_train, g)), diag_reg,
                                        diag_reg_absolute_scale, refine_iters)
        return solvers[g]

    k_inv_y = {}

    def predict_fn(get=None, k_test_train=None, k_test_test=None):
        names = _names(get)
        out = {}
        for g in names:
            k = 'ntk' if g == 'ntkgp' else g
            k_dd = _dev(_kattr(k_train_train, k))
            k_td = None if k_test_train is None else _dev(_kattr(k_test_train, k))
            if k_td is None:
                mean = y
            else:
                if k not in k_inv_y:  # the FP64 solution: the product below cancels
                    k_inv_y[k] = solve(k).solve(y, residual=False, want_x64=True)[1]
                mean = _gemm_df(k_td, k_inv_y[k].reshape(y.shape[0], -1)).reshape(
                    (k_td.shape[0],) + tuple(y.shape[1:]))
            if k_test_test is None:
                out[g] = mean
                continue
            if k_td is None:
                out[g] = Gaussian(mean, torch.zeros_like(k_dd))
                continue
            if g == 'ntk' and (not _has(k_train_train, 'nngp') or not _has(k_test_train, 'nngp')):
                raise ValueError(
                    'If `"ntk" in get`, and `k_test_test is not None`, and `k_test_train is not '
                    'None`, i.e. you request the NTK posterior covariance on the test set, you '
                    'need both NTK and NNGP train-train and test-train matrices contained in '
                    '`k_test_train` and `k_train_train`. Hence they must be `namedtuple`s with '
                    '`nngp` and `ntk` attributes.')
            g_init = 'nngp' if g != 'ntkgp' else 'ntk'
            k_td_g_inv_y = solve(k).solve(_dev(_kattr(k_test_train, g_init)).t().contiguous(),
                                          residual=False)
            k_tt = _dev(_kattr(k_test_test, g_init))
            if g in ('nngp', 'ntkgp'):
                cov = k_tt - _gemm(k_td, k_td_g_inv_y)
            elif g == 'ntk':
                term_1 = solve(g).solve(k_td.t().contiguous(), residual=False)
                nngp_dd = _dev(_kattr(k_train_train, 'nngp'))
                cov = _gemm(term_1.t().contiguous(), _gemm(nngp_dd, term_1))
                term_2 = _gemm(k_td, k_td_g_inv_y)
                cov = cov - (term_2 + term_2.t()) + k_tt
            else:
                raise ValueError(g)
            out[g] = Gaussian(mean, cov)
        return _gaussians(get, names, out)

    return predict_fn


def _dependency(names, compute_cov):
    """predict.py _get_dependency."""
    for g in names:
        if g not in ('nngp', 'ntk'):
            raise NotImplementedError(
                'Can only get either "nngp" or "ntk" predictions, got %s.' % g)
    dep = ()
    if 'nngp' in names or ('ntk' in names and compute_cov):
        dep += ('nngp',)
    if 'ntk' in names:
        dep += ('ntk',)
    return dep


def gradient_descent_mse_ensemble(kernel_fn, x_train, y_train, learning_rate: float = 1.,
                                  diag_reg: float = 0., diag_reg_absolute_scale: bool = False,
                                  trace_axes=(-1,), **kernel_fn_train_train_kwargs):
    """predict.py:753-1005: ``predict_fn(t=None, x_test=None, get=None, compute_cov=False)``,
    the mean (and covariance) of the infinite ensemble of infinite-width networks
    trained by gradient flow on the MSE loss. ``t=None`` is the Cholesky path of
    ``gp_inference`` (this library's kernels); finite ``t`` uses the library's own
    eigendecomposition of the regularised train-train kernel (block Jacobi, FP32), the
    expm1 spectral functions of predict.py:1277-1294 as a kernel, and its FP32 GEMMs."""
    if tuple(trace_axes) not in ((-1,), (1,)):
        raise NotImplementedError('nt_gb300 supports trace_axes=(-1,)')
    y = _dev(y_train)
    k_dd = {}

    def k_train(dep):
        missing = tuple(g for g in dep if g not in k_dd)
        if len(missing) == 1:
            k_dd[missing[0]] = _dev(kernel_fn(x_train, None, missing[0],
                                              **kernel_fn_train_train_kwargs))
        elif missing:
            k = kernel_fn(x_train, None, missing, **kernel_fn_train_train_kwargs)
            for g in missing:
                k_dd[g] = _dev(getattr(k, g))
        return {g: k_dd[g] for g in dep}

    eig = {}

    def eigenspace(g):
        if g not in eig:
            a = k_train((g,))[g]
            n = a.shape[0]
            reg = diag_reg if diag_reg_absolute_scale else \
                diag_reg * float(a.diagonal().double().sum()) / n
            eig[g] = _eigh(a, reg)
        return eig[g]

    inf_cache = {}

    def predict_fn(t=None, x_test=None, get=None, compute_cov: bool = False,
                   **kernel_fn_test_test_kwargs):
        names = _names(get)
        dep = _dependency(names, compute_cov)
        kd = k_train(dep)
        kw_tt = {**kernel_fn_train_train_kwargs, **kernel_fn_test_test_kwargs}
        if x_test is None:
            k_td = None
            nngp_tt = True if compute_cov else None
        else:
            k = kernel_fn(x_test, x_train, dep if len(dep) > 1 else dep[0], **kw_tt)
            k_td = {g: _dev(getattr(k, g) if len(dep) > 1 else k) for g in dep}
            nngp_tt = _dev(kernel_fn(x_test, None, 'nngp', **kw_tt)) if compute_cov else None
        if _is_inf(t):
            t = None  # the limit gp_inference computes (predict.py:860-905 at t = inf)
        if t is None:
            if dep not in inf_cache:
                inf_cache[dep] = gp_inference(kd, y, diag_reg, diag_reg_absolute_scale)
            return inf_cache[dep](get=get, k_test_train=k_td, k_test_test=nngp_tt)
        # eigenbasis path: own block-Jacobi eigenpairs, the spectral weights of
        # predict.py:1277-1294 and every product on this library's kernels (FP32)
        t_shape, ts = _times(t, learning_rate, y.device)
        nt_ = ts.numel()
        norm = y.numel()
        out = {}

        def per_t(x):  # [T, a, b] -> t_shape + [a, b]
            return x.reshape(t_shape + tuple(x.shape[1:]))

        def sym_apply(evecs, evals, kind, x_t):
            # evecs diag(w_kind(t)) evecs^T for every t: [T, n, n]
            return _spectral_apply(evecs, evals, ts, kind, norm, evecs.t().contiguous())

        for g in names:
            evals, evecs = eigenspace(g)
            proj = _gemm_tn(evecs, y)                                   # [n, m]
            if k_td is None:
                mean = _spectral_apply(evecs, evals, ts, _NEG_EXPM1, norm, proj)
            else:
                ktd = k_td[g]
                w = _spectral_apply(evecs, evals, ts, _NEG_INV_EXPM1, norm, proj)  # [T, n, m]
                n, m = proj.shape
                flat = w.permute(1, 0, 2).reshape(n, nt_ * m).contiguous()
                mean = _gemm(ktd, flat).reshape(ktd.shape[0], nt_, m).permute(1, 0, 2)
            mean = per_t(mean.contiguous())
            if nngp_tt is None:
                out[g] = mean
                continue
            nngp_dd = kd['nngp']
            if k_td is None:
                if g == 'nngp':
                    cov = sym_apply(evecs, evals, _POS_EXP2, None)
                else:
                    ex = sym_apply(evecs, evals, _EXP, None)              # [T, n, n]
                    cov = torch.stack([_gemm(_gemm(e.contiguous(), nngp_dd), e.contiguous())
                                       for e in ex])
            else:
                tt_k = nngp_tt[None]
                a = _gemm(ktd, evecs)                                     # [s, n]
                at = a.t().contiguous()                                   # [n, s]
                s_ = a.shape[0]
                if g == 'nngp':
                    w = _spectral(evals, ts, _NEG_INV_EXPM1_2, norm, at)   # [n, T, s]
                    flat = w.reshape(at.shape[0], nt_ * s_)
                    quad = _gemm(a, flat).reshape(s_, nt_, s_).permute(1, 0, 2)
                    cov = tt_k - quad
                else:
                    term_1 = _spectral_apply(evecs, evals, ts, _NEG_INV_EXPM1, norm, at)
                    c = _gemm_tn(evecs, k_td['nngp'].t().contiguous())    # [n, s]
                    w = _spectral(evals, ts, _NEG_INV_EXPM1, norm, c)     # [n, T, s]
                    term_2 = _gemm(a, w.reshape(c.shape[0], nt_ * s_)).reshape(
                        s_, nt_, s_).permute(1, 0, 2)
                    term_2 = term_2 + term_2.transpose(1, 2)
                    quad = torch.stack([_gemm_tn(t1.contiguous(), _gemm(nngp_dd, t1.contiguous()))
                                        for t1 in term_1])
                    cov = quad - term_2 + tt_k
            out[g] = Gaussian(mean, per_t(cov.contiguous()))
        return _gaussians(get, names, out)

    return predict_fn
