"""Adjoint of the device linear solve, and differentiation through backward-
Euler time stepping with checkpointing.

The reference has no adjoint; this module builds one on the C ABI:

* :class:`DiffusionSolve` owns a finite-volume diffusion operator assembled on
  the device from face coefficients (``fs_fv_assemble``), a bound Jacobi-PCG
  solver, and the adjoint: ``A^T lambda = dL/dx`` by the same solver on the
  transposed operator (``fs_krylov_apply_transpose``), ``dL/db = lambda`` and
  ``dL/dc = fs_fv_face_grad(lambda, x)``.
* :class:`LinearSolve` is the ``torch.autograd.Function`` over it (CUDA float64
  tensors in and out, no copies: the library wraps the tensors' memory).
* :func:`heat_loss_and_grad` differentiates a backward-Euler heat equation
  ``(I + dt K(c)) u_{k+1} = u_k`` through all steps, storing the state every
  ``checkpoint`` steps and recomputing each segment during the reverse sweep.
"""
from __future__ import annotations

import numpy as np

from . import api as fs
from . import problems as P
from ._lib import check, lib


class DiffusionSolve:
    """x = A(c)^-1 b for the n^dim finite-volume diffusion operator with face
    coefficients c (layout of :mod:`problems`), with its adjoint."""

    def __init__(self, ctx: fs.Context, dim: int, n: int, rtol: float = 1e-12,
                 maxiter: int = 20000, scale: float = 1.0, shift: float = 0.0):
        self.ctx, self.dim, self.n = ctx, dim, n
        self.scale, self.shift = scale, shift
        self.N = n ** dim
        self.nfaces = P.grid_faces(dim, n)
        pattern = P.assemble_diffusion(dim, n, P.faces_const(dim, n, 1.0))
        self.A = fs.CSR(ctx, pattern)
        self.faces = fs.Vector(ctx, self.nfaces)
        s = fs.cg.settings(maxiter=maxiter, rtol=rtol, use_zero_guess=True)
        self.solver = fs.cg.solver(s)(self.A, fs.op.jacobi)
        self.lam = fs.Vector(ctx, self.N)
        self.gfaces = fs.Vector(ctx, self.nfaces)

    def set_faces(self, faces):
        """faces: numpy array or device Vector of length nfaces."""
        if isinstance(faces, fs.Vector):
            self.faces.copy(faces)
        else:
            self.faces.upload(np.ascontiguousarray(faces, dtype=np.float64))
        self.A.fv_assemble(self.dim, self.n, self.faces, self.scale, self.shift)

    def solve(self, b: fs.Vector, x: fs.Vector):
        info = self.solver(b, x)
        if not info.success():
            raise RuntimeError(f"forward solve did not converge: {info}")
        return info

    def adjoint(self, gx: fs.Vector, x: fs.Vector, gfaces: fs.Vector | None = None,
                accumulate: bool = False, face_scale: float | None = None):
        """lambda = A^-T gx; gfaces (+)= dL/dc.  Returns lambda (= dL/db)."""
        info = self.solver.apply_transpose(gx, self.lam)
        if not info.success():
            raise RuntimeError(f"adjoint solve did not converge: {info}")
        g = gfaces if gfaces is not None else self.gfaces
        sc = self.scale if face_scale is None else face_scale
        check(lib().fs_fv_face_grad(self.ctx.h, self.dim, self.n, self.lam.h, x.h, sc,
                                    1 if accumulate else 0, g.h), self.ctx.h, "face grad")
        return self.lam


def _wrap(ctx, t):
    """fs Vector viewing a contiguous CUDA float64 torch tensor."""
    assert t.is_cuda and t.dtype.is_floating_point and t.element_size() == 8 and t.is_contiguous()
    return fs.Vector.wrap(ctx, t.numel(), t.data_ptr())


def LinearSolve():
    """The ``torch.autograd.Function`` x = A(c)^-1 b (built lazily so that the
    module imports without torch)."""
    import torch

    class _LinearSolve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, faces, b, system: DiffusionSolve):
            torch.cuda.synchronize()
            x = torch.empty_like(b)
            system.set_faces(_wrap(system.ctx, faces.detach().contiguous()))
            system.solve(_wrap(system.ctx, b.detach().contiguous()), _wrap(system.ctx, x))
            ctx.system = system
            ctx.save_for_backward(faces, x)
            return x

        @staticmethod
        def backward(ctx, gx):
            system = ctx.system
            faces, x = ctx.saved_tensors
            torch.cuda.synchronize()
            system.set_faces(_wrap(system.ctx, faces.detach().contiguous()))
            gfaces = torch.empty_like(faces)
            lam = system.adjoint(_wrap(system.ctx, gx.contiguous()), _wrap(system.ctx, x),
                                 _wrap(system.ctx, gfaces))
            gb = torch.empty_like(x)
            _wrap(system.ctx, gb).copy(lam)
            system.ctx.sync()
            return gfaces, gb, None

    return _LinearSolve


# --------------------------------------------------------------- heat ---

def checkpoint_segments(nsteps: int, every: int):
    """The reverse sweep's segments [(s0, s1), ...], last first: the state
    u_{s0} is stored during the forward pass and u_{s0+1} .. u_{s1} are
    recomputed from it."""
    if nsteps <= 0:
        return []
    if every <= 0:
        raise ValueError("checkpoint interval must be positive")
    return [(s0, min(s0 + every, nsteps)) for s0 in range(((nsteps - 1) // every) * every, -1, -every)]


def heat_forward(system: DiffusionSolve, u0: np.ndarray, nsteps: int, checkpoint: int = 0):
    """Backward Euler (I + dt K) u_{k+1} = u_k (system assembled with
    scale = dt, shift = 1).  Returns u_N and {step: state} checkpoints."""
    ctx = system.ctx
    u = fs.Vector(ctx, u0)
    un = fs.Vector(ctx, system.N)
    ckpt = {}
    for k in range(nsteps):
        if checkpoint and k % checkpoint == 0:
            ckpt[k] = u.numpy()
        system.solve(u, un)
        u, un = un, u
    return u, ckpt


def heat_loss_and_grad(system: DiffusionSolve, faces: np.ndarray, u0: np.ndarray,
                       target: np.ndarray, nsteps: int, checkpoint: int):
    """L = ||u_N - target||^2 through nsteps backward-Euler steps; returns
    (L, dL/dfaces, dL/du0) by the discrete adjoint with checkpoints every
    `checkpoint` steps (each segment is recomputed from its checkpoint during
    the reverse sweep, so at most nsteps / checkpoint + checkpoint states are
    held)."""
    ctx = system.ctx
    system.set_faces(faces)
    uN, ckpt = heat_forward(system, u0, nsteps, checkpoint)
    d = uN.numpy() - target
    L = float(d @ d)
    lam = fs.Vector(ctx, 2.0 * d)                 # dL/du_N
    gfaces = fs.Vector(ctx, system.nfaces)
    gfaces.zero()
    states = [fs.Vector(ctx, system.N) for _ in range(checkpoint + 1)]
    for s0, s1 in checkpoint_segments(nsteps, checkpoint):
        # recompute u_{s0} .. u_{s1} from the checkpoint
        states[0].upload(ckpt[s0])
        for k in range(s0, s1):
            system.solve(states[k - s0], states[k - s0 + 1])
        # reverse sweep: u_{k+1} = M^-1 u_k  =>  mu = M^-T lam,
        # dL/dc += -dt mu^T dK/dc u_{k+1},  dL/du_k = mu
        for k in range(s1 - 1, s0 - 1, -1):
            mu = system.adjoint(lam, states[k - s0 + 1], gfaces, accumulate=True)
            lam.copy(mu)
    return L, gfaces.numpy(), lam.numpy()


# ------------------------------------------------------- face helpers ---

def face_cells(dim: int, n: int, f):
    """Cells (a, b) on the lower / upper side of faces f (-1 on a boundary
    side), in the face layout of the generator: x-faces, then y-faces, then
    z-faces, each with the normal index running over n + 1 positions."""
    f = np.asarray(f, dtype=np.int64)
    a = np.full(f.shape, -1, np.int64)
    b = np.full(f.shape, -1, np.int64)
    if dim == 2:
        nx = n * (n + 1)
        m = f < nx
        j, fi = f[m] // (n + 1), f[m] % (n + 1)
        a[m] = np.where(fi > 0, j * n + fi - 1, -1)
        b[m] = np.where(fi < n, j * n + fi, -1)
        q = f[~m] - nx
        fj, i = q // n, q % n
        a[~m] = np.where(fj > 0, (fj - 1) * n + i, -1)
        b[~m] = np.where(fj < n, fj * n + i, -1)
        return a, b
    nx = n * n * (n + 1)
    m0, m1 = f < nx, (f >= nx) & (f < 2 * nx)
    m2 = f >= 2 * nx
    row, fi = f[m0] // (n + 1), f[m0] % (n + 1)
    a[m0] = np.where(fi > 0, row * n + fi - 1, -1)
    b[m0] = np.where(fi < n, row * n + fi, -1)
    q = f[m1] - nx
    i, t = q % n, q // n
    fj, k = t % (n + 1), t // (n + 1)
    a[m1] = np.where(fj > 0, (k * n + fj - 1) * n + i, -1)
    b[m1] = np.where(fj < n, (k * n + fj) * n + i, -1)
    q = f[m2] - 2 * nx
    i, t = q % n, q // n
    j, fk = t % n, t // n
    a[m2] = np.where(fk > 0, ((fk - 1) * n + j) * n + i, -1)
    b[m2] = np.where(fk < n, (fk * n + j) * n + i, -1)
    return a, b


def face_delta_apply(dim: int, n: int, f, dc, x: np.ndarray) -> np.ndarray:
    """K(dc) x for a face-coefficient change dc that is nonzero only on the
    faces f (K is linear in the coefficients): each interior face adds
    dc (x_a - x_b) to row a and the negative to row b, a boundary face adds
    dc x_c to its one cell."""
    f = np.atleast_1d(np.asarray(f, np.int64))
    dc = np.broadcast_to(np.asarray(dc, np.float64), f.shape)
    a, b = face_cells(dim, n, f)
    y = np.zeros_like(x)
    for fa, fb, d in zip(a, b, dc):
        if fa >= 0 and fb >= 0:
            v = d * (x[fa] - x[fb])
            y[fa] += v
            y[fb] -= v
        else:
            c = fa if fa >= 0 else fb
            y[c] += d * x[c]
    return y
