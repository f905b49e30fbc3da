"""femx's Python surface for the time residual, over the GPU assembly path.

femx's Python module (`femx._core`, python/bindings/State.cpp:649-667, and
its trampoline PyTimeResidual, State.cpp:259-460) exposes ``TimeDims``,
``VariableBlock`` and ``TimeResidual``; a residual is an object with
``dims()``, ``residual(ctx)``, ``assemble_next(ctx)``,
``apply_jacobian_transpose(ctx, wrt, adj)``, ``initial_state(prm)`` and
``prepare_linear_solve(ctx, jac, rhs)``, where ``ctx`` is the dict femx
builds (``step``, ``next_state``, ``parameters``, ``history`` — lag-major,
shape (num_hist, num_states); ctxData, State.cpp:249-257).

This module keeps those names and that protocol, and adds
``NavierTimeResidual``: femx's GLS Navier-Stokes operator (NavierOperator,
femx/model/ns/Components.hpp:330-577) with the behaviour of femx's own
NavierResidual (femx/model/ns/NavierStokesModel.cpp:374-543), computed by
libgbfem on the GPU. Vectors are CUDA float64 tensors (numpy arrays are
copied to the device); ``assemble_next`` returns the next-state Jacobian as
a CSR matrix on the device (femx's Python protocol returns a dense host
array, State.cpp:372-401, which does not scale to GPU-sized meshes).

femx builds `_core` with pybind11; the GPU machine's Python has no pybind11, so
this surface is plain Python over the library's C ABI (ctypes).
"""
from __future__ import annotations

import numpy as np
import torch

from . import assembly as A
from . import meshes

__all__ = ["TimeDims", "VariableBlock", "TimeResidual", "NavierTimeResidual"]


class TimeDims:
    """femx::state::TimeDims (femx/state/TimeResidual.hpp:13-21)."""

    def __init__(self, num_steps=0, num_states=0, num_param=0, num_res=0, num_hist=1):
        self.num_steps = int(num_steps)
        self.num_states = int(num_states)
        self.num_param = int(num_param)
        self.num_res = int(num_res)
        self.num_hist = int(num_hist)

    def __repr__(self):
        return (f"TimeDims(num_steps={self.num_steps}, num_states={self.num_states}, "
                f"num_param={self.num_param}, num_res={self.num_res}, "
                f"num_hist={self.num_hist})")


class VariableBlock:
    """femx::state::VariableBlock (femx/state/TimeResidual.hpp:93-166) with
    femx's Python names: ``VariableBlock.history(lag)``, ``is_history_state``,
    ``is_parameter``, ``history_lag``; ``next_state()`` and ``parameter()``
    build the other two kinds."""

    _HIST, _NEXT, _PARAM = 0, 1, 2

    def __init__(self, kind=0, lag=0):
        self._kind, self._lag = int(kind), int(lag)

    @staticmethod
    def history(lag):
        return VariableBlock(VariableBlock._HIST, lag)

    @staticmethod
    def next_state():
        return VariableBlock(VariableBlock._NEXT)

    @staticmethod
    def parameter():
        return VariableBlock(VariableBlock._PARAM)

    @property
    def is_history_state(self):
        return self._kind == self._HIST

    @property
    def is_next_state(self):
        return self._kind == self._NEXT

    @property
    def is_parameter(self):
        return self._kind == self._PARAM

    @property
    def history_lag(self):
        return self._lag


class TimeResidual:
    """Base of femx's Python time residuals (PyTimeResidual's contract):
    subclasses implement dims(), residual(ctx), assemble_next(ctx) and
    apply_jacobian_transpose(ctx, wrt, adj); initial_state(prm) defaults to
    zeros and prepare_linear_solve(ctx, jac, rhs) to leaving rhs as it is
    (State.cpp:281-294, 410-445)."""

    def dims(self) -> TimeDims:
        raise NotImplementedError("TimeResidual.dims() is not implemented")

    def initial_state(self, prm):
        return torch.zeros(self.dims().num_states, dtype=torch.float64, device="cuda")

    def residual(self, ctx):
        raise NotImplementedError("TimeResidual.residual() is not implemented")

    def assemble_next(self, ctx):
        raise NotImplementedError("TimeResidual.assemble_next() is not implemented")

    def apply_jacobian_transpose(self, ctx, wrt, adj):
        raise NotImplementedError("TimeResidual.apply_jacobian_transpose() is not implemented")

    def prepare_linear_solve(self, ctx, jac, rhs):
        return None


def _vec(x, n, what):
    t = x if torch.is_tensor(x) else torch.from_numpy(np.asarray(x))
    t = t.to(device="cuda", dtype=torch.float64).reshape(-1).contiguous()
    if t.numel() != n:
        raise RuntimeError(f"Navier residual {what} size mismatch")
    return t


class NavierTimeResidual(TimeResidual):
    """femx's GLS Navier-Stokes time residual on the GPU: P1/P1 on triangles
    in femx's mixed DOF layout (velocity 2 node + comp, then pressure),
    Crank-Nicolson with AB2 advection after the first step, two history
    lags, no parameters (femx's NavierResidual). coords: node coordinates
    (N, 2); conn: triangles (E, 3)."""

    NUM_HIST = 2

    def __init__(self, coords, conn, rho, mu, dt, num_steps):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        offs, dofs, nd = meshes.navier_elem_dofs(conn, coords.shape[0])
        d = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
        self.amap = A.makeAssemblyMap(nd, nd, d(offs), d(dofs), d(offs), d(dofs))
        self.coords, self.conn = d(coords), d(conn)
        self.rho, self.mu, self.dt = float(rho), float(mu), float(dt)
        self.num_steps = int(num_steps)
        self._hist_grad = torch.empty(self.NUM_HIST * nd, dtype=torch.float64, device="cuda")

    def dims(self) -> TimeDims:
        n = self.amap.numStates()
        return TimeDims(self.num_steps, n, 0, self.amap.numRes(), self.NUM_HIST)

    def pattern(self):
        return self.amap.pattern()

    def initial_state(self, prm):
        if prm is not None and len(prm) != 0:
            raise RuntimeError("Navier physics residual is parameter-free")
        return super().initial_state(prm)

    def _ctx(self, ctx):
        # femx's NavierResidual::checkCtx (NavierStokesModel.cpp:550-558)
        n = self.amap.numStates()
        step = int(ctx["step"])
        if not (0 <= step < self.num_steps):
            raise RuntimeError("Navier residual step is out of range")
        prm = ctx.get("parameters")
        hist = ctx["history"]
        hist = hist if torch.is_tensor(hist) else torch.from_numpy(np.asarray(hist))
        if (prm is not None and len(prm) != 0) or hist.numel() < self.NUM_HIST * n \
                or hist.numel() % max(n, 1) != 0:
            raise RuntimeError("Navier residual vector size mismatch")
        hist = _vec(hist.reshape(-1)[:self.NUM_HIST * n], self.NUM_HIST * n, "history")
        return step, hist, _vec(ctx["next_state"], n, "next state")

    def residual(self, ctx):
        step, hist, nxt = self._ctx(ctx)
        res = torch.empty(self.amap.numRes(), dtype=torch.float64, device="cuda")
        A.assembleNavier(self.amap, self.coords, self.conn, self.rho, self.mu, self.dt, step,
                         hist, nxt, res, None, num_hist=self.NUM_HIST)
        return res

    def assemble_next(self, ctx):
        """The next-state Jacobian (CSR on the device) and the residual."""
        step, hist, nxt = self._ctx(ctx)
        res = torch.empty(self.amap.numRes(), dtype=torch.float64, device="cuda")
        jac = A.CsrMatrix(self.amap.pattern())
        A.assembleNavier(self.amap, self.coords, self.conn, self.rho, self.mu, self.dt, step,
                         hist, nxt, res, jac, num_hist=self.NUM_HIST)
        return jac, res

    def apply_jacobian_transpose(self, ctx, wrt, adj):
        step, hist, nxt = self._ctx(ctx)
        if wrt.is_next_state:
            raise RuntimeError("Navier transpose apply supports only history and parameter blocks")
        adj = _vec(adj, self.amap.numRes(), "adjoint")
        if wrt.is_parameter:
            return torch.empty(0, dtype=torch.float64, device="cuda")
        if not (0 <= wrt.history_lag < self.NUM_HIST):
            raise RuntimeError("Navier residual history lag is out of range")
        A.vjpNavierHist(self.amap, self.coords, self.conn, self.rho, self.mu, self.dt, step,
                        hist, nxt, adj, self._hist_grad, num_hist=self.NUM_HIST)
        n = self.amap.numStates()
        return self._hist_grad[wrt.history_lag * n:(wrt.history_lag + 1) * n].clone()
