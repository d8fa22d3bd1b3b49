"""Explicit Runge–Kutta integration (time-integration/explicit.h,
integrator.h, advance.h).

`integrator_t` mirrors the reference's driver structure: the user supplies
calc_rhs(rhs, q, t) and bc(q, t); the state is kept primitive and every stage
update runs in conservative variables through the fused native RK-stage
kernel (integrate_advance with state_transform_t, advance.h:234-280).
`ssprk3_stepper` is the fused native SSPRK3 step (one C-ABI call per step,
optionally replayed from a captured CUDA graph).
"""
import ctypes
from fractions import Fraction as F

import torch

from . import _native
from .grid import grid_array, _stream, refined_layout_t


class rk_t:
    """Butcher table (A, b, c) as exact fractions (explicit.h:25-35)."""

    def __init__(self, A, b, c):
        self.A = [[F(x) for x in row] for row in A]
        self.b = [F(x) for x in b]
        self.c = [F(x) for x in c]
        self.stages = len(self.b)

    def diff_coeffs(self, prev, curr):
        """ratio_diff_t of two rows (advance.h:48-54, 85-95): the nonzero
        (index, value) pairs of curr - prev, value = num/den in FP64."""
        out = []
        for j in range(len(curr)):
            d = curr[j] - prev[j]
            if d != 0:
                out.append((j, float(d.numerator) / float(d.denominator)))
        return out


# explicit.h:36-116
rk2_t = rk_t([[0, 0], [F(1, 2), 0]], [0, 1], [0, F(1, 2)])
rk4_t = rk_t([[0, 0, 0, 0], [F(1, 2), 0, 0, 0], [0, F(1, 2), 0, 0], [0, 0, 1, 0]],
             [F(1, 6), F(1, 3), F(1, 3), F(1, 6)], [0, F(1, 2), F(1, 2), 1])
ssprk34_t = rk_t([[0, 0, 0, 0], [F(1, 2), 0, 0, 0], [F(1, 2), F(1, 2), 0, 0], [F(1, 6), F(1, 6), F(1, 6), 0]],
                 [F(1, 6), F(1, 6), F(1, 6), F(1, 2)], [0, F(1, 2), 1, F(1, 2)])
ssprk3_t = rk_t([[0, 0, 0], [1, 0, 0], [F(1, 4), F(1, 4), 0]],
                [F(1, 6), F(1, 6), F(2, 3)], [0, 1, F(1, 2)])
rk38r_t = rk_t([[0, 0, 0, 0], [F(1, 3), 0, 0, 0], [F(-1, 3), 1, 0, 0], [1, -1, 1, 0]],
               [F(1, 8), F(3, 8), F(3, 8), F(1, 8)], [0, F(1, 3), F(2, 3), 1])


class time_axis_t:
    """time_integration::time_axis_t(t0, dt)."""

    def __init__(self, t0, dt):
        self.t = float(t0)
        self.dt = float(dt)

    def time(self):
        return self.t

    def timestep(self):
        return self.dt


class integrator_data_t:
    """time_integration::integrator_data_t(q, rhs, scheme): the solution and
    one residual array per stage."""

    def __init__(self, q, rhs, scheme):
        self.q = q
        self.residuals = [rhs] + [grid_array(rhs.grid, 0.0, rhs.ng) for _ in range(scheme.stages - 1)]

    def solution(self):
        return self.q

    def residual(self, i):
        return self.residuals[i]


def rk_stage(q, gas, residuals, coeffs, stream=None):
    """One fused stage update q <- prim(cons(q) + sum_j coeffs[j] R_j)."""
    n = len(residuals)
    ptrs = (ctypes.c_void_p * max(n, 1))(*[r.ptr() for r in residuals])
    cf = (ctypes.c_double * max(n, 1))(*coeffs)
    _native.check(_native.lib().gbns_rk_stage(q.desc(), gas.desc(), q.ptr(), ptrs, cf, n, _stream(stream)))


class integrator_t:
    """time_integration::integrator_t(axis, scheme, data, calc_rhs, bc, trans)
    (integrator.h:18-59); advance() follows integrate_advance with the
    state transform (advance.h:234-280)."""

    def __init__(self, axis, scheme, data, calc_rhs, bc, trans):
        self.axis = axis
        self.scheme = scheme
        self.data = data
        self.calc_rhs = calc_rhs
        self.bc = bc
        self.trans = trans

    def solution(self):
        return self.data.q

    def time(self):
        return self.axis.t

    def advance(self):
        sch = self.scheme
        q = self.data.q
        dt = self.axis.dt
        gas = self.trans.gas
        t0 = self.axis.t
        self.calc_rhs(self.data.residual(0), q, t0 + float(sch.c[0]) * dt)
        for i in range(1, sch.stages):
            pairs = sch.diff_coeffs(sch.A[i - 1], sch.A[i])
            rk_stage(q, gas, [self.data.residual(j) for j, _ in pairs], [v * dt for _, v in pairs])
            ti = t0 + float(sch.c[i]) * dt
            self.bc(q, ti)
            self.calc_rhs(self.data.residual(i), q, ti)
        pairs = sch.diff_coeffs(sch.A[sch.stages - 1], sch.b)
        rk_stage(q, gas, [self.data.residual(j) for j, _ in pairs], [v * dt for _, v in pairs])
        self.axis.t = t0 + dt
        self.bc(q, self.axis.t)


class ssprk3_stepper:
    """Fused native SSPRK3 step of `q` (gbns_ssprk3_step): three flux_div
    launches with the stage update fused into their epilogue and three ghost
    fills per step, with the reference's arithmetic.  With use_graph=True the
    steps are replayed from a CUDA graph of one step that the library captures
    on first use (gbns_ssprk3_run; dt is fixed per graph)."""

    def __init__(self, q, scheme_desc, bc_desc, dt, use_graph=False):
        self.q = q
        self.scheme = scheme_desc
        self.bc = bc_desc
        self.dt = float(dt)
        n = 1
        for s in q.shape:
            n *= s
        self.work = torch.zeros(3 * n, dtype=torch.float64, device=q.data.device)
        self.use_graph = use_graph

    def step(self, nsteps=1, stream=None):
        st = _stream(stream)
        L = _native.lib()
        if self.use_graph:
            _native.check(L.gbns_ssprk3_run(self.q.desc(), self.scheme, self.bc, self.q.ptr(), self.work.data_ptr(),
                                            ctypes.c_double(self.dt), int(nsteps), st))
            return
        for _ in range(nsteps):
            _native.check(L.gbns_ssprk3_step(self.q.desc(), self.scheme, self.bc, self.q.ptr(), self.work.data_ptr(),
                                             ctypes.c_double(self.dt), st))

    def step_host(self, host_q, ngroups=0, stream=None, copy_stream=None):
        """One step of the state in `host_q` (a page-locked CPU tensor of
        q's shape, float64) through gbns_ssprk3_step_host: copied in block
        groups while stage 1 runs, copied back as stage 3 finishes each group;
        q's device array is the staging copy.  Asynchronous on `stream`."""
        if host_q.device.type != "cpu" or host_q.dtype != torch.float64 or tuple(host_q.shape) != tuple(self.q.shape):
            raise ValueError("host_q must be a float64 CPU tensor of the state's shape")
        if not host_q.is_contiguous():
            raise ValueError("host_q must be contiguous")
        st = _stream(stream)
        cs = None if copy_stream is None else _stream(copy_stream)
        _native.check(_native.lib().gbns_ssprk3_step_host(self.q.desc(), self.scheme, self.bc, host_q.data_ptr(),
                                                          self.q.ptr(), self.work.data_ptr(), ctypes.c_double(self.dt),
                                                          int(ngroups), st, cs))


class ssprk3_refined_stepper:
    """integrator_t with ssprk3_t on a refined layout (grid.refined_layout_t),
    the layout's exchange (grid.exchange_plan_t) as the boundary condition:
    one gbns_ssprk3_step_blocks per step, the stage updates fused into the
    flux launches.  q: a CUDA float64 tensor of the layout's shape holding
    exchanged ghosts (plan.exchange(q) before the first step, as the
    reference's driver refreshes them); bc (a gbns_bc_desc, optional): the
    wall faces filled after each exchange (gbns_wall_fill_blocks)."""

    def __init__(self, layout, q, scheme_desc, plan, dt, bc=None):
        if not isinstance(layout, refined_layout_t):
            raise TypeError("layout must be a grid.refined_layout_t")
        layout.check(q)
        if not q.is_cuda:
            raise ValueError("the refined-layout step runs on CUDA tensors")
        self.layout, self.q, self.scheme, self.plan, self.dt = layout, q, scheme_desc, plan, float(dt)
        self.bc = bc
        self.work = torch.zeros(3 * q.numel(), dtype=torch.float64, device=q.device)

    def step(self, nsteps=1, stream=None):
        for _ in range(nsteps):
            _native.check(_native.lib().gbns_ssprk3_step_blocks(
                self.layout.desc(), self.scheme, self.layout.boxes_ptr(), self.plan.handle, self.bc,
                ctypes.c_void_p(self.q.data_ptr()), ctypes.c_void_p(self.work.data_ptr()), ctypes.c_double(self.dt),
                _stream(stream)))
