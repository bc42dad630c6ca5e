"""Closed-form shallow-water solutions and the cell averages that start a run
from them (the reference's test layer, examples/Tests.h:9-280, and its
initial-condition recipe, examples/Main.cpp:198-222).

Every solution gives the bed b(x, y), the depth h(x, y, t) and the velocity
(u, v)(x, y, t); w = h + b, hu = h u, hv = h v as in Test (Tests.h:9-30).
g = 1.  Coriolis ``cor`` and friction ``tau`` enter the solutions as in the
reference; the step itself runs with friction off (the reference never applies
it, src/TimeDisc.cpp:38-39).

``initial_state`` averages (h, u, v) over each cell with the TriangAverage
quadrature and adds the cell's bathymetry, like the reference's Process().
"""
from __future__ import annotations

import math

import numpy as np

from .mesh import Mesh, triang_average

__all__ = ["Solution", "LakeAtRest", "Ball", "ConservativeThacker", "SolenoidalThacker", "ClassicThacker",
           "cell_averages", "initial_state"]

WET_TOL = 1e-13  # include/Includes.h:30


class Solution:
    """Interface of a closed-form solution; subclasses give b, h, u, v."""

    cor = 0.0
    tau = 0.0

    def b(self, x, y):
        raise NotImplementedError

    def h(self, x, y, t):
        raise NotImplementedError

    def u(self, x, y, t):
        raise NotImplementedError

    def v(self, x, y, t):
        raise NotImplementedError

    def w(self, x, y, t):
        return self.h(x, y, t) + self.b(x, y)

    def hu(self, x, y, t):
        return self.h(x, y, t) * self.u(x, y, t)

    def hv(self, x, y, t):
        return self.h(x, y, t) * self.v(x, y, t)

    def is_wet(self, x, y, t):
        return self.h(x, y, t) >= WET_TOL


class LakeAtRest(Solution):
    """Still water over a bed of -0.2 on (1, 3)^2 and -1 elsewhere, surface at
    0 (Tests.h:32-43)."""

    def b(self, x, y):
        inside = (1.0 < x) & (x < 3.0) & (1.0 < y) & (y < 3.0)
        return np.where(inside, -0.2, -1.0)

    def h(self, x, y, t):
        return np.maximum(0.0, -self.b(x, y))

    def u(self, x, y, t):
        return np.zeros_like(np.asarray(x, dtype=np.float64))

    def v(self, x, y, t):
        return np.zeros_like(np.asarray(x, dtype=np.float64))


class _Bowl(Solution):
    """Paraboloid bed delta ((x - xm)^2 + (y - ym)^2 - 1) (Tests.h:46-57)."""

    def __init__(self, delta, mid=(0.0, 0.0), cor=0.0, tau=0.0):
        self.delta, self.xm, self.ym, self.cor, self.tau = delta, mid[0], mid[1], cor, tau

    def b(self, x, y):
        return self.delta * ((x - self.xm) ** 2 + (y - self.ym) ** 2 - 1.0)


class Ball(_Bowl):
    """A rigid water cap sliding in the bowl (Tests.h:60-133): its centre
    follows a damped, rotating oscillation set by (x0, y0, u0, v0)."""

    def __init__(self, delta, x0, y0, u0, v0, mid=(0.0, 0.0), cor=0.0, tau=0.0):
        super().__init__(delta, mid, cor, tau)
        X, Y = x0 - self.xm, y0 - self.ym
        l1 = 2.0 * delta - 0.25 * tau * tau + 0.25 * cor * cor
        l2 = 0.5 * cor * tau
        s = l1 + math.sqrt(l1 * l1 + l2 * l2)
        self.beta = 0.5 * math.sqrt(2.0 * s)
        self.alpha = l2 / math.sqrt(2.0 * s)
        al, be = self.alpha, self.beta
        n = al * al + be * be
        d = al * al + be * be + 0.5 * al * tau + 0.5 * be * cor
        e = be * tau - al * cor
        self.a1 = (0.5 * d * X + 0.25 * e * Y + 0.5 * (al * u0 + be * v0)) / n
        self.a2 = (0.5 * d * Y - 0.25 * e * X + 0.5 * (al * v0 - be * u0)) / n
        self.a3, self.a4 = X - self.a1, Y - self.a2

    def _modes(self, t):
        """(phi-, phi+, psi-, psi+) at time t."""
        gm = math.exp(-(0.5 * self.tau - self.alpha) * t)
        gp = math.exp(-(0.5 * self.tau + self.alpha) * t)
        om, op = (0.5 * self.cor - self.beta) * t, (0.5 * self.cor + self.beta) * t
        phim = gm * (self.a1 * math.cos(om) + self.a2 * math.sin(om))
        phip = gp * (self.a3 * math.cos(op) + self.a4 * math.sin(op))
        psim = gm * (self.a2 * math.cos(om) - self.a1 * math.sin(om))
        psip = gp * (self.a4 * math.cos(op) - self.a3 * math.sin(op))
        return phim, phip, psim, psip

    def h(self, x, y, t):
        phim, phip, psim, psip = self._modes(t)
        fx = x - self.xm - phip - phim
        fy = y - self.ym - psip - psim
        return np.maximum(0.0, self.delta * (1.0 - fx * fx - fy * fy))

    def _velocity(self, t):
        phim, phip, psim, psip = self._modes(t)
        cp, cm = 0.5 * self.cor + self.beta, 0.5 * self.cor - self.beta
        dp, dm = 0.5 * self.tau + self.alpha, 0.5 * self.tau - self.alpha
        uu = cp * psip - dp * phip + cm * psim - dm * phim
        vv = -cp * phip - dp * psip - cm * phim - dm * psim
        return uu, vv

    def u(self, x, y, t):
        return np.where(self.is_wet(x, y, t), self._velocity(t)[0], 0.0)

    def v(self, x, y, t):
        return np.where(self.is_wet(x, y, t), self._velocity(t)[1], 0.0)


class _Thacker(_Bowl):
    """Linear velocity, quadratic depth (Tests.h:135-162):
    u = p X + q Y, h = max(0, Hc + Hxx X^2 / 2 + Hxy X Y + Hyy Y^2 / 2)
    with X = x - xm, Y = y - ym."""

    def __init__(self, delta, H0, p0, q0, mid=(0.0, 0.0), cor=0.0, tau=0.0):
        super().__init__(delta, mid, cor, tau)
        self.H0, self.p0, self.q0 = H0, p0, q0

    def u(self, x, y, t):
        return self.p(t) * (x - self.xm) + self.q(t) * (y - self.ym)

    def h(self, x, y, t):
        X, Y = x - self.xm, y - self.ym
        r = self.Hc(t) + 0.5 * self.Hxx(t) * X * X + self.Hxy(t) * X * Y + 0.5 * self.Hyy(t) * Y * Y
        return np.maximum(0.0, r)


class ConservativeThacker(_Thacker):
    """Tests.h:165-197: a rotating elliptic solution with constant Hc."""

    def __init__(self, delta, H0, p0, q0, mid=(0.0, 0.0), cor=0.0, tau=0.0):
        super().__init__(delta, H0, p0, q0, mid, cor, tau)
        self.a = p0 * p0 + q0 * q0
        self.om = math.sqrt(0.25 * cor * cor + 2.0 * self.a + 4.0 * delta) + 0.5 * cor

    def p(self, t):
        return self.p0 * math.cos(self.om * t) + self.q0 * math.sin(self.om * t)

    def q(self, t):
        return self.q0 * math.cos(self.om * t) - self.p0 * math.sin(self.om * t)

    def v(self, x, y, t):
        return self.q(t) * (x - self.xm) - self.p(t) * (y - self.ym)

    def Hc(self, t):
        return self.H0

    def Hxx(self, t):
        return -self.a - self.q(t) * (self.om - self.cor) - 2.0 * self.delta

    def Hxy(self, t):
        return self.p(t) * (self.om - self.cor)

    def Hyy(self, t):
        return -self.a + self.q(t) * (self.om - self.cor) - 2.0 * self.delta


class SolenoidalThacker(_Thacker):
    """Tests.h:199-235: a steady (or frictionally decaying) vortex; without
    Coriolis and friction it solves the equations for p0 = 0 and any q0."""

    def p(self, t):
        return self.p0 * math.exp(-self.tau * t)

    def q(self, t):
        return self.q0 * math.exp(-self.tau * t)

    def v(self, x, y, t):
        return -self.q(t) * (x - self.xm) - self.p(t) * (y - self.ym)

    def Hc(self, t):
        return self.H0

    def Hxx(self, t):
        if self.tau != 0:
            return 0.0
        return self.q0 * self.q0 - self.p0 * self.p0 - self.q0 * self.cor - 2.0 * self.delta

    def Hxy(self, t):
        return self.p0 * self.cor

    def Hyy(self, t):
        return self.Hxx(t)


class ClassicThacker(_Thacker):
    """Tests.h:237-280: the periodic parabolic-bowl solution."""

    def __init__(self, delta, H0, p0=0.0, q0=0.0, mid=(0.0, 0.0), cor=0.0, tau=0.0):
        super().__init__(delta, H0, p0, q0, mid, cor, tau)
        self.om = math.sqrt(cor * cor + 8.0 * delta)
        qz = (q0 - 0.5 * cor) ** 2
        rz = qz + 2.0 * H0 * H0 + p0 * p0 - 0.25 * self.om ** 2
        self.a = math.sqrt(rz * rz + (self.om * p0) ** 2) / (rz + 0.5 * self.om ** 2)
        self.phase = math.atan(self.om * p0 / rz)

    def _den(self, t):
        return 1.0 - self.a * math.cos(self.om * t + self.phase)

    def p(self, t):
        return 0.5 * self.om * self.a * math.sin(self.om * t + self.phase) / self._den(t)

    def q(self, t):
        return (self.q0 - 0.5 * self.cor) * (1.0 - self.a * math.cos(self.phase)) / self._den(t) + 0.5 * self.cor

    def v(self, x, y, t):
        return -self.q(t) * (x - self.xm) + self.p(t) * (y - self.ym)

    def Hc(self, t):
        return self.H0 * (1.0 - self.a * math.cos(self.phase)) / self._den(t)

    def Hxx(self, t):
        qz = (self.q0 - 0.5 * self.cor) ** 2
        az0 = (1.0 - self.a * math.cos(self.phase)) ** 2
        return (0.25 * self.om ** 2 * (self.a * self.a - 1.0) + qz * az0) / self._den(t) ** 2

    def Hxy(self, t):
        return 0.0

    def Hyy(self, t):
        return self.Hxx(t)

    def period(self):
        return 2.0 * math.pi / self.om


def cell_averages(mesh: Mesh, sol: Solution, t: float, n: int = 100, chunk: int = 2048) -> np.ndarray:
    """(C, 3): the TriangAverage<3, n> of (h, hu, hv) of the solution over every cell."""
    p = mesh.geometry[mesh.cell_nodes]
    out = np.zeros((mesh.num_cells, 3))
    for s in range(0, mesh.num_cells, chunk):
        sl = slice(s, s + chunk)

        def f(x, y):
            return np.stack([sol.h(x, y, t), sol.hu(x, y, t), sol.hv(x, y, t)])

        out[sl] = triang_average(p[sl, 0], p[sl, 1], p[sl, 2], f, n).T
    return out


def initial_state(mesh: Mesh, sol: Solution, t: float = 0.0, n: int = 100, chunk: int = 2048) -> np.ndarray:
    """(C, 3) primitive state (w, u, v): the cell averages of (h, u, v) with the
    cell's centroid bathymetry added to h (examples/Main.cpp:209-221)."""
    p = mesh.geometry[mesh.cell_nodes]
    out = np.zeros((mesh.num_cells, 3))
    for s in range(0, mesh.num_cells, chunk):
        sl = slice(s, s + chunk)

        def f(x, y):
            one = np.ones_like(x)
            return np.stack([sol.h(x, y, t), sol.u(x, y, t) * one, sol.v(x, y, t) * one])

        out[sl] = triang_average(p[sl, 0], p[sl, 1], p[sl, 2], f, n).T
    out[:, 0] += mesh.centroids()[:, 2]
    return out
