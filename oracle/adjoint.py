"""CPU restatement of the differentiable form (test infrastructure only).

The forward step is the reference's time step, src/main.c:283-383 (velocity Dirichlet values,
wall vorticity DX v - DY u, Euler update of src/fluiddyn.c:98, Poisson solve with f = -w,
u = DY psi, v = -(DX psi)), with the derivative matrices built from the oracle's bands
(cnv_oracle.c, src/finitediff.c) and the Poisson equation of src/poisson.c solved exactly by a
dense factorisation: the answer the reference's SOR converges to. The backward step is the
discrete adjoint of that map, written with dense matrices; tests check it against finite
differences here, and the GPU adjoint kernels against it. Small grids only (dense n^2 x n^2
Poisson matrix).
"""
from __future__ import annotations

import numpy as np

import orc


class DenseStep:
    def __init__(self, n, order=6, Lx=1.0, Ly=1.0, re=400.0, dt=None, u_bc=(0.0, 0.0, 0.0), v_bc=(0.0, 0.0, 0.0, 0.0)):
        self.n = n
        self.dx, self.dy = Lx / n, Ly / n
        self.re = re
        self.dt = dt
        self.u_bc = u_bc          # u1, u2, u3 (j = 0, j = n-1, i = 0); the lid u4 is an argument
        self.v_bc = v_bc
        self.D1x = self._dense(orc.fd_band(n, order, 1, self.dx))
        self.D1y = self._dense(orc.fd_band(n, order, 1, self.dy))
        self.D2x = self._dense(orc.fd_band(n, order, 2, self.dx))
        self.D2y = self._dense(orc.fd_band(n, order, 2, self.dy))
        m = n - 2
        T = np.diag(np.ones(m - 1), 1) + np.diag(np.ones(m - 1), -1)
        I = np.eye(m)
        dx2, dy2 = self.dx * self.dx, self.dy * self.dy
        # den psi - dy^2 (up + down) - dx^2 (left + right) = c4 w   (src/poisson.c:247 at convergence)
        self.M = 2 * (dx2 + dy2) * np.kron(I, I) - dy2 * np.kron(T, I) - dx2 * np.kron(I, T)
        self.c4 = dx2 * dy2
        self.edge = np.zeros((n, n), bool)
        self.edge[0] = self.edge[-1] = True
        self.edge[:, 0] = self.edge[:, -1] = True

    def _dense(self, band):
        n = self.n
        D = np.zeros((n, n))
        for r in range(n):
            for o in range(-3, 4):
                if 0 <= r + o < n:
                    D[r, r + o] = band[r, o + 3]
        return D

    # operators on row-major fields (i = row); DX acts along j, DY along i
    def DX(self, x, D=None):
        return x @ (self.D1x if D is None else D).T

    def DY(self, x, D=None):
        return (self.D1y if D is None else D) @ x

    def solve(self, rhs):
        n, m = self.n, self.n - 2
        out = np.zeros((n, n))
        out[1:-1, 1:-1] = (self.c4 * np.linalg.solve(self.M, rhs[1:-1, 1:-1].ravel())).reshape(m, m)
        return out

    def bc(self, u, v, lid):
        ub, vb = u.copy(), v.copy()
        ub[0, :], ub[-1, :] = self.u_bc[2], lid     # rows first, then the columns (corners: u1/u2)
        ub[:, 0], ub[:, -1] = self.u_bc[0], self.u_bc[1]
        vb[0, :], vb[-1, :] = self.v_bc[2], self.v_bc[3]
        vb[:, 0], vb[:, -1] = self.v_bc[0], self.v_bc[1]
        return ub, vb

    def step(self, w, u, v, lid):
        ub, vb = self.bc(u, v, lid)
        wb = np.where(self.edge, self.DX(vb) - self.DY(ub), w)
        wn = (-ub * self.DX(wb) - vb * self.DY(wb) + (1 / self.re) * (self.DX(wb, self.D2x) + self.DY(wb, self.D2y))) \
            * self.dt + wb
        psi = self.solve(wn)
        return wn, self.DY(psi), -self.DX(psi), (wb, ub, vb)

    def run(self, w0, lid, nsteps, ui=0.0, vi=0.0):
        n = self.n
        w = w0.copy()
        u, v = np.zeros((n, n)), np.zeros((n, n))
        u[1:-1, 1:-1], v[1:-1, 1:-1] = ui, vi
        tape = []
        for _ in range(nsteps):
            w, u, v, t = self.step(w, u, v, lid)
            tape.append(t)
        return w, tape

    def backward(self, g_final, tape):
        """dJ/dw0 and dJ/dlid for dJ/dw(T) = g_final."""
        n = self.n
        lw, lu, lv = g_final.copy(), np.zeros((n, n)), np.zeros((n, n))
        glid = 0.0
        E = self.edge
        for wb, ub, vb in reversed(tape):
            lpsi = self.D1y.T @ lu - lv @ self.D1x
            lam = lw + self.solve(lpsi)            # M is symmetric: the adjoint solve is the solve
            lwb = lam + self.dt * (-(ub * lam) @ self.D1x - self.D1y.T @ (vb * lam)
                                   + (1 / self.re) * (lam @ self.D2x + self.D2y.T @ lam))
            lub = -self.dt * self.DX(wb) * lam
            lvb = -self.dt * self.DY(wb) * lam
            lwe = np.where(E, lwb, 0.0)
            lub = lub - self.D1y.T @ lwe
            lvb = lvb + lwe @ self.D1x
            glid += float(lub[-1, 1:-1].sum())
            lw, lu, lv = np.where(E, 0.0, lwb), np.where(E, 0.0, lub), np.where(E, 0.0, lvb)
        return lw, glid

    def enstrophy_gradient(self, w0, lid, nsteps):
        wT, tape = self.run(w0, lid, nsteps)
        h2 = self.dx * self.dy
        gw, glid = self.backward(h2 * wT, tape)
        return 0.5 * h2 * float(np.sum(wT * wT)), gw, glid
