"""CPU restatement of FC 1's crack-tip evaluation (2D): SIFs by the interaction
integral and the growth decision.  Test infrastructure (the checker), not part of
the product; it follows

  b_cracPropag_qusiaStatic_BYKeq        SourceFiles/Solver/pdsolve.cpp:7375-7495
  SIFsAndPropaDire_GaussPointPDnode     pdsolve.cpp:8514-8679  (path points)
  Jintegrand_GPPDN                      pdsolve.cpp:8681-8869  (chord integrals)
  DispGradAndStressAndPqPx_FEM          pdsolve.cpp:8303-8408  (FE centre fields)
  DispGrad                              pdsolve.cpp:3254-3315  (PD node gradient)

in numpy, from a host-only pdx.Model's set-up arrays, the oracle's PDLSM
coefficients (orc.Oracle.coeffs: g per bond) and node stresses
(orc.Oracle.stress).  The block grid, element order and node order are the
reference's, so the path and its sort order are the same.
"""
from __future__ import annotations

import math

import numpy as np


class Fc1Oracle:
    def __init__(self, model, oracle, mr: float = 6.0, dcf: float = 1.0):
        self.X = model.array("X").reshape(-1, 3)
        self.conn = model.array("conn").reshape(-1, 8)
        self.nn = model.array("elem_nn")
        self.n_elem = len(self.nn)
        pde = set(model.array("pde_idx").tolist())
        self.algo = np.array([1 if e in pde else 2 for e in range(self.n_elem)])
        geom = model.array("geom")
        self.min_delta, self.block, self.lbc, self.rtc = geom[0], geom[2], geom[3:6], geom[6:9]
        mat = model.array("material")
        self.E, self.nu, self.KIc = mat[0], mat[1], mat[3]
        self.nlf, self.factor, self.protype = mat[5], mat[6], int(mat[7])
        self.mr, self.dcf = mr, dcf
        self.off = model.array("fam_off")
        self.mem = model.array("fam_members")
        self.horizon = model.array("fam_horizon")
        self.vol = model.array("vol_node")
        self.fam_of = -np.ones(len(self.X), dtype=np.int64)
        self.fam_of[self.mem[self.off[:-1]]] = np.arange(len(self.off) - 1)
        self.nbx = int((self.rtc[0] - self.lbc[0]) / self.block + 1)
        self.nby = int((self.rtc[1] - self.lbc[1]) / self.block + 1)
        # block lists in insertion order: nodes by index, elements by index (centre)
        self.block_nodes = [[] for _ in range(self.nbx * self.nby)]
        for k, x in enumerate(self.X):
            self.block_nodes[self._bidx(x)].append(k)
        self.block_elems = [[] for _ in range(self.nbx * self.nby)]
        for e in range(self.n_elem):
            c = self.X[self.conn[e, :self.nn[e]]].sum(axis=0) / self.nn[e]
            self.block_elems[self._bidx(c)].append(e)
        # strain-operator columns c = omega g dv_m per bond (bond layout, self excluded)
        _, g, _, _ = oracle.coeffs()
        self.c = np.zeros_like(g)
        b = 0
        for f in range(len(self.off) - 1):
            k = self.mem[self.off[f]]
            dk = self.horizon[f]
            for q in range(self.off[f] + 1, self.off[f + 1]):
                m = self.mem[q]
                xi = self.X[m] - self.X[k]
                omega = math.exp(-(xi @ xi) / (self.nlf * self.nlf * dk * dk))
                self.c[b] = omega * g[b] * self.vol[m]
                b += 1
        self.oracle = oracle
        E, nu = self.E, self.nu
        if self.protype == 1:
            self.D = E / (1 - nu * nu) * np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]])
        else:
            f = E / ((1 + nu) * (1 - 2 * nu))
            self.D = f * np.array([[1 - nu, nu, 0], [nu, 1 - nu, 0], [0, 0, (1 - 2 * nu) / 2]])

    def _bidx(self, x):
        i = int((x[0] - self.lbc[0]) / self.block)
        j = int((x[1] - self.lbc[1]) / self.block)
        return i + j * self.nbx

    def _fe_centre(self, q, u):
        """Displacement gradient (dux/dx, duy/dy, dux/dy, duy/dx) and stress at the bilinear element's centre."""
        dNdp = np.array([-0.25, 0.25, 0.25, -0.25])
        dNdq = np.array([-0.25, -0.25, 0.25, 0.25])
        x = self.X[q, :2]
        J = np.array([[dNdp @ x[:, 0], dNdp @ x[:, 1]], [dNdq @ x[:, 0], dNdq @ x[:, 1]]])
        inv = np.linalg.inv(J)
        B1 = inv[0, 0] * dNdp + inv[0, 1] * dNdq
        B2 = inv[1, 0] * dNdp + inv[1, 1] * dNdq
        ue = u[q]
        dg = np.array([B1 @ ue[:, 0], B2 @ ue[:, 1], B2 @ ue[:, 0], B1 @ ue[:, 1]])
        sig = self.D @ np.array([dg[0], dg[1], dg[2] + dg[3]])
        return dg, sig

    def _pd_grad(self, k, u, bond_state):
        f = self.fam_of[k]
        dg = np.zeros(4)
        b0 = self.off[f] - f          # bond index of the family's first member after the node itself
        for q in range(self.off[f] + 1, self.off[f + 1]):
            if not bond_state[q]:
                continue
            m = self.mem[q]
            c = self.c[b0 + (q - self.off[f] - 1)]
            du = u[m] - u[k]
            dg += [c[0] * du[0], c[1] * du[1], c[1] * du[0], c[0] * du[1]]
        return dg

    def _chord(self, p1, p2, tip0, tip1):
        E, nu = self.E, self.nu
        kappa = (3 - nu) / (1 + nu) if self.protype == 1 else 3 - 4 * nu
        al = math.atan2(tip1[1] - tip0[1], tip1[0] - tip0[0])
        ca, sa = math.cos(al), math.sin(al)
        nx, ny = p2[0][1] - p1[0][1], -(p2[0][0] - p1[0][0])
        n0, n1 = ca * nx + sa * ny, -sa * nx + ca * ny
        I1 = I2 = 0.0
        for x, dg, g in (p1, p2):
            dx, dy = x[0] - tip1[0], x[1] - tip1[1]
            r = math.hypot(dx, dy)
            th = math.atan2(-sa * dx + ca * dy, ca * dx + sa * dy)
            s = [(ca * g[0] + sa * g[2]) * ca + (ca * g[2] + sa * g[1]) * sa,
                 -(-sa * g[0] + ca * g[2]) * sa + (-sa * g[2] + ca * g[1]) * ca,
                 -(ca * g[0] + sa * g[2]) * sa + (ca * g[2] + sa * g[1]) * ca]
            gx = (ca * dg[0] + sa * dg[3]) * ca + (ca * dg[2] + sa * dg[1]) * sa
            gy = (-sa * dg[0] + ca * dg[3]) * ca + (-sa * dg[2] + ca * dg[1]) * sa
            c = 1 / math.sqrt(2 * math.pi * r)
            ch, sh, c3, s3, st = math.cos(th / 2), math.sin(th / 2), math.cos(1.5 * th), math.sin(1.5 * th), math.sin(th)
            m1 = [c * ch * (1 - sh * s3), c * ch * (1 + sh * s3), c * sh * ch * c3]
            m2 = [-c * sh * (2 + ch * c3), c * sh * ch * c3, c * ch * (1 - sh * s3)]
            sz = nu * (m1[0] + m1[1]) if self.protype == 2 else 0.0   # mode I's, for both modes

            def eps(a):
                return [(a[0] - nu * (a[1] + sz)) / E, (a[1] - nu * (a[0] + sz)) / E, a[2] * (1 + nu) / E]

            def w(a, e):
                return (a[0] * e[0] + a[1] * e[1] + 2 * a[2] * e[2]) * n0

            def tg(a, ux, uy):
                return a[0] * ux * n0 + a[2] * (ux * n1 + uy * n0) + a[1] * uy * n1

            fct = (1 + nu) / E / math.sqrt(2 * math.pi * r)
            u1 = (fct * ch * ((kappa - 1) / 2 - sh * s3), fct * sh * (-(kappa + 1) / 2 + ch * ch - st * st))
            u2 = (fct * sh * (st * st - ch * ch - (kappa + 1) / 2), fct * ch * (-sh * s3 - (kappa - 1) / 2))
            I1 += 0.5 * (w(s, eps(m1)) - tg(s, *u1) - tg(m1, gx, gy))
            I2 += 0.5 * (w(s, eps(m2)) - tg(s, *u2) - tg(m2, gx, gy))
        return I1, I2

    def evaluate(self, crack, u_all, bond_state):
        """KI, KII, kink angle, Keq and the new tip (None without growth) of the
        crack segment crack = [[x0, y0], [x1, y1]] (x1, y1 the tip) for the
        displacements u_all (n_node x 2) and bond states (member layout)."""
        u = np.asarray(u_all, dtype=np.float64).reshape(-1, 2)
        tip0, tip = np.asarray(crack[0], dtype=np.float64), np.asarray(crack[1], dtype=np.float64)
        sig_nodes, _ = self.oracle.stress(u.reshape(-1), bond_state)
        ib = (int((tip[0] - self.lbc[0]) / self.block), int((tip[1] - self.lbc[1]) / self.block))
        best, near = 1e200, -1
        for k in self.block_nodes[ib[0] + ib[1] * self.nbx]:
            d = (self.X[k, 0] - tip[0]) ** 2 + (self.X[k, 1] - tip[1]) ** 2
            if d <= best:
                best, near = d, k
        R = self.mr * (self.horizon[self.fam_of[near]] / self.factor)
        nsb = int(self.mr / self.factor) + 1
        pts = []
        for ix in range(ib[0] - nsb, ib[0] + nsb + 1):
            for iy in range(ib[1] - nsb, ib[1] + nsb + 1):
                if not (0 <= ix < self.nbx and 0 <= iy < self.nby):
                    continue
                for e in self.block_elems[ix + iy * self.nbx]:
                    nn = self.nn[e]
                    q = list(self.conn[e, :3]) + [self.conn[e, 2] if nn == 3 else self.conn[e, 3]]
                    d2 = [(self.X[n, 0] - tip[0]) ** 2 + (self.X[n, 1] - tip[1]) ** 2 for n in q]
                    inside = sum(d < R * R for d in d2)
                    if inside in (0, 4):
                        continue
                    if self.algo[e] == 2:
                        x = np.zeros(2)
                        for n in q:
                            x = x + self.X[n, :2] * 0.25
                        dg, sig = self._fe_centre(np.array(q), u)
                        pts.append((math.atan2(x[1] - tip[1], x[0] - tip[0]), x, dg, sig))
                    else:
                        for a in range(nn):
                            n = self.conn[e, a]
                            if not (d2[a] > R * R):
                                continue
                            x = self.X[n, :2]
                            s6 = sig_nodes[n]
                            pts.append((math.atan2(x[1] - tip[1], x[0] - tip[0]), x, self._pd_grad(n, u, bond_state),
                                        np.array([s6[0], s6[1], s6[3]])))
        pts.sort(key=lambda p: p[0])
        pts.append(pts[0])
        I1 = I2 = 0.0
        for a, b in zip(pts[:-1], pts[1:]):
            i1, i2 = self._chord(a[1:], b[1:], tip0, tip)
            I1 += i1
            I2 += i2
        Ep = self.E if self.protype == 1 else self.E / (1 - self.nu ** 2)
        KI, KII = 0.5 * Ep * I1, 0.5 * Ep * I2
        if KII > 0:
            tc = 2 * math.atan(0.25 * (KI / KII - math.sqrt(KI * KI / KII / KII + 8.0)))
        elif KII < 0:
            tc = 2 * math.atan(0.25 * (KI / KII + math.sqrt(KI * KI / KII / KII + 8.0)))
        else:
            tc = 0.0
        keq = math.cos(tc / 2) * (KI * math.cos(tc / 2) ** 2 - 1.5 * KII * math.sin(tc))
        new_tip = None
        if keq > self.KIc:
            al = math.atan2(tip[1] - tip0[1], tip[0] - tip0[0])
            step = self.dcf * self.min_delta
            new_tip = tip + step * np.array([math.cos(al + tc), math.sin(al + tc)])
        return KI, KII, tc, keq, new_tip
