"""Deterministic reference solutions for one-group slabs (test infrastructure).

A discrete-ordinates (S_N) solve of the 1-D transport equation

    mu dpsi/dx + Sigma_t psi = (Sigma_s / 2) phi,   phi = int psi dmu,

with a double-Gauss half-range quadrature (Gauss-Legendre on (0,1) and on
(-1,0)), step-characteristic sweeps (exact for a cell-wise constant source)
on a fine mesh, and source iteration.  The left face receives particles
whose direction cosine is uniform on (0, 1] at unit rate -- mu psi(0, mu) = 1
-- which is the inward hemisphere source of the slab workloads; the right
face receives nothing.  Regions may differ (the layered differentiation
slab).  Returns transmitted and reflected currents, absorption rate, the
flux integrated over chosen bins, and the balance T + R + A = 1.
"""
from __future__ import annotations

import numpy as np


def solve_slab(widths, sig_t, sig_s, n_mu=64, dx_max=0.005, tol=1e-12, max_iter=5000,
               flux_edges=None):
    widths = np.asarray(widths, float)
    sig_t = np.asarray(sig_t, float)
    sig_s = np.asarray(sig_s, float)
    # mesh
    edges = [0.0]
    st, ss = [], []
    for w, t, s in zip(widths, sig_t, sig_s):
        n = max(1, int(np.ceil(w / dx_max)))
        h = w / n
        for _ in range(n):
            edges.append(edges[-1] + h)
            st.append(t)
            ss.append(s)
    edges = np.array(edges)
    dx = np.diff(edges)
    st = np.array(st)
    ss = np.array(ss)
    nc = dx.size
    # half-range Gauss-Legendre
    x, w = np.polynomial.legendre.leggauss(n_mu)
    mu = 0.5 * (x + 1.0)
    wt = 0.5 * w
    phi = np.zeros(nc)
    j_right = j_left = 0.0
    psi_edge_last = None
    for it in range(max_iter):
        q = 0.5 * ss * phi          # isotropic emission per unit mu
        phi_new = np.zeros(nc)
        # mu > 0 sweep, inflow psi = 1/mu
        psi_in = 1.0 / mu
        tr = 0.0
        for i in range(nc):
            tau = st[i] * dx[i] / mu
            e = np.exp(-tau)
            src = q[i] / st[i] if st[i] > 0 else 0.0
            psi_out = psi_in * e + src * (1.0 - e)
            avg = np.where(tau > 1e-12, src + (psi_in - psi_out) / np.maximum(tau, 1e-300), psi_in)
            phi_new[i] += np.sum(wt * avg)
            psi_in = psi_out
        j_right = float(np.sum(wt * mu * psi_in))
        # mu < 0 sweep from the right, no inflow
        psi_in = np.zeros_like(mu)
        for i in range(nc - 1, -1, -1):
            tau = st[i] * dx[i] / mu
            e = np.exp(-tau)
            src = q[i] / st[i] if st[i] > 0 else 0.0
            psi_out = psi_in * e + src * (1.0 - e)
            avg = np.where(tau > 1e-12, src + (psi_in - psi_out) / np.maximum(tau, 1e-300), psi_in)
            phi_new[i] += np.sum(wt * avg)
            psi_in = psi_out
        j_left = float(np.sum(wt * mu * psi_in))
        diff = np.max(np.abs(phi_new - phi)) / max(np.max(np.abs(phi_new)), 1e-300)
        phi = phi_new
        if diff < tol:
            break
    absorption = float(np.sum((st - ss) * phi * dx))
    out = {"transmission": j_right, "reflection": j_left, "absorption": absorption,
           "balance": j_right + j_left + absorption, "iterations": it + 1,
           "phi": phi, "edges": edges}
    if flux_edges is not None:
        fe = np.asarray(flux_edges, float)
        centers = 0.5 * (edges[1:] + edges[:-1])
        idx = np.searchsorted(fe, centers, side="right") - 1
        fl = np.zeros(fe.size - 1)
        for i in range(nc):
            if 0 <= idx[i] < fl.size:
                fl[idx[i]] += phi[i] * dx[i]
        out["flux"] = fl
    return out


def slab_1g_reference(thickness=20.0, sig_t=1.0, sig_s=0.5, n_bins=100, **kw):
    return solve_slab([thickness], [sig_t], [sig_s],
                      flux_edges=np.linspace(0.0, thickness, n_bins + 1), **kw)
