"""FP64 numpy restatement of the learned force model (test infrastructure).

TEST INFRASTRUCTURE ONLY: the oracle of the engine's learned-model kernels
(descriptors, per-species MLP, forces by the chain rule, training gradients).
The reference has no learned model; this file restates this project's model
definition (the same constants as the CUDA engine) so that every GPU quantity
has an FP64 counterpart:

  descriptor of atom i over neighbours j of other molecules with r < RD:
    radial   G[s][k] = sum_{j in s} exp(-(r - mu_k)^2 / (2 w^2)) fc(r),
             mu_k = R0 + k w, k < 24, w = (RD - R0) / 23, s = species of j
    angular  p[s][a] = sum psi_a(r) rhat,  Q[s][a] = sum psi_a (rhat rhat^T - I/3),
             psi_a(r) = fc(r) exp(-r^2 / (2 rho_a^2)),
             A1 = |p|^2, A2 = |Q|_F^2
    fc(r) = (cos(pi r / RD) + 1) / 2
    D = [G_O(24), G_H(24), A1_O(4), A1_H(4), A2_O(4), A2_H(4)]
  model of species c:  x = (D - mu_D) / sd_D
    z1 = x W1 + b1, a1 = tanh z1, z2 = a1 W2 + b2, a2 = tanh z2,
    E = sd_E (a2 . w3 + b3) + mu_E
  short-range label: E_i = 1/2 sum_{j, other molecule} phi(r) S(r),
    phi = LJ (O-O) + k q_i q_j erfc(ALPHA r) / r (the real-space part of an
    Ewald-type split of the Coulomb term), S = 1 below RS, C2 smoothstep to 0
    at RD.
"""
import math

import numpy as np
from scipy.special import erfc

RD = 0.6
R0 = 0.07
NK = 24
W = (RD - R0) / (NK - 1)
RS = 0.45
RHO = (0.1, 0.2, 0.3, 10.0)
ALPHA = 4.0
NDESC = 64
NH1 = 128
NH2 = 128


def n_params():
    """Per-species parameter count: W1, b1, W2, b2, w3, b3, then normalisation."""
    return NDESC * NH1 + NH1 + NH1 * NH2 + NH2 + NH2 + 1 + 2 * NDESC + 2


def unpack(theta):
    o = 0

    def take(k, shape=None):
        nonlocal o
        a = theta[o:o + k]
        o += k
        return a.reshape(shape) if shape else a
    W1 = take(NDESC * NH1, (NDESC, NH1))
    b1 = take(NH1)
    W2 = take(NH1 * NH2, (NH1, NH2))
    b2 = take(NH2)
    w3 = take(NH2)
    b3 = take(1)[0]
    muD = take(NDESC)
    sdD = take(NDESC)
    muE = take(1)[0]
    sdE = take(1)[0]
    return W1, b1, W2, b2, w3, b3, muD, sdD, muE, sdE


def fc(r):
    return 0.5 * (np.cos(np.pi * r / RD) + 1.0)


def dfc(r):
    return -0.5 * np.pi / RD * np.sin(np.pi * r / RD)


def min_image(d, L):
    return d - L * np.round(d / L)


def neighbours(u, L, i, ids=None):
    """(j, rij vector j - i, r) of atoms of other molecules within RD. ids:
    the atom indices of u's rows when u holds a subset of the system (rows
    of the whole system by default); j indexes u's rows."""
    ids = np.arange(len(u)) if ids is None else ids
    d = min_image(u - u[i], L)
    r = np.sqrt((d * d).sum(axis=1))
    m = (r < RD) & (ids // 3 != ids[i] // 3)
    j = np.nonzero(m)[0]
    return j, d[j], r[j]


def species(j):
    return np.where(j % 3 == 0, 0, 1)


def descriptor(u, L, i, ids=None):
    """D (64,) and the moments (p[2,4,3], Q[2,4,3,3]) of atom i."""
    ids = np.arange(len(u)) if ids is None else ids
    j, d, r = neighbours(u, L, i, ids)
    s = species(ids[j])
    f = fc(r)
    mu = R0 + W * np.arange(NK)
    G = np.zeros((2, NK))
    g = np.exp(-((r[:, None] - mu[None, :]) ** 2) / (2 * W * W)) * f[:, None]
    for sp in (0, 1):
        G[sp] = g[s == sp].sum(axis=0)
    rh = d / r[:, None]
    p = np.zeros((2, 4, 3))
    Q = np.zeros((2, 4, 3, 3))
    outer = rh[:, :, None] * rh[:, None, :] - np.eye(3)[None] / 3.0
    for a, rho in enumerate(RHO):
        psi = f * np.exp(-r * r / (2 * rho * rho))
        for sp in (0, 1):
            m = s == sp
            p[sp, a] = (psi[m, None] * rh[m]).sum(axis=0)
            Q[sp, a] = (psi[m, None, None] * outer[m]).sum(axis=0)
    A1 = (p * p).sum(axis=2)
    A2 = (Q * Q).sum(axis=(2, 3))
    D = np.concatenate([G[0], G[1], A1[0], A1[1], A2[0], A2[1]])
    return D, p, Q


def mlp(theta, D):
    """Energy and dE/dD of one atom (FP64)."""
    W1, b1, W2, b2, w3, b3, muD, sdD, muE, sdE = unpack(theta)
    x = (D - muD) / sdD
    a1 = np.tanh(x @ W1 + b1)
    a2 = np.tanh(a1 @ W2 + b2)
    E = sdE * (a2 @ w3 + b3) + muE
    g2 = sdE * w3 * (1 - a2 * a2)
    g1 = (g2 @ W2.T) * (1 - a1 * a1)
    dx = g1 @ W1.T
    return E, dx / sdD


def forces(u, L, thetas):
    """Learned energy and forces -dE/dx of all atoms (FP64)."""
    n = len(u)
    F = np.zeros_like(u)
    Etot = 0.0
    for i in range(n):
        E, j, grad = atom_energy_grad(u, L, thetas, i)
        Etot += E
        F[j] -= grad
        F[i] += grad.sum(axis=0)
    return Etot, F


def local_rows(u, L, i, radius):
    """Indices of the atoms within `radius` of atom i (minimum image), i first."""
    d = min_image(u - u[i], L)
    near = np.nonzero((d * d).sum(axis=1) < radius * radius)[0]
    return np.concatenate([[i], near[near != i]])


def forces_on(u, L, thetas, idx):
    """Learned forces -d(sum_k E_k)/dx_i of the atoms idx only (FP64), from
    local neighbourhoods: only atoms k within RD of i have E_k depend on x_i,
    and their own neighbours lie within 2 RD of i, so each force needs the
    atoms within 2 RD of i (a sample of a large box, without all atoms)."""
    out = np.zeros((len(idx), 3))
    for t, i in enumerate(idx):
        rows = local_rows(u, L, i, 2 * RD + 1e-6)
        sub = u[rows]
        j0, _, _ = neighbours(sub, L, 0, rows)
        f = np.zeros(3)
        _, jj, grad = atom_energy_grad(sub, L, thetas, 0, rows)
        f += grad.sum(axis=0)  # dE_i/dx_i = -sum_j dE_i/dx_j
        for k in j0:
            _, jk, gk = atom_energy_grad(sub, L, thetas, k, rows)
            f -= gk[jk == 0].sum(axis=0)  # dE_k/dx_i
        out[t] = f
    return out


def atom_energy_grad(u, L, thetas, i, ids=None):
    """Energy E_i of atom i and dE_i/dr_j for its neighbours j (rows of u,
    as neighbours() returns them); dE_i/dr_i is minus their sum."""
    ids = np.arange(len(u)) if ids is None else ids
    D, p, Q = descriptor(u, L, i, ids)
    E, dD = mlp(thetas[0 if ids[i] % 3 == 0 else 1], D)
    j, d, r = neighbours(u, L, i, ids)
    s = species(ids[j])
    f, df = fc(r), dfc(r)
    rh = d / r[:, None]
    mu = R0 + W * np.arange(NK)
    g = np.exp(-((r[:, None] - mu[None, :]) ** 2) / (2 * W * W))
    # radial: dG/dr = g' fc + g fc'
    dgr = (g * (-(r[:, None] - mu[None, :]) / (W * W)) * f[:, None] + g * df[:, None])
    coef = np.where(s[:, None] == 0, dD[None, :NK], dD[None, NK:2 * NK])
    dEdr = (coef * dgr).sum(axis=1)
    grad = dEdr[:, None] * rh  # dE_i / d r_j  (radial part)
    for a, rho in enumerate(RHO):
        e = np.exp(-r * r / (2 * rho * rho))
        psi = f * e
        dpsi = df * e + f * e * (-r / (rho * rho))
        for sp in (0, 1):
            m = s == sp
            if not m.any():
                continue
            cA1 = dD[48 + 4 * sp + a]
            cA2 = dD[56 + 4 * sp + a]
            pv = p[sp, a]
            Qm = Q[sp, a]
            rr = rh[m]
            pr = rr @ pv
            # d|p|^2/dr_j = 2 [psi' (p.rh) rh + psi/r (p - (p.rh) rh)]
            g1 = 2 * (dpsi[m, None] * pr[:, None] * rr + (psi[m] / r[m])[:, None] * (pv[None] - pr[:, None] * rr))
            Qr = rr @ Qm
            rQr = (Qr * rr).sum(axis=1)
            # d|Q|^2/dr_j = 2 [psi' rQr rh + psi 2/r (Q rh - rQr rh)]
            g2 = 2 * (dpsi[m, None] * rQr[:, None] * rr + (2 * psi[m] / r[m])[:, None] * (Qr - rQr[:, None] * rr))
            grad[m] += cA1 * g1 + cA2 * g2
    return E, j, grad


def smoothstep(r):
    t = np.clip((r - RS) / (RD - RS), 0.0, 1.0)
    S = 1 - 10 * t ** 3 + 15 * t ** 4 - 6 * t ** 5
    dS = (-30 * t ** 2 + 60 * t ** 3 - 30 * t ** 4) / (RD - RS)
    return S, dS


def short_range_labels(u, L, q, lj_eps, lj_sigma, k_el):
    """Per-atom short-range energies E_i and the exact short-range forces."""
    return labels_on(u, L, q, lj_eps, lj_sigma, k_el, np.arange(len(u)))


def labels_on(u, L, q, lj_eps, lj_sigma, k_el, idx):
    """short_range_labels of the atoms idx only: (E[len(idx)], F[len(idx), 3])."""
    E = np.zeros(len(idx))
    F = np.zeros((len(idx), 3))
    for t, i in enumerate(idx):
        j, d, r = neighbours(u, L, i)
        S, dS = smoothstep(r)
        kqq = k_el * q[i] * q[j]
        ec = erfc(ALPHA * r)
        phi = kqq * ec / r
        dphi = -kqq * ec / (r * r) - kqq * (2.0 * ALPHA / math.sqrt(math.pi)) * np.exp(-(ALPHA * r) ** 2) / r
        if i % 3 == 0:
            o = j % 3 == 0
            sr6 = (lj_sigma / r[o]) ** 6
            phi[o] += 4 * lj_eps * (sr6 * sr6 - sr6)
            dphi[o] += 4 * lj_eps * (-12 * sr6 * sr6 + 6 * sr6) / r[o]
        E[t] = 0.5 * (phi * S).sum()
        # dE_total/dr_j for the pair (counted once per ordered pair with the 1/2)
        fpair = (dphi * S + phi * dS)[:, None] * (d / r[:, None])
        F[t] += fpair.sum(axis=0)
    return E, F


def train_gradients(theta, X, y):
    """Mean squared error of standardised energies over a batch and its
    gradient with respect to W1, b1, W2, b2, w3, b3 (X standardised inputs,
    y standardised labels)."""
    W1, b1, W2, b2, w3, b3 = unpack(theta)[:6]
    a1 = np.tanh(X @ W1 + b1)
    a2 = np.tanh(a1 @ W2 + b2)
    out = a2 @ w3 + b3
    e = out - y
    B = len(y)
    loss = float((e * e).mean())
    de = 2 * e / B
    gw3 = a2.T @ de
    gb3 = de.sum()
    g2 = de[:, None] * w3[None, :] * (1 - a2 * a2)
    gW2 = a1.T @ g2
    gb2 = g2.sum(axis=0)
    g1 = (g2 @ W2.T) * (1 - a1 * a1)
    gW1 = X.T @ g1
    gb1 = g1.sum(axis=0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
