"""Seeded synthetic workloads with the shapes and distributions of the
benchmark configurations. No external dataset is used: the same generator
output feeds the GPU engine and the CPU oracle.

- lj_argon_lattice: simple-cubic lattice (spacing L/side, offset L/(2 side),
  the site layout of generate_bodies_in_cell_nodes, bodies.jl:139-159), reduced
  units sigma = eps = m = kb = 1, Maxwell-Boltzmann velocities with the
  centre-of-mass drift removed, optional jitter of the sites.
- plummer_sphere: Plummer model (Aarseth, Henon & Wielen 1974 sampling:
  radius from the cumulative mass, speed by von Neumann rejection of
  q^2 (1-q^2)^(7/2)), total mass M, scale radius a, G = 1 units; centre of
  mass and its velocity removed.
- spcfw_water_box: SPC/Fw molecules on a jittered cubic lattice, random
  orientations of the equilibrium geometry, all three sites moving with the
  molecule's Maxwell-Boltzmann velocity.
"""
import math

import numpy as np

from .bodies import MassBody, WaterMolecule

# SPC/Fw water in kJ/mol, nm, ps, Da (the units of the reference's water tests)
KB_KJ = 8.3144598e-3
# SPC/Fw force constants of the benchmark workload: bond 4637 kJ/mol/A^2
# (= 463,700 kJ/mol/nm^2, read per square angstrom: per nm^2 the O-H bond is too
# soft to hold an H against a neighbouring O's Coulomb pull), angle 383 kJ/mol/rad^2
SPCFW_KB = 4637.0 * 100.0
SPCFW_KA = 383.0
M_O = 15.999
M_H = 1.00794
K_EL = 138.935458


def lj_argon_lattice(n, rho=0.8, T=1.0, seed=0, jitter=0.0, m=1.0, kb=1.0):
    """Positions (n, 3), velocities (n, 3) and box L of an LJ liquid start."""
    rng = np.random.default_rng(seed)
    L = (n / rho) ** (1.0 / 3.0)
    side = int(math.ceil(n ** (1.0 / 3.0) - 1e-9))
    dL = L / side
    g = (np.arange(side) + 0.5) * dL
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)[:n].copy()
    if jitter > 0:
        pos += rng.uniform(-jitter, jitter, size=pos.shape) * dL
    vel = rng.standard_normal((n, 3)) * math.sqrt(kb * T / m)
    vel -= vel.mean(axis=0)
    return pos, vel, L


def plummer_sphere(n, seed=0, M=1.0, a=1.0, G=1.0, rmax_frac=0.999):
    """Positions (n, 3), velocities (n, 3), masses (n,) of a Plummer sphere."""
    rng = np.random.default_rng(seed)
    m = np.full(n, M / n)
    X1 = rng.uniform(0.0, rmax_frac, n)
    X1 = np.maximum(X1, 1e-10)
    r = a / np.sqrt(X1 ** (-2.0 / 3.0) - 1.0)
    cost = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * math.pi, n)
    sint = np.sqrt(1 - cost ** 2)
    pos = np.stack([r * sint * np.cos(phi), r * sint * np.sin(phi), r * cost], axis=1)
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x = rng.uniform(0.0, 1.0, todo.size)
        y = rng.uniform(0.0, 0.1, todo.size)
        ok = y < x * x * (1 - x * x) ** 3.5
        q[todo[ok]] = x[ok]
        todo = todo[~ok]
    ve = math.sqrt(2.0 * G * M / a) * (1.0 + (r / a) ** 2) ** (-0.25)
    speed = q * ve
    cost = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * math.pi, n)
    sint = np.sqrt(1 - cost ** 2)
    vel = np.stack([speed * sint * np.cos(phi), speed * sint * np.sin(phi), speed * cost], axis=1)
    pos -= (m[:, None] * pos).sum(axis=0) / M
    vel -= (m[:, None] * vel).sum(axis=0) / M
    return pos, vel, m


def _random_rotations(rng, k):
    """k uniformly distributed rotation matrices (random unit quaternions)."""
    qv = rng.standard_normal((k, 4))
    qv /= np.linalg.norm(qv, axis=1, keepdims=True)
    w, x, y, z = qv.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], axis=1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], axis=1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], axis=1),
    ], axis=1)


def _lattice_contacts(O, H1, H2, side, n_mol, L, d_ho, d_hh):
    """Molecules whose H lies closer than d_ho to a neighbouring site's O or
    closer than d_hh to its H (26 lattice neighbours, periodic)."""
    idx = np.arange(n_mol)
    ix, iy, iz = idx // (side * side), (idx // side) % side, idx % side
    bad = np.zeros(n_mol, dtype=bool)
    for ox in (-1, 0, 1):
        for oy in (-1, 0, 1):
            for oz in (-1, 0, 1):
                if ox == oy == oz == 0:
                    continue
                nb = (((ix + ox) % side) * side + (iy + oy) % side) * side + (iz + oz) % side
                ok = nb < n_mol
                nbv = np.where(ok, nb, 0)
                for H in (H1, H2):
                    for other, lim in ((O, d_ho), (H1, d_hh), (H2, d_hh)):
                        d = H - other[nbv]
                        d -= L * np.round(d / L)
                        bad |= ok & ((d * d).sum(axis=1) < lim * lim)
    return bad


def spcfw_water_box(n_mol, density_g_cm3=0.997, T=300.0, seed=0, rOH=0.1012,
                    aHOH=113.24 * math.pi / 180, jitter=0.05):
    """Atom positions (3 n_mol, 3) ordered O,H1,H2, velocities, box L (nm).
    Orientations are uniform random, re-drawn (up to 200 times) for any
    molecule whose H lands within 0.17 nm of a neighbouring O or 0.15 nm of a
    neighbouring H, so that the start holds no H-O contact that Coulomb
    attraction would collapse."""
    rng = np.random.default_rng(seed)
    m_mol = M_O + 2 * M_H
    # 1 g/cm^3 = 602.214 Da/nm^3
    rho_mol = density_g_cm3 * 602.214076 / m_mol
    L = (n_mol / rho_mol) ** (1.0 / 3.0)
    side = int(math.ceil(n_mol ** (1.0 / 3.0) - 1e-9))
    dL = L / side
    g = (np.arange(side) + 0.5) * dL
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    O = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)[:n_mol].copy()
    O += rng.uniform(-jitter, jitter, size=O.shape) * dL
    h1 = np.array([rOH, 0.0, 0.0])
    h2 = np.array([math.cos(aHOH) * rOH, math.sin(aHOH) * rOH, 0.0])
    R = _random_rotations(rng, n_mol)
    H1 = O + R @ h1
    H2 = O + R @ h2
    for _ in range(200):
        bad = _lattice_contacts(O, H1, H2, side, n_mol, L, 0.17, 0.15)
        if not bad.any():
            break
        Rb = _random_rotations(rng, int(bad.sum()))
        H1[bad] = O[bad] + Rb @ h1
        H2[bad] = O[bad] + Rb @ h2
    pos = np.empty((3 * n_mol, 3))
    pos[0::3], pos[1::3], pos[2::3] = O, H1, H2
    vmol = rng.standard_normal((n_mol, 3)) * math.sqrt(KB_KJ * T / m_mol)
    vmol -= vmol.mean(axis=0)
    vel = np.repeat(vmol, 3, axis=0)
    return pos, vel, L


def water_molecules(pos, vel):
    """WaterMolecule bodies from atom arrays ordered O,H1,H2."""
    out = []
    for i in range(pos.shape[0] // 3):
        o = 3 * i
        out.append(WaterMolecule(MassBody(pos[o], vel[o], M_O), MassBody(pos[o + 1], vel[o + 1], M_H),
                                 MassBody(pos[o + 2], vel[o + 2], M_H)))
    return out


def lj_ensemble(n_rep=256, n_min=256, n_max=8192, T_min=0.7, T_max=1.5, rho=0.8, seed=0, jitter=0.02):
    """Uneven replica ensemble of LJ liquids: N_r ~ U[n_min, n_max] and
    T_r ~ U[T_min, T_max] (seeded), each on its own jittered lattice at
    density rho. Returns a list of dicts with pos, vel, L, T, n."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_min, n_max + 1, size=n_rep)
    Ts = rng.uniform(T_min, T_max, size=n_rep)
    out = []
    for r in range(n_rep):
        pos, vel, L = lj_argon_lattice(int(ns[r]), rho=rho, T=float(Ts[r]), seed=seed * 100003 + r, jitter=jitter)
        out.append(dict(pos=pos, vel=vel, L=L, T=float(Ts[r]), n=int(ns[r])))
    return out
