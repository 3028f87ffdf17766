"""The FP32 pair classification of the force kernels (pair_cutoff), emulated
in numpy on the CPU, against the reference's pair set: j != i with
r^2 < R^2, r^2 from the loop minimum image in FP64
(basic_potentials.jl:253-258, boundary_conditions.jl:138-165).

Positions are split as the force kernels split them: the wrapped position's
hi part on the grid 2^-k, k = 22 - ceil(log2 L), and an FP32 lo remainder;
the difference subtracts s (Lh + Ll), s = rint(dh / L), L split the same
way. r^2 below lo = min(R^2 (1 - m), (L/2 (1 - m))^2) is in, at or above
hi = R^2 (1 + m) out, m = CLASSIFY_MARGIN = 1e-5; anything between goes to
the reference's FP64 arithmetic. Every pair the emulation decides must agree
with the reference, on pairs crowded at the cutoff and at half the box.
Fused multiply-adds are emulated in float64 and rounded once more. CPU only."""
import math

import numpy as np
import pytest

F = np.float32
M = 1.0e-5  # CLASSIFY_MARGIN


def _f_down(x):
    f = F(x)
    return np.nextafter(f, F(0)) if float(f) > x else f


def _f_up(x):
    f = F(x)
    return np.nextafter(f, F(np.inf)) if float(f) < x else f


def _split(x, L):
    """Wrapped position, hi on the 2^-k grid and the lo remainder."""
    k = 22 - math.ceil(math.log2(L))
    w = x - L * np.floor(x * (1.0 / L))
    w = np.where(w < 0, w + L, w)
    w = np.where(w >= L, w - L, w)
    hq = np.rint(w * 2.0 ** k) * 2.0 ** -k
    return hq.astype(F), (w - hq).astype(F)


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


@pytest.mark.parametrize("L,R", [(10.772173450159421, 2.5), (4.971816450054878, 0.9), (3.0, 1.45),
                                 (9.942, 0.9)])
def test_pair_screen_decides_only_reference_pairs(L, R):
    rng = np.random.default_rng(int(L * 1000))
    n = 400000
    xi = rng.uniform(-2 * L, 3 * L, size=(n, 3))
    sel = rng.random(n)
    r = R * (1 + rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-10, -3, n))
    r = np.where(sel < 0.2, 0.5 * L * (1 + rng.uniform(-3e-5, 3e-5, n)), r)
    r = np.where(sel > 0.9, rng.uniform(0, 0.8 * L, n), r)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    xj = xi + r[:, None] * d + L * rng.integers(-2, 3, size=(n, 3))
    # the reference
    dd = xi - xj
    for _ in range(8):
        dd = np.where(dd >= 0.5 * L, dd - L, dd)
    for _ in range(8):
        dd = np.where(dd < -0.5 * L, dd + L, dd)
    r2 = (dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1]) + dd[:, 2] * dd[:, 2]
    ref_in = r2 < R * R
    # the emulated screen
    k = 22 - math.ceil(math.log2(L))
    Lh_d = np.rint(L * 2.0 ** k) * 2.0 ** -k
    Lh, Ll, invLf = F(Lh_d), F(L - Lh_d), F(1.0 / L)
    hi_i, lo_i = _split(xi, L)
    hi_j, lo_j = _split(xj, L)
    magic = F(12582912.0)
    dh = hi_i - hi_j
    dl = lo_i - lo_j
    s = _fma(dh, np.full_like(dh, invLf), np.full_like(dh, magic)) - magic
    dxh = _fma(-s, np.full_like(s, Lh), dh)
    dxl = _fma(-s, np.full_like(s, Ll), dl)
    dx = dxh + dxl
    r2f = _fma(dx[:, 0], dx[:, 0], _fma(dx[:, 1], dx[:, 1], dx[:, 2] * dx[:, 2]))
    img2 = (0.5 * L * (1 - M)) ** 2
    lo = _f_down(min(R * R * (1 - M), img2))
    hi = _f_up(R * R * (1 + M))
    decided_in = r2f < lo
    decided_out = r2f >= hi
    assert not (decided_in & ~ref_in).any(), "a decided pair outside the reference's cutoff"
    assert not (decided_out & ref_in).any(), "a pair inside the cutoff decided out"
    assert (decided_in | decided_out)[sel > 0.9].mean() > 0.99
