"""The FP32 screen of the GPU rdf histogram (k_rdf_pairs), emulated in numpy
float32 on the CPU, against the reference's FP64 bin of each pair
(nbody_simulation_result.jl:678-690, boundary_conditions.jl:138-165).

The kernel decides a pair in FP32 only when it is clear of every bin edge and
of (L/2)^2 by its margins, and hands every other pair to the reference's FP64
arithmetic. This checks that argument on pairs crowded onto the bin edges and
the half-box distance: every pair the emulated screen decides must fall in
the reference's bin. The emulation rounds each operation separately (the
kernel's fused multiply-adds round less) and perturbs 1/sqrt by up to 2 ulp
(the approximate instruction). CPU only."""
import numpy as np
import pytest

F = np.float32
MARGIN, MARGIN_ABS = 2e-6, 4e-7  # RDF_MARGIN, RDF_MARGIN_ABS
MAGIC = F(12582912.0)


def _pairs(rng, L, maxbin, n):
    """Pairs with r / dr near an integer (most), near maxbin / 2, or anywhere
    (the third value marks these), each atom up to two boxes out."""
    dr = L / maxbin
    xi = rng.uniform(-2 * L, 3 * L, size=(n, 3))
    k = rng.integers(1, maxbin // 2 + 1, size=n).astype(np.float64)
    sel = rng.random(n)
    q = k + rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-9, -2, n)
    q = np.where(sel < 0.1, 0.5 * maxbin * (1 + rng.uniform(-1e-5, 1e-5, n)), q)
    q = np.where(sel > 0.9, rng.uniform(0, 0.9 * maxbin, n), q)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    xj = xi + (q * dr)[:, None] * d + L * rng.integers(-2, 3, size=(n, 3))
    return xi, xj, sel > 0.9


def _reference_bin(xi, xj, L, maxbin):
    """The reference's loop minimum image, r^2 = (x^2 + y^2) + z^2 and
    ceil(sqrt(r^2) / dr); 0 for a pair it does not count."""
    d = xi - xj
    radius = 0.5 * L
    for _ in range(8):
        d = np.where(d >= radius, d - L, d)
    for _ in range(8):
        d = np.where(d < -radius, d + L, d)
    assert (d >= -radius).all() and (d < radius).all()
    r2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    b = np.ceil(np.sqrt(r2) / (L / maxbin))
    return np.where((r2 < radius * radius) & (b > 1) & (b <= maxbin), b, 0).astype(np.int64)


def _box_units(x, L):
    """k_rdf_pack: wrap into [0, L), then u = w / L in FP64."""
    w = x - L * np.floor(x * (1.0 / L))
    w = np.where(w < 0, w + L, w)
    w = np.where(w >= L, w - L, w)
    return w * (1.0 / L)


def _screen(xi, xj, L, maxbin, split, rng):
    """(decided, bin) of the emulated FP32 screen; bin 0 = not counted."""
    ui, uj = _box_units(xi, L), _box_units(xj, L)
    if split:
        hi = (np.rint(ui * 4194304.0) / 4194304.0).astype(F)
        hj = (np.rint(uj * 4194304.0) / 4194304.0).astype(F)
        dl = (ui - hi).astype(F) - (uj - hj).astype(F)
    else:
        hi, hj = ui.astype(F), uj.astype(F)
        dl = np.zeros_like(hi)
    dh = hi - hj
    s = (dh + MAGIC) - MAGIC
    dx = (dh - s) + dl
    r2 = (dx[:, 0] * dx[:, 0] + dx[:, 1] * dx[:, 1]) + dx[:, 2] * dx[:, 2]
    q2 = r2 * F(float(maxbin) * maxbin)
    with np.errstate(divide="ignore", invalid="ignore"):
        rs = (F(1) / np.sqrt(q2)).astype(F)
    ulp = np.spacing(rs)
    rs = rs + rng.integers(-2, 3, size=rs.shape).astype(F) * ulp
    q = q2 * rs
    tq = q + F(8388607.5)
    e = q + (F(8388607.5) - tq)
    half_thr = F(0.5 - (0.0 if split else MARGIN_ABS * maxbin))
    thr = half_thr - F(MARGIN) * q
    hband = MARGIN if split else 2 * MARGIN
    qmax2 = (0.5 * maxbin) ** 2
    inside = q2 <= F(qmax2 * (1 - hband))
    beyond = q2 >= F(qmax2 * (1 + hband))
    decided = (inside & (np.abs(e) < thr)) | beyond
    counted = inside & (np.abs(e) < thr) & (q > F(1))
    b = np.where(counted, (tq.view(np.int32).astype(np.int64) - 0x4B000000) + 1, 0)
    return decided, b


@pytest.mark.parametrize("L,maxbin,split", [(4.971816450054878, 1000, False), (1.0, 2048, False),
                                            (37.5, 333, False), (4.971816450054878, 16384, True),
                                            (10.0, 1000, True)])
def test_rdf_screen_decides_only_exact_bins(L, maxbin, split):
    rng = np.random.default_rng(maxbin)
    xi, xj, anywhere = _pairs(rng, L, maxbin, 400000)
    ref = _reference_bin(xi, xj, L, maxbin)
    decided, b = _screen(xi, xj, L, maxbin, split, rng)
    wrong = decided & (b != ref)
    assert not wrong.any(), f"{int(wrong.sum())} decided pairs in the wrong bin"
    # pairs at arbitrary distances rarely need the exact pass
    assert decided[anywhere].mean() > 0.95
