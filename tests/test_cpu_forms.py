"""The algebraic forms the face kernels use in place of the reference's
expressions, checked in plain float64 on seeded random inputs: each equals
the reference's expression (compute_flux_3d.H:33-65 for the limiter,
flux_schemes.H:107-310 for AUSM+-up) to a few units in the last place of the
quantities involved.  The GPU kernels are checked against the reference's own
code in tests/test_gpu_ref_pin.py; these tests pin the identities the forms
rest on, independently of the hardware."""
import numpy as np

rng = np.random.default_rng(2026)
EPS = np.finfo(np.float64).eps


def signed_mags(n, lo=-12, hi=6):
    x = np.sign(rng.standard_normal(n)) * 10.0 ** rng.uniform(lo, hi, n)
    x[rng.random(n) < 0.05] = 0.0
    return x


def test_tmj_limiter_closed_form():
    n = 400000
    d1 = signed_mags(n)
    # d2 near d1 (smooth regions), of either sign, or unrelated
    d2 = np.where(rng.random(n) < 0.5, d1 * (1 + rng.uniform(-0.9, 2, n)), signed_mags(n))
    # the reference: q = |d1 - d2| / (|d1| + |d2| + 1e-20), psi = 1 - q^2,
    # L = psi (d1 + d2) / 2, the states move by L / 2
    q = np.abs((d1 - d2) / (np.abs(d1) + np.abs(d2) + 1e-20))
    half_ref = 0.5 * (0.5 * (1.0 - q ** 2) * (d1 + d2))
    # the kernels: d1 d2 / (d1 + d2) when d1 d2 > 0, else 0
    p = d1 * d2
    with np.errstate(divide="ignore", invalid="ignore"):
        half = np.where(p > 0, p / (d1 + d2), 0.0)
    scale = np.abs(d1) + np.abs(d2)
    # With t = 1e-20 and S = |d1| + |d2| the exact difference of the two is
    # at most t/2 (same signs: psi differs by D^2 (2 S t + t^2) / (S^2 (S + t)^2)
    # <= 2 t / S, times |d1 + d2| / 4; opposite signs: psi <= 2 t / S), and the
    # reference's 1 - q^2 cancels where q is near 1, so a few ulp of S on top
    assert np.all(np.abs(half - half_ref) <= 8 * EPS * scale + 0.5001e-20)
    big = scale > 1e-4  # where the guard is below rounding: within one ulp of S
    assert np.all(np.abs(half - half_ref)[big] <= EPS * scale[big])


def test_ausm_interface_speed_selection():
    n = 200000
    as2L = 10.0 ** rng.uniform(3, 6, n)
    as2R = as2L * 10.0 ** rng.uniform(-0.3, 0.3, n)
    # mostly subsonic, some supersonic sides
    vL = np.sqrt(as2L) * rng.uniform(-1.6, 1.6, n)
    vR = np.sqrt(as2R) * rng.uniform(-1.6, 1.6, n)
    # the reference: a_hat = a*^2 / max(a*, |v|) per side, a_1/2 = min
    aL = np.sqrt(as2L)
    aR = np.sqrt(as2R)
    ah_ref = np.minimum(as2L / np.maximum(aL, np.abs(vL)), as2R / np.maximum(aR, np.abs(vR)))
    # the kernels: both subsonic (a*^2 >= v^2 per side) -> sqrt of the smaller a*^2,
    # else per side a* or a*^2 / |v|, the smaller
    sub = (as2L >= vL * vL) & (as2R >= vR * vR)
    m = np.minimum(as2L, as2R)
    ahL = np.where(as2L >= vL * vL, aL, as2L / np.abs(vL))
    ahR = np.where(as2R >= vR * vR, aR, as2R / np.abs(vR))
    ah = np.where(sub, m / np.sqrt(m), np.minimum(ahL, ahR))
    assert np.all(np.abs(ah - ah_ref) <= 4 * EPS * ah_ref)
    assert sub.any() and (~sub).any()


def test_mach_split_supersonic_branches_are_selects():
    M = np.concatenate([10.0 ** rng.uniform(0, 3, 10000), -(10.0 ** rng.uniform(0, 3, 10000))])
    M = M[np.abs(M) > 1]
    assert np.array_equal(0.5 * (M + np.abs(M)), np.where(M > 0, M, 0.0))
    assert np.array_equal(0.5 * (M - np.abs(M)), np.where(M < 0, M, 0.0))


def test_alpha_and_mean_mach_forms():
    fa = rng.uniform(0.0, 1.0, 100000)
    alpha_ref = (3.0 / 16.0) * (-4.0 + 5.0 * fa * fa)
    alpha = (15.0 / 16.0) * fa * fa - 0.75
    assert np.all(np.abs(alpha - alpha_ref) <= 4 * EPS * 0.75)
    vL, vR = rng.standard_normal(100000), rng.standard_normal(100000)
    ah = 10.0 ** rng.uniform(1, 3, 100000)
    iah = 1.0 / ah
    mb2_ref = (vL * vL + vR * vR) / (2.0 * ah * ah)
    ML, MR = vL * iah, vR * iah
    mb2 = 0.5 * (ML * ML + MR * MR)
    assert np.all(np.abs(mb2 - mb2_ref) <= 8 * EPS * mb2_ref)


def test_momentum_forms_of_pressure_and_enthalpy():
    n = 100000
    rho = 10.0 ** rng.uniform(-1, 1, n)
    u = rng.standard_normal((3, n)) * 10.0
    p = 1e5 * 10.0 ** rng.uniform(-0.5, 0.5, n)
    gm1 = 0.4
    E = p / gm1 + 0.5 * rho * (u * u).sum(0)
    m = rho * u
    # the reference: velocities first, then rho e = E - rho |v|^2 / 2 and H = gamma/(gamma-1) p/rho + |v|^2/2
    v = m / rho
    k = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]
    p_ref = (E - 0.5 * rho * k) * gm1
    H_ref = (1.4 / gm1) * (p_ref / rho) + 0.5 * k
    # the kernels: |m|^2 / (2 rho) from the momenta
    hk = (0.5 * ((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2])) * (1.0 / rho)
    pk = (E - hk) * gm1
    Hk = ((1.4 / gm1) * pk + hk) * (1.0 / rho)
    assert np.all(np.abs(pk - p_ref) <= 8 * EPS * E * gm1)
    assert np.all(np.abs(Hk - H_ref) <= 8 * EPS * np.abs(H_ref) + 8 * EPS * E / rho)
