"""External-stress generators (Tools/ExternalStress): uniform backslip and
Rudnicki's point-injection poroelastic solution, in the layout
Simulation.set_external_stress takes.  Host code: runs without a GPU."""
import math

import numpy as np
import pytest

from qdfn import external as E
from qdfn import geometry as Gm


def test_uniform_backslip_is_minus_k_times_backslip():
    rng = np.random.default_rng(0)
    N = 37
    Ks, Kn = rng.normal(size=(N, N)), rng.normal(size=(N, N))
    ext = E.uniform_backslip(Ks, Kn, loading_rate=2e-9, t_end=3e10)
    assert ext["t"].tolist() == [0.0, 3e10]
    for k in ("normal", "shear", "pressure"):
        assert ext[k].shape == (2, N) and np.all(ext[k][0] == 0)
    assert np.allclose(ext["shear"][1], -(Ks @ np.ones(N)) * 3e10 * 2e-9, rtol=1e-14, atol=0)
    assert np.allclose(ext["normal"][1], -(Kn @ np.ones(N)) * 3e10 * 2e-9, rtol=1e-14, atol=0)
    assert np.all(ext["pressure"] == 0)
    # an operator given as a product (an H-matrix, say)
    ext2 = E.uniform_backslip(lambda x: Ks @ x, lambda x: Kn @ x, 2e-9, 3e10, N=N)
    assert np.array_equal(ext2["shear"], ext["shear"]) and np.array_equal(ext2["normal"], ext["normal"])
    with pytest.raises(ValueError):
        E.uniform_backslip(lambda x: Ks @ x, lambda x: Kn @ x)


def _one_patch(c, strike, dip, rake, G, nu, t, q=100.0, origin=(0.0, 0.0, -2000.0), k=1e-16, eta=0.4e-3,
               B=0.75, nu_u=0.3, rho0=1e3):
    """The same solution for one patch and one time, written out with 3x3
    matrices (an independent restatement of the vectorised code)."""
    lam = 2 * G * nu / (1 - 2 * nu)
    lam_u = 2 * G * nu_u / (1 - 2 * nu_u)
    alpha = 3 * (nu_u - nu) / (B * (1 + nu_u) * (1 - 2 * nu))
    cdiff = k / eta * (lam_u - lam) * (lam + 2 * G) / alpha ** 2 / (lam_u + 2 * G)
    d = np.array([c[0], c[1], -c[2]]) - np.array(origin)
    r = np.linalg.norm(d)
    xi = r / math.sqrt(cdiff * t)
    g = math.erf(xi / 2) - xi / math.sqrt(math.pi) * math.exp(-xi ** 2 / 4)
    a = -q * (lam_u - lam) * G / (4 * math.pi * rho0 * cdiff * r * alpha * (lam_u + 2 * G))
    sig = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            sig[i, j] = a * ((i == j) * (math.erfc(xi / 2) - 2 * g / xi ** 2) +
                             d[i] * d[j] / r ** 2 * (math.erfc(xi / 2) + 6 * g / xi ** 2))
    p = q * eta * math.erfc(xi / 2) / (4 * math.pi * rho0 * r * k)
    eff = sig + p * np.eye(3)
    rs = np.array([[Gm.cosd(-strike), -Gm.sind(-strike), 0], [Gm.sind(-strike), Gm.cosd(-strike), 0], [0, 0, 1]])
    rd = np.array([[1, 0, 0], [0, Gm.cosd(-dip), -Gm.sind(-dip)], [0, Gm.sind(-dip), Gm.cosd(-dip)]])
    R = rd @ rs
    sf = R @ eff @ R.T
    return -sf[2, 2], Gm.cosd(rake) * sf[0, 2] + Gm.sind(rake) * sf[1, 2], p


def test_rudnicki_matches_a_per_patch_restatement():
    rng = np.random.default_rng(4)
    n = 12
    centre = np.column_stack([rng.uniform(-3e3, 3e3, n), rng.uniform(-3e3, 3e3, n), rng.uniform(500, 5e3, n)])
    strike, dip, rake = rng.uniform(0, 180, n), rng.uniform(30, 90, n), rng.uniform(-180, 180, n)
    times = np.array([3.6e3, 8.64e4, 3e6, 3e8])
    ext = E.spherical_diffusion_rudnicki(centre, strike, dip, rake, 32e9, 0.25, times=times)
    for k, t in enumerate(times):
        for i in range(n):
            dn, ds, p = _one_patch(centre[i], strike[i], dip[i], rake[i], 32e9, 0.25, t)
            for got, want in ((ext["normal"][k, i], dn), (ext["shear"][k, i], ds), (ext["pressure"][k, i], p)):
                assert abs(got - want) <= 1e-9 * max(abs(want), 1e-3 * abs(p) + 1e-30)


def test_rudnicki_pressure_grows_in_time_and_decays_with_distance():
    centre = np.array([[0.0, 500.0, 2000.0], [0.0, 1500.0, 2000.0], [0.0, 3000.0, 2000.0]])
    ext = E.spherical_diffusion_rudnicki(centre, np.zeros(3), np.full(3, 90.0), np.zeros(3), 32e9, 0.25)
    p = ext["pressure"]
    assert ext["t"].shape == (150,) and p.shape == (150, 3)
    assert np.all(p >= 0) and np.all(np.diff(p, axis=0) >= 0)        # continuous injection
    assert np.all(p[-1, :-1] > p[-1, 1:])                             # nearer patches see more
    # late time: the steady point-source pressure q eta / (4 pi rho0 r k)
    r = np.linalg.norm(np.column_stack([centre[:, 0], centre[:, 1], -centre[:, 2]]) - [0.0, 0.0, -2000.0], axis=1)
    steady = 100.0 * 0.4e-3 / (4 * math.pi * 1e3 * r * 1e-16)
    late = E.spherical_diffusion_rudnicki(centre, np.zeros(3), np.full(3, 90.0), np.zeros(3), 32e9, 0.25,
                                          times=[1e24])
    assert np.allclose(late["pressure"][0], steady, rtol=1e-6)
    assert np.all(np.isfinite(ext["normal"])) and np.all(np.isfinite(ext["shear"]))
