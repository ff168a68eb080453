"""Small seeded fault systems shared by the GPU parity tests."""
import numpy as np

from qdfn import geometry, synth


def cols(rec):
    return dict(cx=rec[:, 0], cy=rec[:, 1], cz=rec[:, 2], ls=rec[:, 3], ld=rec[:, 4], strike=rec[:, 5],
                dip=rec[:, 6], rake=rec[:, 7])


def small_network(seed=3, n_faults=4, patch=400.0):
    return synth.fault_network(seed=seed, n_faults=n_faults, patch=patch, length=(1200.0, 2400.0))


def mixed_rects():
    """Faults with assorted strike/dip/rake, including vertical, shallow-dipping,
    surface-near and pure dip-slip patches."""
    return np.vstack([
        synth.grid_fault(0.0, 0.0, 3000.0, 2000.0, 1500.0, 30.0, 70.0, 20.0, 500.0),
        synth.grid_fault(2500.0, 800.0, 2500.0, 1000.0, 500.0, 120.0, 85.0, 180.0, 500.0),
        synth.grid_fault(-3000.0, 1500.0, 1200.0, 1500.0, 2000.0, 200.0, 20.0, 90.0, 500.0),
        synth.grid_fault(1000.0, -3000.0, 4000.0, 2000.0, 1000.0, 90.0, 90.0, 0.0, 500.0),
        synth.grid_fault(-500.0, -1500.0, 300.0, 600.0, 500.0, 0.0, 45.0, 270.0, 300.0),
    ])


def bumpy_triangles(nx=6, ny=4, seed=0):
    """Triangulated smooth surface z = -2 km + sum of sinusoids, 2*nx*ny triangles."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-2000.0, 2000.0, nx + 1)
    zs = np.linspace(-3500.0, -600.0, ny + 1)
    amp, k, ph = 150.0, rng.uniform(0.5e-3, 2e-3, 3), rng.uniform(0, 2 * np.pi, 3)
    y = lambda x, z: sum(amp * np.sin(k[i] * (x + z) + ph[i]) for i in range(3))
    tris = []
    for i in range(nx):
        for j in range(ny):
            p = [(xs[i], zs[j]), (xs[i + 1], zs[j]), (xs[i + 1], zs[j + 1]), (xs[i], zs[j + 1])]
            P = [np.array([x, y(x, z), z]) for x, z in p]
            tris.append((P[0], P[1], P[2]))
            tris.append((P[0], P[2], P[3]))
    seg = np.zeros((len(tris), 20))
    for t, (a, b, c) in enumerate(tris):
        seg[t, 0:3], seg[t, 3:6], seg[t, 6:9] = a, b, c
        seg[t, 9] = 30.0 * (t % 4)   # rakes 0, 30, 60, 90
    return seg


def problem_for(rec, Ks, G=32e9, a=0.010, b=0.015, sigma=40e6, Dc=1e-3, seed=None):
    n = rec.shape[0]
    rho = G / 3500.0 ** 2
    if seed is None:
        av, bv, Dcv = np.full(n, a), np.full(n, b), np.full(n, Dc)
    else:
        rng = np.random.default_rng(seed)
        av = rng.uniform(0.008, 0.012, n)
        bv = av + rng.uniform(-0.004, 0.004, n)
        Dcv = 10 ** rng.uniform(-4, -2, n)
    Vi = np.full(n, 1e-9)
    prob = dict(N=n, Nload=0, a=av, b=bv, Dc=Dcv, theta_i=Dcv / Vi, V_i=Vi,
                f_i=0.6 + (av - bv) * np.log(1e-9 / 1e-6), sigma0=np.full(n, sigma), V_const=np.zeros(n),
                mass=geometry.fault_mass(rec[:, 3], rec[:, 4], rho), G=G, rho=rho, sigma_min=1e6, switch_v=1e-2,
                dt_cut=5.0, max_dt=1e7, alpha_evo=0.0, evolution_dr=1, interp_at_told=0)
    prob["rupture_dt"] = geometry.rupture_dt(prob["mass"], np.diag(Ks), 3.0)
    return prob
