"""Seeded synthetic fault systems with the shapes of the benchmark workloads
(the reference ships no benchmark data; these generators stand in for it).

  single_fault   one vertical strike-slip fault, 20 km x 10 km (top at 0.5 km),
                 40 x 20 = 800 patches of 500 m, velocity-weakening core with a
                 2-km velocity-strengthening border ring, sigma = 40 MPa,
                 0.01 MPa/yr background shear stressing
  fault_network  N_f random rectangular faults (strike U[0,180), dip U[60,90],
                 length U[1,5] km, aspect 2:1) with centres in a 10 x 10 km box at
                 2-7 km depth, 100 m patches, a U[0.008,0.012], b-a U[-0.004,0.004],
                 Dc log-uniform [1e-4,1e-2] m, sigma = 18 MPa/km x depth
  friction_draws per-patch (a-b, Dc) redraws on one geometry (ensemble members)

Friction is specified with mu0 = 0.6 at a reference slip rate of 1e-6 m/s; the
reference's laws are written around V0 = 1e-9, so the initial friction is
f_i = mu0 + (a - b) ln(V_i / 1e-6) at steady state (theta_i = Dc / V_i).
"""
import math

import numpy as np

from .geometry import cosd, sind, fault_mass

YEAR = 365.25 * 24 * 3600.0
CS = 3500.0  # shear-wave speed used for radiation damping G / (2 cs)


def _rot_center(cx, cy, cz, L, W, strike, dip, li, wi, lc, wc):
    rs = np.array([[cosd(strike), -sind(strike), 0.0], [sind(strike), cosd(strike), 0.0], [0.0, 0.0, 1.0]])
    rd = np.array([[1.0, 0.0, 0.0], [0.0, cosd(dip), -sind(dip)], [0.0, sind(dip), cosd(dip)]])
    v = np.array([-L / 2 + L * (2 * li - 1) / lc / 2, -W / 2 + W * (2 * wi - 1) / wc / 2, 0.0])
    c = rs @ (rd @ v) + np.array([cx, cy, -cz])
    return c[0], c[1], -c[2]


def grid_fault(cx, cy, cz, L, W, strike, dip, rake, patch):
    """Patch records of one rectangular fault (BulkToSegment gridding)."""
    lc, wc = math.ceil(L / patch), math.ceil(W / patch)
    out = []
    for li in range(1, lc + 1):
        for wi in range(1, wc + 1):
            px, py, pz = (cx, cy, cz) if lc * wc == 1 else _rot_center(cx, cy, cz, L, W, strike, dip, li, wi, lc, wc)
            out.append([px, py, pz, L / lc, W / wc, strike, dip, rake])
    return np.array(out)


def _friction_f0(a, b, V_i, mu0=0.6, vref=1e-6):
    return mu0 + (a - b) * np.log(V_i / vref)


def external_ramp(N, rate_pa_per_yr, t_end_s):
    """Linear shear-stress ramp as Input_ExternalStressChange would hold it."""
    t = np.array([0.0, t_end_s])
    shear = np.vstack([np.zeros(N), np.full(N, rate_pa_per_yr * t_end_s / YEAR)])
    zeros = np.zeros((2, N))
    return dict(t=t, normal=zeros.copy(), shear=shear, pressure=zeros.copy())


def single_fault(patch=500.0, G=32e9, nu=0.25):
    """The 800-patch single-fault workload."""
    rho = G / CS ** 2
    L, W, top = 20000.0, 10000.0, 500.0
    rec = grid_fault(0.0, 0.0, top + W / 2, L, W, 90.0, 90.0, 0.0, patch)
    N = rec.shape[0]
    # along-strike coordinate and depth of each patch for the border ring
    s = rec[:, 1]            # strike 90 -> along y
    z = rec[:, 2]
    ring = (np.abs(s) > L / 2 - 2000.0) | (z < top + 2000.0) | (z > top + W - 2000.0)
    a = np.where(ring, 0.020, 0.010)
    b = np.full(N, 0.015)
    Dc = np.full(N, 1e-3)
    V_i = np.full(N, 1e-9)
    theta = Dc / V_i
    f_i = _friction_f0(a, b, V_i)
    sigma0 = np.full(N, 40e6)
    mass = fault_mass(rec[:, 3], rec[:, 4], rho)
    return dict(records=rec, N=N, Nload=0, G=G, nu=nu, rho=rho, a=a, b=b, Dc=Dc, theta_i=theta, V_i=V_i, f_i=f_i,
                sigma0=sigma0, V_const=np.zeros(N), mass=mass, sigma_min=1e6, years=500.0,
                stressing_rate=0.01e6)


def fault_network(seed=0, n_faults=30, patch=100.0, G=32e9, nu=0.25, length=(1000.0, 5000.0),
                  min_separation=150.0, max_tries=20000):
    """Random network of rectangular faults; faults whose patches come closer
    than min_separation to an existing fault are redrawn (no intersections)."""
    rng = np.random.default_rng(seed)
    rho = G / CS ** 2
    faults = []
    tries = 0
    while len(faults) < n_faults:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d separated faults" % n_faults)
        strike = rng.uniform(0.0, 180.0)
        dip = rng.uniform(60.0, 90.0)
        L = rng.uniform(*length)
        W = L / 2
        cx, cy = rng.uniform(-5000.0, 5000.0, size=2)
        cz = rng.uniform(2000.0, 7000.0)
        if cz - W / 2 * sind(dip) < 100.0:   # keep the top below the surface
            continue
        rec = grid_fault(cx, cy, cz, L, W, strike, dip, 0.0, patch)
        ok = True
        for other in faults:
            d = np.min(np.linalg.norm(rec[:, None, :3] - other[None, :, :3], axis=2)) if len(rec) * len(other) < 4e6 \
                else _min_dist_chunked(rec[:, :3], other[:, :3])
            if d < min_separation:
                ok = False
                break
        if ok:
            faults.append(rec)
    rec = np.vstack(faults)
    N = rec.shape[0]
    a = rng.uniform(0.008, 0.012, N)
    b = a + rng.uniform(-0.004, 0.004, N)
    Dc = 10 ** rng.uniform(-4, -2, N)
    V_i = np.full(N, 1e-9)
    return dict(records=rec, N=N, Nload=0, G=G, nu=nu, rho=rho, a=a, b=b, Dc=Dc, theta_i=Dc / V_i, V_i=V_i,
                f_i=_friction_f0(a, b, V_i), sigma0=18e6 * rec[:, 2] / 1000.0, V_const=np.zeros(N),
                mass=fault_mass(rec[:, 3], rec[:, 4], rho), sigma_min=1e6, years=200.0, stressing_rate=0.01e6,
                n_faults=n_faults, seed=seed)


def _min_dist_chunked(A, B, chunk=2048):
    best = np.inf
    for k in range(0, len(A), chunk):
        d = np.linalg.norm(A[k:k + chunk, None, :] - B[None, :, :], axis=2)
        best = min(best, float(d.min()))
    return best


def friction_draws(base, n_draws, seed=1, amb=(-0.005, 0.002), dc_log=(-4, -2)):
    """Per-patch (a-b, Dc) redraws on one geometry; a is kept, b = a - (a-b)."""
    rng = np.random.default_rng(seed)
    N = base["N"]
    out = {k: [] for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i")}
    for _ in range(n_draws):
        a = np.array(base["a"], dtype=float)
        b = a - rng.uniform(*amb, size=N)
        Dc = 10 ** rng.uniform(*dc_log, size=N)
        V_i = np.full(N, 1e-9)
        out["a"].append(a); out["b"].append(b); out["Dc"].append(Dc)
        out["theta_i"].append(Dc / V_i); out["V_i"].append(V_i); out["f_i"].append(_friction_f0(a, b, V_i))
    return {k: np.concatenate(v) for k, v in out.items()}


def problem_dict(sys, kself_diag, switch_v=1e-2, dt_cut=5.0, rupture_multiple=3.0, max_dt=1e7,
                 n_inst=1, draws=None):
    """Simulation problem for qdfn.simulate.Simulation / the oracle from a
    synthetic system; RuptureDt from the assembled self stiffness."""
    from .geometry import rupture_dt
    p = dict(N=sys["N"], Nload=sys["Nload"], G=sys["G"], rho=sys["rho"], sigma_min=sys["sigma_min"],
             switch_v=switch_v, dt_cut=dt_cut, max_dt=max_dt, alpha_evo=0.0, evolution_dr=1,
             interp_at_told=0, rupture_dt=rupture_dt(sys["mass"], kself_diag, rupture_multiple))
    for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
        p[k] = draws[k] if draws is not None else sys[k]
    for k in ("sigma0", "V_const", "mass"):
        p[k] = np.tile(sys[k], n_inst) if n_inst > 1 else sys[k]
    if n_inst > 1 and draws is None:
        for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
            p[k] = np.tile(p[k], n_inst)
    return p


def curved_fault_network(seed=0, n_faults=5, length=8000.0, width=4000.0, edge=80.0, amplitude=200.0, G=32e9,
                         nu=0.25, top=500.0, spacing=3000.0):
    """Triangulated curved faults (the triangle-mesh configuration): n_faults
    surfaces of length x width (along strike x down dip), each the plane
    through its trace bent out of plane by w(u, v) = sum of 3 sinusoids of
    amplitude `amplitude` and random wavelengths and phases, meshed at `edge`
    into 2 triangles per grid cell; near-parallel strikes (a random base
    strike +- 5 degrees), dips U[70, 85], traces `spacing` apart, tops `top`
    below the surface.  Friction as in
    fault_network.  Returns the 20-column triangle bulk table (P1, P2, P3,
    rake, ...) and the per-triangle problem fields."""
    rng = np.random.default_rng(seed)
    nu_c, nv_c = int(round(length / edge)), int(round(width / edge))
    tris = []
    base = rng.uniform(0.0, 180.0)
    n_base = np.array([-sind(base), cosd(base), 0.0])
    s_base = np.array([cosd(base), sind(base), 0.0])
    for f in range(n_faults):
        # near-parallel strands `spacing` apart (strikes within 5 degrees, so no two surfaces meet)
        strike = base + rng.uniform(-5.0, 5.0)
        # dips below 85 degrees: a TD side along the vertical is a singular
        # configuration of the angular dislocations
        dip = rng.uniform(70.0, 85.0)
        k = 2 * np.pi / rng.uniform(2000.0, 8000.0, 3)
        phase = rng.uniform(0.0, 2 * np.pi, (3, 2))
        origin = (f - (n_faults - 1) / 2) * spacing * n_base + rng.uniform(-1000.0, 1000.0) * s_base
        us = np.array([cosd(strike), sind(strike), 0.0])                          # along strike
        nh = np.array([-sind(strike), cosd(strike), 0.0])                         # horizontal normal
        ud = cosd(dip) * nh + np.array([0.0, 0.0, -sind(dip)])                    # down dip (z up)
        nrm = np.cross(us, ud)
        uu = np.linspace(-length / 2, length / 2, nu_c + 1)
        vv = np.linspace(0.0, width, nv_c + 1)
        U, Vv = np.meshgrid(uu, vv, indexing="ij")
        w = sum(amplitude / 3 * np.sin(k[i] * U + phase[i, 0]) * np.cos(k[i] * Vv + phase[i, 1]) for i in range(3))
        P = origin + U[..., None] * us + Vv[..., None] * ud + w[..., None] * nrm
        P[..., 2] -= top
        for i in range(nu_c):
            for j in range(nv_c):
                a, b, c, d = P[i, j], P[i + 1, j], P[i + 1, j + 1], P[i, j + 1]
                tris.append((a, b, c))
                tris.append((a, c, d))
    n = len(tris)
    seg = np.zeros((n, 20))
    for t, (a, b, c) in enumerate(tris):
        seg[t, 0:3], seg[t, 3:6], seg[t, 6:9] = a, b, c
    seg[:, 9] = 0.0                       # rake
    a = rng.uniform(0.008, 0.012, n)
    bb = a + rng.uniform(-0.004, 0.004, n)
    Dc = 10 ** rng.uniform(-4, -2, n)
    V_i = np.full(n, 1e-9)
    depth = -(seg[:, 2] + seg[:, 5] + seg[:, 8]) / 3
    rho = G / CS ** 2
    return dict(seg=seg, N=n, Nload=0, G=G, nu=nu, rho=rho, a=a, b=bb, Dc=Dc, theta_i=Dc / V_i, V_i=V_i,
                f_i=_friction_f0(a, bb, V_i), sigma0=18e6 * depth / 1000.0, V_const=np.zeros(n),
                mass=np.full(n, edge * rho / 2), sigma_min=1e6, years=100.0, stressing_rate=0.01e6,
                n_faults=n_faults, seed=seed)
