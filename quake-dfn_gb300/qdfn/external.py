"""External-stress generators: the forcing files the reference's tools write as
Input_ExternalStressChange (time array, then per time and patch the normal and
shear stress changes and the pore pressure), in the layout
Simulation.set_external_stress takes (nt x N, row-major).

  uniform_backslip              Tools/ExternalStress/UniformBackslip.jl:13-95
  spherical_diffusion_rudnicki  Tools/ExternalStress/SphericalDiffusion_Rudnicki_RectangleOnly.jl:11-158

The second evaluates Rudnicki's solution for fluid injected at a constant mass
rate at a point of an infinite poroelastic solid (J. W. Rudnicki, "Fluid mass
sources and point forces in linear elastic diffusive solids", Mechanics of
Materials 5, 1986): pore pressure and total stress at each patch centre, the
effective stress (tension positive) rotated into the fault frame, and the
normal (compression positive) and rake-direction shear changes.
"""
import math

import numpy as np

from .geometry import cosd, sind


def uniform_backslip(Ks, Kn, loading_rate=1e-9, t_end=1e11, N=None):
    """Backslip of every patch at `loading_rate` (m/s): the stress changes reach
    -(K . 1) * loading_rate * t_end at t_end, linearly from 0 at t = 0.
    Ks, Kn: N x N stiffness matrices K[receiver, source], or callables
    returning K @ x (an H-matrix product, say; then N is required)."""
    def apply(K, x):
        return np.asarray(K(x)) if callable(K) else np.asarray(K) @ x
    if N is None:
        if callable(Ks):
            raise ValueError("N is required when the operators are callables")
        N = np.asarray(Ks).shape[1]
    ones = np.ones(int(N))
    shear = np.zeros((2, N))
    normal = np.zeros((2, N))
    shear[1] = -apply(Ks, ones) * t_end * loading_rate
    normal[1] = -apply(Kn, ones) * t_end * loading_rate
    return dict(t=np.array([0.0, float(t_end)]), normal=normal, shear=shear, pressure=np.zeros((2, N)))


def rudnicki_times(count=150):
    """The tool's time array: 0.001 * 1.2^i s for i = 1..count."""
    return np.array([0.001 * 1.2 ** i for i in range(1, count + 1)])


def _rotation(strike, dip):
    """Fault-frame rotation R_dip(-dip) R_strike(-strike) per patch (n x 3 x 3)."""
    n = strike.shape[0]
    rs = np.zeros((n, 3, 3))
    rd = np.zeros((n, 3, 3))
    cs = np.array([cosd(-a) for a in strike])
    ss = np.array([sind(-a) for a in strike])
    cd = np.array([cosd(-a) for a in dip])
    sd = np.array([sind(-a) for a in dip])
    rs[:, 0, 0], rs[:, 0, 1], rs[:, 1, 0], rs[:, 1, 1], rs[:, 2, 2] = cs, -ss, ss, cs, 1.0
    rd[:, 0, 0], rd[:, 1, 1], rd[:, 1, 2], rd[:, 2, 1], rd[:, 2, 2] = 1.0, cd, -sd, sd, cd
    return np.einsum("nij,njk->nik", rd, rs)


def spherical_diffusion_rudnicki(centre, strike, dip, rake, G, nu, times=None, flow_rate=100.0,
                                 origin=(0.0, 0.0, -2000.0), permeability=1e-16, viscosity=0.4e-3,
                                 skempton=0.75, nu_u=0.3, rho0=1e3):
    """Normal/shear stress change and pore pressure at the patch centres
    (centre: n x 3 with depth positive, angles in degrees) for injection at
    `origin` (z up, metres) at `flow_rate` kg/s, at each of `times` (s).
    Returns dict(t, normal, shear, pressure) with nt x n arrays."""
    from scipy.special import erf, erfc
    times = rudnicki_times() if times is None else np.asarray(times, dtype=float)
    centre = np.asarray(centre, dtype=float)
    n = centre.shape[0]
    lam = 2 * G * nu / (1 - 2 * nu)
    lam_u = 2 * G * nu_u / (1 - 2 * nu_u)
    alpha = 3 * (nu_u - nu) / (skempton * (1 + nu_u) * (1 - 2 * nu))
    c = permeability / viscosity * (lam_u - lam) * (lam + 2 * G) / alpha ** 2 / (lam_u + 2 * G)   # diffusivity
    pos = np.column_stack([centre[:, 0], centre[:, 1], -centre[:, 2]])
    d = pos - np.asarray(origin, dtype=float)
    r = np.sqrt(np.sum(d * d, axis=1))
    dd = d[:, :, None] * d[:, None, :] / (r * r)[:, None, None]          # x_i x_j / r^2
    R = _rotation(np.asarray(strike, dtype=float), np.asarray(dip, dtype=float))
    cr = np.array([cosd(a) for a in rake])
    sr = np.array([sind(a) for a in rake])
    amp = -flow_rate * (lam_u - lam) * G / (4 * math.pi * rho0 * c * r * alpha * (lam_u + 2 * G))
    normal = np.zeros((times.shape[0], n))
    shear = np.zeros((times.shape[0], n))
    pressure = np.zeros((times.shape[0], n))
    eye = np.eye(3)
    for k, t in enumerate(times):
        xi = r / np.sqrt(c * t)
        g = erf(xi / 2) - xi / math.sqrt(math.pi) * np.exp(-xi * xi / 4)
        iso = erfc(xi / 2) - 2 * g / (xi * xi)        # coefficient of delta_ij
        dev = erfc(xi / 2) + 6 * g / (xi * xi)        # coefficient of x_i x_j / r^2
        sig = amp[:, None, None] * (iso[:, None, None] * eye + dev[:, None, None] * dd)
        p = flow_rate * viscosity * erfc(xi / 2) / (4 * math.pi * rho0 * r * permeability)
        eff = sig + p[:, None, None] * eye                                 # effective, tension positive
        sf = np.einsum("nij,njk,nlk->nil", R, eff, R)                     # R eff R^T
        normal[k] = -sf[:, 2, 2]
        shear[k] = cr * sf[:, 0, 2] + sr * sf[:, 1, 2]
        pressure[k] = p
    return dict(t=times, normal=normal, shear=shear, pressure=pressure)
