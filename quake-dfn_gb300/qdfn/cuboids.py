"""One-way coupling of reservoir cuboids to the faults: the poroelastic stress
change on every fault patch from pore-pressure and temperature histories of
rectangular cuboids, written as an external-stress forcing (the reference's
CuboidCoupling module).

  input files         CuboidCoupling/Functions_Kuvshinov_Cuboids.jl:21-31,
                      CuboidCoupling/CalculatePoroElasticStress.jl:103-122
  cuboid vertices     Functions_Kuvshinov_Cuboids.jl:4-18
  Green's functions   Functions_Kuvshinov_Cuboids.jl:80-154
  forcing on faults   CalculatePoroElasticStress.jl:35-214

The Green's function is the full-space displacement and stress of a cuboid
under a uniform pressure (or temperature) change (B. P. Kuvshinov, "Elastic
and piezoelectric fields due to polyhedral inclusions", Int. J. Solids Struct.
45, 2008): sums over the 8 vertices of closed-form atan/log terms.
Conventions as the module's: compression positive and z (depth) down in the
Green's functions; the fault-frame stresses come out with normal compression
positive, as the simulation's external stress expects.
"""
import math

import numpy as np

from .geometry import cosd, sind

# the sign of each vertex term, in the vertex order of cuboid_vertices
_SIGNS = np.array([-1.0, 1.0, 1.0, -1.0, 1.0, -1.0, -1.0, 1.0])
# The reference module evaluates its prefactors with pi = 3.1415; pass
# pi=math.pi to the functions below for the exact constant.
REFERENCE_PI = 3.1415


def read_cuboids(path):
    """Input_Cuboids.txt: a header line, then per cuboid
    index, centre x, y, z (depth, m), lengths x, y, z (comma separated).
    Returns (centres n x 3, lengths n x 3)."""
    rows = [ln for ln in open(path).read().splitlines() if ln.strip()]
    data = np.array([[float(t) for t in ln.split(",")] for ln in rows[1:]], dtype=float).reshape(-1, 7)
    return data[:, 1:4].copy(), data[:, 4:7].copy()


def read_history(path):
    """Input_PorePressure.txt / Input_Temperature.txt: first line
    'time(sec), t1, t2, ...', then one line per cuboid 'name, v1, v2, ...'.
    Returns (times nt, values nt x n_cuboids)."""
    rows = [[t.strip() for t in ln.split(",")] for ln in open(path).read().splitlines() if ln.strip()]
    t = np.array([float(x) for x in rows[0][1:]])
    v = np.array([[float(x) for x in r[1:]] for r in rows[1:]], dtype=float).reshape(-1, t.shape[0])
    return t, v.T.copy()


def cuboid_vertices(centre, length):
    """The 8 vertices (8 x 3) in the module's order: x fastest, then y, then z."""
    cx, cy, cz = centre
    hx, hy, hz = np.asarray(length, dtype=float) / 2
    return np.array([[cx + sx * hx, cy + sy * hy, cz + sz * hz]
                     for sz in (-1, 1) for sy in (-1, 1) for sx in (-1, 1)])


def _f(x, y, z, R):
    return z * np.arctan((x * y) / (z * R)) - x * np.log(np.abs(R + y)) - y * np.log(np.abs(R + x))


def green_functions(points, centres, lengths, compressibility, G, pi=REFERENCE_PI):
    """Displacement (3) and stress (6: 11, 22, 33, 12, 13, 23) at `points`
    (n x 3, depth positive) per unit pressure change in each cuboid:
    arrays (3, n, m) and (6, n, m)."""
    points = np.asarray(points, dtype=float)
    n, m = points.shape[0], centres.shape[0]
    V = np.stack([cuboid_vertices(centres[j], lengths[j]) for j in range(m)])     # m x 8 x 3
    xb = V[None, :, :, 0] - points[:, None, None, 0]                             # n x m x 8
    yb = V[None, :, :, 1] - points[:, None, None, 1]
    zm = V[None, :, :, 2] - points[:, None, None, 2]
    rm = np.sqrt(xb * xb + yb * yb + zm * zm)
    s = _SIGNS[None, None, :]
    pd = compressibility / (4 * pi)
    ps = compressibility * G / (2 * pi)
    with np.errstate(divide="ignore", invalid="ignore"):
        disp = np.stack([pd * np.sum(s * _f(yb, zm, xb, rm), axis=2),
                         pd * np.sum(s * _f(xb, zm, yb, rm), axis=2),
                         -pd * np.sum(s * _f(xb, yb, zm, rm), axis=2)])
        sig = np.stack([ps * np.sum(s * np.arctan((xb * rm) / (yb * zm)), axis=2),
                        ps * np.sum(s * np.arctan((yb * rm) / (xb * zm)), axis=2),
                        ps * np.sum(s * np.arctan((zm * rm) / (xb * yb)), axis=2),
                        -ps * np.sum(s * np.log(rm - zm), axis=2),
                        ps * np.sum(s * np.log(rm + yb), axis=2),
                        ps * np.sum(s * np.log(rm + xb), axis=2)])
    return disp, sig


def fault_forcing(centre, strike, dip, rake, G, nu, cuboid_centres, cuboid_lengths, times, pore_pressure,
                  temperature=None, thermal_expansivity=1e-5, biot=1.0, pi=REFERENCE_PI, normals=None, slips=None):
    """External-stress forcing on the fault patches (centre n x 3, depth
    positive; angles in degrees) from the cuboids' pore-pressure and
    temperature changes (nt x n_cuboids).  Returns dict(t, normal, shear,
    pressure) with nt x n arrays, plus the inputs of the projection
    (poro_stress 6 x nt x n, compression positive; poro_disp 3 x nt x n).
    Triangles (CalculatePoroElasticStress_Tri.jl:182-256): pass the unit
    normals and slip vectors (n x 3) instead; the traction on the normal is
    projected on them and strike/dip/rake are not used."""
    centre = np.asarray(centre, dtype=float)
    pw = 2 * G * (1 - nu) / (1 - 2 * nu)               # P-wave modulus
    cm = 1 / pw
    K = pw - 4 / 3 * G
    pore_pressure = np.asarray(pore_pressure, dtype=float)
    temperature = np.zeros_like(pore_pressure) if temperature is None else np.asarray(temperature, dtype=float)
    disp_gf, sig_gf = green_functions(centre, cuboid_centres, cuboid_lengths, cm, G, pi=pi)
    dp_eff = biot * pore_pressure + thermal_expansivity * K * temperature          # nt x m
    stress = np.einsum("cnm,tm->ctn", sig_gf, dp_eff)                             # 6 x nt x n
    disp = np.einsum("cnm,tm->ctn", disp_gf, dp_eff)
    # pore pressure on a patch inside its nearest cuboid (by centre distance)
    near = np.argmin(np.sum((cuboid_centres[None, :, :] - centre[:, None, :]) ** 2, axis=2), axis=1)
    inside = np.all(np.abs(centre - cuboid_centres[near]) <= cuboid_lengths[near] / 2, axis=1)
    p_fault = np.where(inside[None, :], pore_pressure[:, near], 0.0)               # nt x n
    # effective stress, tension positive: -poro stress + p I
    s11, s22, s33, s12, s13, s23 = (-stress[k] for k in range(6))
    eff = np.stack([np.stack([s11 + p_fault, s12, s13], -1),
                    np.stack([s12, s22 + p_fault, s23], -1),
                    np.stack([s13, s23, s33 + p_fault], -1)], -2)                  # nt x n x 3 x 3
    if normals is not None:
        nv = np.asarray(normals, dtype=float)
        tr = np.einsum("tnij,nj->tni", eff, nv)                                   # traction on the patch
        return dict(t=np.asarray(times, dtype=float), normal=-np.einsum("tni,ni->tn", tr, nv),
                    shear=np.einsum("tni,ni->tn", tr, np.asarray(slips, dtype=float)), pressure=p_fault,
                    poro_stress=stress, poro_disp=disp)
    strike, dip, rake = (np.asarray(a, dtype=float) for a in (strike, dip, rake))
    Rs = np.zeros((centre.shape[0], 3, 3))
    Rd = np.zeros_like(Rs)
    cs, ss = np.array([cosd(-a) for a in strike]), np.array([sind(-a) for a in strike])
    cd, sd = np.array([cosd(-a) for a in dip]), np.array([sind(-a) for a in dip])
    Rs[:, 0, 0], Rs[:, 0, 1], Rs[:, 1, 0], Rs[:, 1, 1], Rs[:, 2, 2] = cs, -ss, ss, cs, 1.0
    Rd[:, 0, 0], Rd[:, 1, 1], Rd[:, 1, 2], Rd[:, 2, 1], Rd[:, 2, 2] = 1.0, cd, -sd, sd, cd
    R = np.einsum("nij,njk->nik", Rd, Rs)
    sf = np.einsum("nij,tnjk,nlk->tnil", R, eff, R)
    cr, sr = np.array([cosd(a) for a in rake]), np.array([sind(a) for a in rake])
    return dict(t=np.asarray(times, dtype=float), normal=-sf[:, :, 2, 2],
                shear=cr[None, :] * sf[:, :, 0, 2] + sr[None, :] * sf[:, :, 1, 2], pressure=p_fault,
                poro_stress=stress, poro_disp=disp)
