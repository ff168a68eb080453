"""Known-answer tests pinning the CPU oracle.

The reference ships no tests or golden vectors and Julia cannot run here, so
the oracle is pinned by physics: two independent closed forms (Okada
rectangles vs Nikkhoo-Walter triangles) must agree, the free surface must be
traction free, gradients must match finite differences, the far field must
decay as r^-3, and the friction inversion must return the steady state.
"""
import itertools

import numpy as np
import pytest

G, NU = 32e9, 0.25
LAM = 2 * G * NU / (1 - 2 * NU)
ALPHA = (LAM + G) / (LAM + 2 * G)


def okada_stress(O, x, y, z, dep, dip, L, W, d1, d2):
    U, _ = O.okada_dc3d(ALPHA, x, y, z, dep, dip, L / 2, L / 2, W / 2, W / 2, d1, d2, 0.0)
    UXX, UYX, UZX, UXY, UYY, UZY, UXZ, UYZ, UZZ = U[3:]
    tr = UXX + UYY + UZZ
    return np.array([LAM * tr + 2 * G * UXX, LAM * tr + 2 * G * UYY, LAM * tr + 2 * G * UZZ,
                     (UXY + UYX) * G, (UXZ + UZX) * G, (UYZ + UZY) * G])


@pytest.mark.parametrize("dip", [90.0, 60.0, 30.0])
@pytest.mark.parametrize("rake", [0.0, 35.0, 120.0])
def test_rectangle_equals_two_triangles(oracle_mod, dip, rake):
    O = oracle_mod
    L, W, dep = 2000.0, 1000.0, 1500.0
    cd, sd = np.cos(np.radians(dip)), np.sin(np.radians(dip))
    corner = lambda xs, ws: np.array([xs * L / 2, ws * W / 2 * cd, -dep + ws * W / 2 * sd])
    A, B, C, D = corner(-1, -1), corner(1, -1), corner(1, 1), corner(-1, 1)
    d1, d2 = np.cos(np.radians(rake)), np.sin(np.radians(rake))
    pts = [(300.0, 800.0, -1200.0), (-1500.0, -400.0, -2500.0), (100.0, 1500.0, -300.0), (2500.0, -2000.0, -50.0)]
    best = np.inf
    for sgn in itertools.product([1, -1], [1, -1]):
        err = 0.0
        for p in pts:
            so = okada_stress(O, *p, dep, dip, L, W, d1, d2)
            s1, _ = O.tdstress_hs(*p, A, B, C, sgn[0] * d1, sgn[1] * d2, 0.0, G, LAM)
            s2, _ = O.tdstress_hs(*p, A, C, D, sgn[0] * d1, sgn[1] * d2, 0.0, G, LAM)
            err = max(err, np.max(np.abs(s1 + s2 - so)) / np.max(np.abs(so)))
        best = min(best, err)
    assert best < 1e-10


def test_okada_traction_free_surface(oracle_mod):
    for (x, y, dep, dip, rake) in [(700.0, 300.0, 1000.0, 60.0, 30.0), (-200.0, 900.0, 600.0, 90.0, 0.0),
                                   (1500.0, -700.0, 2000.0, 25.0, 90.0)]:
        s = okada_stress(oracle_mod, x, y, 0.0, dep, dip, 2000.0, 1000.0, np.cos(np.radians(rake)),
                         np.sin(np.radians(rake)))
        scale = np.max(np.abs(s))
        assert abs(s[2]) < 1e-12 * scale and abs(s[4]) < 1e-12 * scale and abs(s[5]) < 1e-12 * scale


def test_td_traction_free_surface(oracle_mod):
    P1 = np.array([-1000.0, 0.0, -500.0])
    P2 = np.array([1000.0, -300.0, -1500.0])
    P3 = np.array([0.0, 800.0, -200.0])
    for x, y in [(300.0, -200.0), (-900.0, 1200.0), (50.0, 50.0)]:
        st, _ = oracle_mod.tdstress_hs(x, y, 0.0, P1, P2, P3, 0.4, 0.8, 0.1, G, LAM)
        scale = np.max(np.abs(st))
        assert abs(st[2]) < 1e-12 * scale and abs(st[4]) < 1e-12 * scale and abs(st[5]) < 1e-12 * scale


def test_okada_gradient_matches_finite_difference(oracle_mod):
    for (x, y, z, dep, dip) in [(1000.0, 2000.0, -3000.0, 5000.0, 70.0), (300.0, -800.0, -100.0, 2000.0, 90.0),
                                (-2500.0, 500.0, -6000.0, 4000.0, 35.0)]:
        args = (dep, dip, 1500.0, 1500.0, 800.0, 800.0, 0.7, 0.3, 0.0)
        U, _ = oracle_mod.okada_dc3d(ALPHA, x, y, z, *args)
        h = 1e-2
        num = []
        for ax in range(3):
            p, m = [x, y, z], [x, y, z]
            p[ax] += h
            m[ax] -= h
            Up, _ = oracle_mod.okada_dc3d(ALPHA, *p, *args)
            Um, _ = oracle_mod.okada_dc3d(ALPHA, *m, *args)
            num.append((Up[:3] - Um[:3]) / (2 * h))
        ana = np.array(U[3:]).reshape(3, 3)
        assert np.max(np.abs(np.array(num) - ana)) / np.max(np.abs(ana)) < 1e-7


def test_far_field_decay(oracle_mod):
    # very deep source (free surface negligible), receivers along a ray:
    # |stress| r^3 tends to a constant once r >> source size
    vals = []
    for r in (10e3, 20e3, 40e3):
        s = okada_stress(oracle_mod, r * 0.6, r * 0.8, -1000e3, 1000e3, 60.0, 500.0, 500.0, 1.0, 0.0)
        vals.append(np.linalg.norm(s) * r ** 3)
    assert abs(vals[2] / vals[1] - 1) < 0.01 and abs(vals[1] / vals[0] - 1) < 0.02


def test_self_stiffness_negative_and_reciprocal(oracle_mod):
    import qdfn.synth as synth
    rec = synth.grid_fault(0.0, 0.0, 3000.0, 2000.0, 1000.0, 90.0, 90.0, 0.0, 500.0)
    cols = dict(cx=rec[:, 0], cy=rec[:, 1], cz=rec[:, 2], ls=rec[:, 3], ld=rec[:, 4], strike=rec[:, 5],
                dip=rec[:, 6], rake=rec[:, 7])
    Ks, Kn = oracle_mod.assemble_rect(cols, cols, G, NU)
    assert np.all(np.diag(Ks) < 0)
    # equal coplanar patches at equal depth and rake: the collocated shear
    # stiffness is symmetric by mirror symmetry (pairs at different depths are
    # not, because the free surface breaks the symmetry of centre collocation)
    same = np.abs(rec[:, 2][:, None] - rec[:, 2][None, :]) < 1e-9
    assert np.max(np.abs((Ks - Ks.T)[same])) < 1e-12 * np.max(np.abs(Ks))
    assert np.max(np.abs(Ks - Ks.T)) < 1e-6 * np.max(np.abs(Ks))
    # a vertical planar fault with pure strike slip carries no normal stress change
    assert np.max(np.abs(Kn)) < 1e-6 * np.max(np.abs(Ks))


def test_deep_source_halfspace_tends_to_fullspace(oracle_mod):
    # moving source and receiver down together, the half-space stress converges
    # (the image and free-surface terms vanish with depth)
    P1 = np.array([-500.0, 0.0, 0.0]); P2 = np.array([500.0, 0.0, 0.0]); P3 = np.array([0.0, 0.0, 1000.0])
    out = []
    for d in (-50e3, -100e3, -200e3):
        sh = np.array([0.0, 0.0, d])
        st, _ = oracle_mod.tdstress_hs(300.0, 400.0, 500.0 + d, P1 + sh, P2 + sh, P3 + sh, 1.0, 0.0, 0.0, G, LAM)
        out.append(st)
    e1 = np.max(np.abs(out[1] - out[2])) / np.max(np.abs(out[2]))
    e0 = np.max(np.abs(out[0] - out[2])) / np.max(np.abs(out[2]))
    assert e1 < 1e-6 and e1 < e0


def test_td_edge_points_are_nan(oracle_mod):
    P1 = np.array([-1000.0, 0.0, -2000.0]); P2 = np.array([1000.0, 0.0, -2000.0]); P3 = np.array([0.0, 0.0, -1000.0])
    st, _ = oracle_mod.tdstress_hs(0.0, 0.0, -2000.0, P1, P2, P3, 1.0, 0.0, 0.0, G, LAM)
    assert np.all(np.isnan(st))


def test_td_rejects_points_above_surface(oracle_mod):
    P1 = np.array([-1000.0, 0.0, -2000.0]); P2 = np.array([1000.0, 0.0, -2000.0]); P3 = np.array([0.0, 0.0, -1000.0])
    with pytest.raises(ValueError):
        oracle_mod.tdstress_hs(0.0, 0.0, 10.0, P1, P2, P3, 1.0, 0.0, 0.0, G, LAM)


def _one_patch_problem(V_i=1e-9, a=0.01, b=0.015, n=1):
    Dc = 1e-3
    return dict(N=n, Nload=0, a=np.full(n, a), b=np.full(n, b), Dc=np.full(n, Dc), theta_i=np.full(n, Dc / V_i),
                V_i=np.full(n, V_i), f_i=np.full(n, 0.6), sigma0=np.full(n, 40e6), V_const=np.zeros(n),
                mass=np.full(n, 6.5e5), G=32e9, rho=2612.0, sigma_min=1e6, switch_v=1e-2, dt_cut=5.0,
                rupture_dt=0.01, max_dt=1e7, alpha_evo=0.0, evolution_dr=1, interp_at_told=0)


def test_steady_state_is_preserved(oracle_mod):
    # one isolated patch at steady state: the low-V friction inversion returns
    # V_i up to the ~0.07 Pa stress drop of the first 1.2 s of slip (K D / (a sigma) ~ 2e-7)
    p = _one_patch_problem()
    Ks = np.array([[-6.0e7]]); Kn = np.zeros((1, 1))
    sim = oracle_mod.Simulation(p, ("dense", Ks, Kn))
    sim.run(1)
    assert abs(sim.state["V"][0] / 1e-9 - 1) < 1e-6
    # with no loading the patch relaxes: V decays monotonically and Dt grows
    sim.run(60)
    assert sim.state["V"][0] < 1e-9 and sim.dt > 100.0


def test_oracle_run_is_deterministic(oracle_mod):
    import qdfn.synth as synth
    sysd = synth.single_fault(patch=2500.0)
    cols = dict(cx=sysd["records"][:, 0], cy=sysd["records"][:, 1], cz=sysd["records"][:, 2],
                ls=sysd["records"][:, 3], ld=sysd["records"][:, 4], strike=sysd["records"][:, 5],
                dip=sysd["records"][:, 6], rake=sysd["records"][:, 7])
    Ks, Kn = oracle_mod.assemble_rect(cols, cols, sysd["G"], sysd["nu"])
    prob = synth.problem_dict(sysd, np.diag(Ks))
    ext = synth.external_ramp(sysd["N"], 1e6, 1e11)
    prob.update(ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    outs = []
    for nth in (1, 4):
        s = oracle_mod.Simulation(prob, ("dense", Ks, Kn), nthreads=nth)
        s.run(200)
        outs.append((s.T, s.state["D"].copy()))
    assert outs[0][0] == outs[1][0]
    assert np.array_equal(outs[0][1], outs[1][1])
