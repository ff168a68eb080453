"""The discrete adjoint (qdfn_adjoint_run) against central finite differences of
the FP64 oracle, on a small loaded fault network run up to its first event
onset: loss = squared misfit of the final slip against a run with perturbed
a, b and Dc, plus the squared misfit of the first event onset time (the
interpolated time at which the slip rate first reaches 1e-2 m/s, the onset of
an event fragment, scripts/Functions_Plot.jl:430-510).  Along this window the
step map is smooth -- every solve is the low-velocity one until the onset
step, and no decision flips under the differences' perturbations (asserted) --
so the differences are a faithful check of the gradient.  Also: the FP32
operator's adjoint against the all-FP64 one, the gradient's independence of
the checkpoint spacing, and the torch.autograd wrapper."""
import numpy as np
import pytest

from _systems import problem_for, small_network

pytestmark = pytest.mark.gpu
G, NU = 32e9, 0.25
V_CRIT = 1e-2


def _setup():
    from qdfn import assemble, synth
    rec = small_network(seed=5, n_faults=3, patch=500.0)["records"]
    Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
    prob = problem_for(rec, Ks, seed=3)
    ext = synth.external_ramp(rec.shape[0], 2e7, 1e11)    # fast loading: an event within the window
    return rec, Ks, Kn, prob, ext


def _oracle_hist(oracle_mod, prob, ext, Ks, Kn, nsteps):
    p = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
    o = oracle_mod.Simulation(p, ("dense", Ks, Kn))
    V0, D0 = o.state["V"].copy(), o.state["D"].copy()
    h = o.run(nsteps, record_step=1, max_rec=nsteps)
    T = np.concatenate([[0.0], h["T"]])
    V = np.vstack([V0, h["V"]])
    D = np.vstack([D0, h["D"]])
    return T, V, D


def _gpu_sim(prob, Ks, Kn, ext, precision="fp64", record=0):
    from qdfn import simulate
    sim = simulate.Simulation(prob, record_step=1 if record else 0, max_records=record)
    sim.set_dense(Ks, Kn, precision)
    sim.set_external_stress(ext["t"], ext["normal"], ext["shear"], ext["pressure"])
    return sim


def _loss_parts(T, V, D, n, Dstar, tstar, ns):
    from qdfn import adjoint
    ons = adjoint.onset_times(T[:n + 1], V[:n + 1], ns, V_CRIT, count=1)
    te = ons[0][0] if ons else None
    L = float(np.sum((D[n] - Dstar) ** 2)) + (0.0 if te is None else (te - tstar) ** 2)
    return L, ons


@pytest.fixture(scope="module")
def window(oracle_mod):
    """The oracle window up to the first onset, the targets, and the loss's
    derivatives along the GPU trajectory."""
    rec, Ks, Kn, prob, ext = _setup()
    N = rec.shape[0]
    T, V, D = _oracle_hist(oracle_mod, prob, ext, Ks, Kn, 600)
    from qdfn import adjoint
    ons = adjoint.onset_times(T, V, N, V_CRIT, count=1)
    assert ons, "no event onset within 600 steps"
    n = ons[0][1]                                           # the window ends at the onset step
    assert np.all(np.max(V[:n, :N], axis=1) <= V_CRIT)      # every earlier step is a low-velocity one
    # targets: the same window with a, b, Dc perturbed by 1 %
    rng = np.random.default_rng(11)
    pert = dict(prob)
    for k in ("a", "b", "Dc"):
        pert[k] = prob[k] * (1 + 0.01 * rng.standard_normal(N))
    Tp, Vp, Dp = _oracle_hist(oracle_mod, pert, ext, Ks, Kn, n)
    Dstar = Dp[n]
    tstar = ons[0][0] * (1 + 1e-3)
    return dict(rec=rec, Ks=Ks, Kn=Kn, prob=prob, ext=ext, N=N, n=n, Dstar=Dstar, tstar=tstar, onset=ons[0])


def _adjoint_grad(w, precision="fp64", checkpoint_every=0):
    """Gradient of the window's loss through the GPU adjoint: the GPU forward
    gives the loss's derivatives (final slip, onset seeds), a fresh context
    runs the adjoint."""
    from qdfn import adjoint
    N, n = w["N"], w["n"]
    sim = _gpu_sim(w["prob"], w["Ks"], w["Kn"], w["ext"], precision, record=n)
    st0 = sim.state(0)
    sim.run(n, timeout_s=120)
    h = sim.history(0)
    T = np.concatenate([[0.0], h["T"]])
    V = np.vstack([st0["V"], h["V"]])
    D = np.vstack([st0["D"], h["D"]])
    sim.close()
    ons = adjoint.onset_times(T, V, N, V_CRIT, count=1)
    assert ons and ons[0][1] == n and ons[0][2] == w["onset"][2]
    te = ons[0][0]
    seeds = adjoint.onset_seeds(T, V, ons[0], 2 * (te - w["tstar"]), v_crit=V_CRIT)
    sim = _gpu_sim(w["prob"], w["Ks"], w["Kn"], w["ext"], precision)
    g = adjoint.gradient(sim, n, dL_dD_final=2 * (D[n] - w["Dstar"]), seeds=seeds,
                         checkpoint_every=checkpoint_every, timeout_s=300)
    assert sim.state(0)["step"] == n                       # the context ends at the window's end
    sim.close()
    return g


def test_adjoint_gradient_matches_central_differences(qdfn_mod, oracle_mod, window):
    w = window
    N, n = w["N"], w["n"]
    g = _adjoint_grad(w)
    rng = np.random.default_rng(5)
    patches = rng.choice(N, size=min(50, N), replace=False)
    for key in ("a", "b", "Dc"):
        fd = np.zeros(len(patches))
        for j, i in enumerate(patches):
            vals = []
            for sgn in (1, -1):
                p = dict(w["prob"])
                p[key] = w["prob"][key].copy()
                eps = 1e-6 * abs(p[key][i])
                p[key][i] += sgn * eps
                T, V, D = _oracle_hist(oracle_mod, p, w["ext"], w["Ks"], w["Kn"], n)
                L, ons = _loss_parts(T, V, D, n, w["Dstar"], w["tstar"], N)
                assert ons and ons[0][1] == n and ons[0][2] == w["onset"][2]   # no decision flipped
                vals.append(L)
            fd[j] = (vals[0] - vals[1]) / (2 * eps)
        ga = g[key][0, patches]
        err = np.max(np.abs(ga - fd)) / np.max(np.abs(fd))
        assert err <= 1e-4, (key, err, ga[:5], fd[:5])


def test_fp32_operator_adjoint_tracks_the_fp64_adjoint(qdfn_mod, window):
    g64 = _adjoint_grad(window, "fp64")
    g32 = _adjoint_grad(window, "fp32")
    for key in ("a", "b", "Dc"):
        err = np.max(np.abs(g32[key] - g64[key])) / np.max(np.abs(g64[key]))
        assert err <= 1e-3, (key, err)


def test_gradient_does_not_depend_on_checkpoint_spacing(qdfn_mod, window):
    ref = _adjoint_grad(window, checkpoint_every=0)
    for cp in (1, 7, window["n"]):
        g = _adjoint_grad(window, checkpoint_every=cp)
        for key in ("a", "b", "Dc"):
            assert np.array_equal(g[key], ref[key]), (cp, key)


def test_autograd_function_gives_the_adjoint_gradient(qdfn_mod, window):
    import torch
    from qdfn import adjoint
    w = window
    n = w["n"] - 1

    def make_sim(a, b, Dc):
        p = dict(w["prob"], a=a.ravel(), b=b.ravel(), Dc=Dc.ravel())
        return _gpu_sim(p, w["Ks"], w["Kn"], w["ext"])

    a = torch.tensor(w["prob"]["a"][None, :], requires_grad=True)
    b = torch.tensor(w["prob"]["b"][None, :], requires_grad=True)
    Dc = torch.tensor(w["prob"]["Dc"][None, :], requires_grad=True)
    D = adjoint.CycleLoss.apply(a, b, Dc, make_sim, n)
    wts = torch.from_numpy(np.random.default_rng(2).standard_normal(D.shape))
    (D * wts).sum().backward()
    sim = make_sim(a.detach().numpy(), b.detach().numpy(), Dc.detach().numpy())
    g = adjoint.gradient(sim, n, dL_dD_final=wts.numpy())
    sim.close()
    assert np.array_equal(a.grad.numpy(), g["a"]) and np.array_equal(Dc.grad.numpy(), g["Dc"])
    assert np.max(np.abs(b.grad.numpy())) > 0
