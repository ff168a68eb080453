"""Batched ensemble of geometries of uneven size (one context per geometry,
SM shares via qdfn_set_blocks, runs side by side on separate streams)."""
import numpy as np
import pytest

from _systems import small_network


def test_sm_shares_are_proportional_and_fit():
    from qdfn.ensemble import sm_shares
    s = sm_shares([1.0, 1.0, 2.0, 4.0], 152)
    assert s.sum() == 152 and list(s) == [19, 19, 38, 76]
    s = sm_shares([1e6] + [1.0] * 20, 152)          # tiny members still get one SM each
    assert s.sum() <= 152 and s.min() == 1 and s[0] == 152 - 20
    with pytest.raises(ValueError):
        sm_shares(np.ones(200), 152)


@pytest.mark.gpu
def test_ensemble_members_follow_their_oracles(qdfn_mod, oracle_mod):
    """Three geometries (49, 56, 72 patches) with 2, 3 and 1 friction draws,
    FP64 operator, advanced together: every instance matches its own oracle run."""
    from qdfn import assemble, ensemble, synth
    from test_sim_gpu import G, NU, _rel
    from _systems import problem_for
    members, refs = [], []
    for seed, R in ((1, 2), (2, 3), (4, 1)):
        rec = small_network(seed=seed)["records"]
        N = rec.shape[0]
        Ks, Kn = assemble.assemble_rect(rec, rec, G, NU)
        prob = problem_for(rec, Ks)
        ext = synth.external_ramp(N, 1e6, 1e11)
        draws = synth.friction_draws(dict(prob, N=N), R, seed=seed)
        mprob = dict(prob)
        for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
            mprob[k] = draws[k]
        for k in ("sigma0", "V_const", "mass"):
            mprob[k] = np.tile(prob[k], R)
        members.append(dict(problem=mprob, n_inst=R, Ks=Ks, Kn=Kn, ext=ext))
        refs.append((prob, ext, draws, Ks, Kn, N, R))
    ens = ensemble.Ensemble(members, precision="fp64")
    assert sum(ens.blocks) <= 152 and min(ens.blocks) >= 1
    ens.run(80, timeout_s=120)
    for sim, (prob, ext, draws, Ks, Kn, N, R) in zip(ens.members, refs):
        for r in range(R):
            op = dict(prob, ext_t=ext["t"], ext_n=ext["normal"], ext_s=ext["shear"], ext_p=ext["pressure"])
            for k in ("a", "b", "Dc", "theta_i", "V_i", "f_i"):
                op[k] = draws[k][r * N:(r + 1) * N]
            o = oracle_mod.Simulation(op, ("dense", Ks, Kn))
            o.run(80)
            st = sim.state(r)
            assert st["step"] == o.step == 80
            assert abs(st["T"] / o.T - 1) < 1e-9
            assert _rel(st["D"], o.state["D"]) < 1e-9
