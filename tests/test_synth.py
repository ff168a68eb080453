"""The seeded synthetic workloads stand in for the configurations' inputs (the
reference ships no benchmark data), so their shapes and value distributions
are checked here: the 30-fault network of the benchmark line (C2), the
friction draws of the ensemble, and the single fault (C1).  Host code."""
import numpy as np

from qdfn import synth


def test_benchmark_network_shape_and_distributions():
    s = synth.fault_network(seed=2, n_faults=30)
    rec = s["records"]
    assert s["N"] == rec.shape[0] == 12813          # the bench line's patch count
    assert np.all((rec[:, 5] >= 0) & (rec[:, 5] < 180))                 # strike U[0, 180)
    assert np.all((rec[:, 6] >= 60) & (rec[:, 6] <= 90))                # dip U[60, 90]
    assert np.all(rec[:, 2] > 0)
    # patches of at most 100 m (a fault's length split into ceil(L / 100) equal parts)
    assert np.all((rec[:, 3] <= 100.0) & (rec[:, 3] > 50.0)) and np.all((rec[:, 4] <= 100.0) & (rec[:, 4] > 50.0))
    a, b, Dc = s["a"], s["b"], s["Dc"]
    assert np.all((a >= 0.008) & (a <= 0.012)) and np.all(np.abs(b - a) <= 0.004)
    assert np.all((Dc >= 1e-4) & (Dc <= 1e-2))
    assert np.allclose(s["sigma0"], 18e6 * rec[:, 2] / 1000.0)          # 18 MPa/km x depth
    assert np.allclose(s["theta_i"], Dc / 1e-9) and s["Nload"] == 0
    again = synth.fault_network(seed=2, n_faults=30)
    assert np.array_equal(again["records"], rec) and np.array_equal(again["Dc"], Dc)   # seeded


def test_friction_draws_keep_a_and_redraw_b_and_dc():
    s = synth.fault_network(seed=3, n_faults=4, patch=400.0, length=(1200.0, 2400.0))
    N = s["N"]
    d = synth.friction_draws(s, 4, seed=1)
    assert all(v.shape == (4 * N,) for v in d.values())
    a = d["a"].reshape(4, N)
    assert np.all(a == s["a"][None, :])
    amb = (d["a"] - d["b"]).reshape(4, N)
    assert np.all((amb >= -0.005) & (amb <= 0.002))
    assert np.all((d["Dc"] >= 1e-4) & (d["Dc"] <= 1e-2))
    assert not np.array_equal(d["Dc"][:N], d["Dc"][N:2 * N])           # draws differ


def test_external_ramp_layout():
    e = synth.external_ramp(5, 0.01e6, 1e12)
    assert e["t"].tolist() == [0.0, 1e12]
    assert e["shear"].shape == (2, 5) and np.all(e["shear"][0] == 0)
    assert np.allclose(e["shear"][1], 0.01e6 * 1e12 / (365.25 * 86400.0))


def test_curved_fault_network_shapes(oracle_mod):
    """The triangle-mesh workload: 5 near-parallel curved faults of 8 x 4 km
    (edge 400 m here: 2 x 20 x 10 triangles each), every vertex below the
    surface, every self stiffness negative (the oracle's TDstressHS), friction
    in the network's ranges."""
    import numpy as np
    from qdfn import synth
    d = synth.curved_fault_network(seed=2, edge=400.0)
    seg = d["seg"]
    assert d["N"] == seg.shape[0] == 5 * 2 * 20 * 10 and seg.shape[1] == 20
    assert np.max(seg[:, [2, 5, 8]]) < 0
    assert np.all((d["a"] >= 0.008) & (d["a"] <= 0.012)) and np.all(np.abs(d["b"] - d["a"]) <= 0.004)
    assert np.all(d["sigma0"] > 0)
    from qdfn import geometry
    P1, P2, P3, un, _, _, us = geometry.rot_verts_unit_vectors_abi(seg, seg[:, 9])
    c = (P1 + P2 + P3) / 3
    for i in range(0, d["N"], 7):
        Ks, _ = oracle_mod.assemble_tri(P1[i:i + 1], P2[i:i + 1], P3[i:i + 1], seg[i:i + 1, 9], c[i:i + 1],
                                        un[i:i + 1], us[i:i + 1], d["G"], d["nu"], nthreads=1)
        assert Ks[0, 0] < 0, i
