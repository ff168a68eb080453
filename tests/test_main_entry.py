"""The drop-in entry points qdfn.simulate.main / main_H (the reference's
Functions_RSFDFN3DMain_D.jl `main` and _H.jl `main_H` signatures): the host
glue -- positional arguments to the problem, the record count, the normal
stiffness switch, the external-stress file, the SaveStep loop and the result
file -- checked on the CPU against a stand-in for the device context.  The
device calls themselves are covered by the GPU tests."""
import numpy as np
import pytest

from qdfn import hmatrix, simulate


class FakeSimulation:
    """Records what main() asks of the context; its history grows by one
    record per RecordStep steps."""
    made = []

    def __init__(self, problem, n_inst=1, record_step=0, max_records=0):
        self.problem, self.record_step, self.max_records = problem, record_step, max_records
        self.N = problem["N"]
        self.steps, self.runs, self.dense, self.ext, self.closed = 0, [], None, None, False
        FakeSimulation.made.append(self)

    def set_dense(self, Ks, Kn, precision="fp64"):
        self.dense = (np.asarray(Ks), np.asarray(Kn), precision)

    def set_external_stress(self, t, normal, shear, pressure):
        self.ext = (np.asarray(t), np.asarray(normal), np.asarray(shear), np.asarray(pressure))

    def run(self, n, timeout_s=0.0):
        self.runs.append(n)
        self.steps += n

    def history(self, inst=0):
        n = min(self.steps // self.record_step, self.max_records) if self.record_step else 0
        T = np.arange(1, n + 1) * 10.0
        return dict(T=T, Dt=np.full(n, 10.0), V=np.ones((n, self.N)), D=np.zeros((n, self.N)),
                    theta=np.ones((n, self.N)), sigma=np.ones((n, self.N)))

    def state(self, inst=0):
        return dict(T=self.steps * 10.0, V=np.ones(self.N), dt=10.0)

    def close(self):
        self.closed = True


def _args(N, Ks, Kn, zero_normal=0, total=100, record=10, save_step=30, out=""):
    rng = np.random.default_rng(0)
    v = lambda: rng.uniform(0.5, 1.5, N)   # noqa: E731
    return (Ks, Kn, zero_normal, 3.2e10, N, 1, v(), v(), v(), v(), v(), v(), v(), v(), v(),
            total, record, 1e-2, 4.0, 0.05, 3e6, out, 2670.0,
            rng.normal(size=(N, 3)), v(), v(), v(), v(), v(), save_step, 1e6, 0.0, 1)


def test_main_maps_the_reference_arguments(monkeypatch, tmp_path):
    monkeypatch.setattr(simulate, "Simulation", FakeSimulation)
    monkeypatch.chdir(tmp_path)
    N = 7
    Ks, Kn = np.eye(N) * -1e9, np.eye(N) * 2e8
    args = _args(N, Ks, Kn, out=str(tmp_path / "res.npz"))
    hist = simulate.main(*args, external_stress=None, precision="fp32")
    sim = FakeSimulation.made[-1]
    p = sim.problem
    assert p["N"] == N and p["Nload"] == 1 and p["G"] == 3.2e10 and p["rho"] == 2670.0
    assert p["switch_v"] == 1e-2 and p["dt_cut"] == 4.0 and p["rupture_dt"] == 0.05 and p["max_dt"] == 3e6
    assert p["sigma_min"] == 1e6 and p["alpha_evo"] == 0.0 and p["evolution_dr"] == 1
    assert p["interp_at_told"] == 0                        # main: external stress at TOld + Dt
    assert np.array_equal(p["a"], args[7]) and np.array_equal(p["mass"], args[6])
    assert np.array_equal(p["V_const"], args[14]) and np.array_equal(p["sigma0"], args[13])
    assert sim.record_step == 10 and sim.max_records == 10   # round(TotalStep / RecordStep)
    assert sim.dense[2] == "fp32" and np.array_equal(sim.dense[1], Kn)
    assert sim.runs == [30, 30, 30, 10] and sim.closed     # SaveStep chunks
    z = np.load(tmp_path / "res.npz")
    assert sorted(z.files) == sorted(["History_V", "History_Disp", "History_Time", "History_Theta",
                                      "History_NormalStress", "History_Dt"])
    assert z["History_V"].shape == (10, N) and z["History_Time"].shape == (10, 1)
    # saved at step 90, the last multiple of SaveStep (Main_D :286): 9 records,
    # the 10th row still the zeros the reference allocates
    assert np.all(z["History_V"][:9] == 1.0) and np.all(z["History_V"][9] == 0.0)
    assert z["History_Time"][8, 0] == 90.0 and z["History_Time"][9, 0] == 0.0
    assert hist["T"].shape == (10,)


def test_saved_history_is_padded_to_total_record(monkeypatch, tmp_path):
    """Every save holds TotalRecord x N arrays (Main_D :133-141, 287-289),
    zero past the records written so far."""
    monkeypatch.setattr(simulate, "Simulation", FakeSimulation)
    N = 5
    Ks, Kn = np.eye(N) * -1e9, np.eye(N) * 2e8
    out = str(tmp_path / "res.npz")
    simulate.main(*_args(N, Ks, Kn, total=100, record=10, save_step=50, out=out), external_stress=None)
    z = np.load(out)                      # last save at step 100: all 10 records
    for k in ("History_V", "History_Disp", "History_Theta", "History_NormalStress"):
        assert z[k].shape == (10, N), k
    assert z["History_Time"].shape == (10, 1) and z["History_Time"][9, 0] == 100.0
    simulate.main(*_args(N, Ks, Kn, total=100, record=10, save_step=50, out=out), external_stress=None)
    sim = FakeSimulation.made[-1]
    assert sim.runs == [50, 50]


def test_main_zero_normal_and_external_stress_file(monkeypatch, tmp_path):
    monkeypatch.setattr(simulate, "Simulation", FakeSimulation)
    monkeypatch.chdir(tmp_path)
    N = 5
    Ks, Kn = np.eye(N) * -1e9, np.ones((N, N))
    t = np.array([0.0, 1e9])
    np.savez(tmp_path / "Input_ExternalStressChange.npz", ExternalStress_TimeArray=t,
             ExternalStress_Normal=np.zeros((2, N)), ExternalStress_Shear=np.ones((2, N)), Pressure=np.zeros((2, N)))
    simulate.main(*_args(N, Ks, Kn, zero_normal=1, total=20, record=5, save_step=0))
    sim = FakeSimulation.made[-1]
    assert np.all(sim.dense[1] == 0)                       # NormalStiffnessZero == 1
    assert sim.ext is not None and np.array_equal(sim.ext[0], t) and np.all(sim.ext[2] == 1)
    assert sim.runs == [20]                                 # SaveStep 0: one run
    # a file for another fault count is ignored, as the reference does
    np.savez(tmp_path / "Input_ExternalStressChange.npz", ExternalStress_TimeArray=t,
             ExternalStress_Normal=np.zeros((2, N + 1)), ExternalStress_Shear=np.ones((2, N + 1)),
             Pressure=np.zeros((2, N + 1)))
    simulate.main(*_args(N, Ks, Kn, total=20, record=5, save_step=0))
    assert FakeSimulation.made[-1].ext is None


def test_main_H_passes_the_reference_blocks(monkeypatch, tmp_path):
    monkeypatch.setattr(simulate, "Simulation", FakeSimulation)
    got = {}
    monkeypatch.setattr(hmatrix, "set_hmatrix", lambda sim, H, precision: got.update(H=H, precision=precision))
    monkeypatch.chdir(tmp_path)
    N = 6
    # two blocks, 1-based inclusive ranges: a dense one and a low-rank (U, Vt) one
    rng_sr = np.array([[1, 3, 1, 6], [4, 6, 1, 6]])
    dense = np.ones((6, 3))
    lowrank = (np.ones((6, 1)), np.ones((1, 3)))
    a = _args(N, None, None, total=10, record=5, save_step=0)
    args = (a[3], N, 1, a[6], 0, *a[7:15], 10, 5, 1e-2, 4.0, 0.05, 3e6, "", 2670.0, a[23], *a[24:29], 0,
            1e6, 0.0, [1, 1], [0, 1], rng_sr, [dense, lowrank], [dense, lowrank], 4, 1, [0, 1])
    simulate.main_H(*args, external_stress=None)
    sim = FakeSimulation.made[-1]
    assert sim.problem["interp_at_told"] == 1               # main_H: external stress at TOld
    H = got["H"]
    assert H.ranges.tolist() == (rng_sr - 1).tolist()       # 0-based
    assert H.dense_s[0] is not None and H.U_s[1] is not None and H.Vt_s[1].shape == (1, 3)
    assert got["precision"] == "fp64" and sim.runs == [10]
