"""Event catalogue (qdfn.events) on hand-built histories, following the
reference's get_event_fragments / merge_fragments (scripts/Functions_Plot.jl)."""
import numpy as np

from qdfn import events


def test_fragments_follow_the_rate_threshold_per_patch():
    T = np.array([0.0, 1.0, 2.0, 3.0, 4.0, 5.0])
    # patch 0 slips fast over records 2-3 (one fragment), patch 1 twice (two
    # fragments), patch 2 creeps below the threshold
    D = np.zeros((6, 3))
    D[:, 0] = [0, 0, 0.5, 1.0, 1.0, 1.0]
    D[:, 1] = [0, 0.2, 0.2, 0.2, 0.6, 0.6]
    D[:, 2] = np.arange(6) * 1e-3
    centers = np.array([[0.0, 0, -1e3], [0.0, 100, -1e3], [5e3, 0, -1e3]])
    area = np.array([1e4, 2e4, 1e4])
    t, loc, m0, n = events.event_fragments(T, D, centers, area, G=3e10, rate_crit=0.1)
    assert n == 3
    # fragments: patch 1 at T=1, patch 0 at T=2, patch 1 at T=4 (time order)
    assert np.array_equal(t, [1.0, 2.0, 4.0])
    assert np.array_equal(loc, centers[[1, 0, 1]])
    assert np.allclose(m0, [0.2 * 2e4 * 3e10, 1.0 * 1e4 * 3e10, 0.4 * 2e4 * 3e10], rtol=1e-15)


def test_equal_start_times_keep_patch_order():
    T = np.array([0.0, 1.0])
    D = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]])
    c = np.array([[2.0, 0, 0], [0.0, 0, 0], [1.0, 0, 0]])
    t, loc, _, n = events.event_fragments(T, D, c, np.ones(3), G=1.0, rate_crit=0.5)
    assert n == 3 and np.array_equal(loc, c)   # stable: ties stay in patch order


def test_merge_by_time_and_distance():
    t = np.array([0.0, 0.5, 0.7, 5.0, 5.1])
    loc = np.array([[0.0, 0, 0], [10.0, 0, 0], [1e4, 0, 0], [0.0, 0, 0], [1e4, 0, 0]])
    m0 = np.array([1e15, 1e15, 2e15, 3e15, 4e15])
    et, mw, eloc, of = events.merge_fragments(t, loc, m0, merge_time=1.0, merge_distance=100.0)
    # 0 and 1 merge (close in time and space); 2 is close in time, far in space;
    # 3 and 4 are past the window of the first group, far from each other
    assert np.array_equal(of, [0, 0, 1, 2, 3])
    assert np.array_equal(et, [0.0, 0.7, 5.0, 5.1])
    assert np.allclose(mw, (np.log10([2e15, 2e15, 3e15, 4e15]) - 9.05) / 1.5)


def test_fragment_looks_back_past_a_distant_one():
    # the third fragment is near the first: it skips the distant second one
    t = np.array([0.0, 0.1, 0.2])
    loc = np.array([[0.0, 0, 0], [5e3, 0, 0], [10.0, 0, 0]])
    _, _, _, of = events.merge_fragments(t, loc, np.ones(3) * 1e12, merge_time=1.0, merge_distance=100.0)
    assert np.array_equal(of, [0, 1, 0])


def test_areas():
    assert np.array_equal(events.patch_area_rect([2.0, 3.0], [4.0, 5.0]), [8.0, 15.0])
    a = events.patch_area_tri([[0.0, 0, 0]], [[3.0, 0, 0]], [[0.0, 4.0, 0]])
    assert abs(a[0] - 6.0) < 1e-12
