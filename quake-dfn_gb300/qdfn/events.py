"""Event catalogue from a recorded slip history (host side, post-processing).

Restates the reference's event definition on in-memory arrays instead of the
JLD2 result files:

* ``event_fragments``  -- scripts/Functions_Plot.jl:430-510 (get_event_fragments):
  per patch, a fragment starts at the first record whose slip rate
  ``(D[t] - D[t-1]) / (T[t] - T[t-1])`` exceeds ``rate_crit`` after a record
  that did not, and accumulates the moment ``dD * area * G`` of every
  consecutive record above it; fragments are ordered by start time with a
  stable sort (Julia's ``sortperm``), ties in patch order.
* ``merge_fragments`` -- scripts/Functions_Plot.jl:513-588 (merge_fragments):
  each fragment joins the event of the most recent earlier fragment that
  started less than ``merge_time`` before it and lies closer than
  ``merge_distance``; otherwise it opens a new event.  Magnitudes are
  ``(log10(M0) - 9.05) / 1.5``.

``rate_crit`` defaults to 1e-2 m/s, the value Results/3_Seismicity_CatalogGenerator.jl:16
sets for ``DispRateCrits``.  Onset times defined this way are the event times
the slip histories are compared on.
"""
import numpy as np


def patch_area_rect(length_strike, length_dip):
    """Rectangle areas, Functions_Plot.jl:456-458 (RorT == "R")."""
    return np.asarray(length_strike, dtype=np.float64) * np.asarray(length_dip, dtype=np.float64)


def patch_area_tri(P1, P2, P3):
    """Triangle areas by Heron's formula, Functions_Plot.jl:448-455 (RorT == "T")."""
    P1, P2, P3 = (np.asarray(x, dtype=np.float64) for x in (P1, P2, P3))
    a = np.linalg.norm(P1 - P2, axis=1)
    b = np.linalg.norm(P1 - P3, axis=1)
    c = np.linalg.norm(P2 - P3, axis=1)
    s = (a + b + c) / 2
    return np.sqrt(s * (s - a) * (s - b) * (s - c))


def event_fragments(T, D, centers, area, G, rate_crit=1e-2):
    """Fragments of a history: T (nrec,), D (nrec, N) record-major slip,
    centers (N, 3), area (N,), shear modulus G.  Returns (times (F,),
    locations (F, 3), moments (F,), count F), ordered by time."""
    T = np.asarray(T, dtype=np.float64).ravel()
    D = np.asarray(D, dtype=np.float64)
    centers = np.asarray(centers, dtype=np.float64)
    area = np.asarray(area, dtype=np.float64).ravel()
    nrec, N = D.shape
    if T.shape[0] != nrec:
        raise ValueError("T and D disagree on the record count")
    times, locs, moments = [], [], []
    if nrec >= 2:
        dD = D[1:] - D[:-1]                            # (nrec-1, N)
        with np.errstate(divide="ignore", invalid="ignore"):   # IEEE, as Julia: x/0 = +-Inf, 0/0 = NaN
            rate = dD / (T[1:] - T[:-1])[:, None]
        above = rate > rate_crit
        for i in range(N):                             # patch-major, as the reference loops
            on = False
            for t in range(nrec - 1):
                if above[t, i]:
                    m = dD[t, i] * area[i] * G
                    if not on:
                        on = True
                        times.append(T[t + 1])
                        locs.append(centers[i])
                        moments.append(m)
                    else:
                        moments[-1] += m
                else:
                    on = False
    times = np.asarray(times, dtype=np.float64)
    locs = np.asarray(locs, dtype=np.float64).reshape(-1, 3)
    moments = np.asarray(moments, dtype=np.float64)
    order = np.argsort(times, kind="stable")
    return times[order], locs[order], moments[order], int(times.shape[0])


def merge_fragments(times, locations, moments, merge_time, merge_distance):
    """Events from time-ordered fragments.  Returns (event start times (E,),
    moment magnitudes (E,), locations (E, 3), event index of every fragment)."""
    times = np.asarray(times, dtype=np.float64).ravel()
    locations = np.asarray(locations, dtype=np.float64).reshape(-1, 3)
    moments = np.asarray(moments, dtype=np.float64).ravel()
    F = times.shape[0]
    event_of = np.zeros(F, dtype=np.int64)
    ev_time, ev_loc = [], []
    for k in range(F):
        if k == 0:
            ev_time.append(times[0]); ev_loc.append(locations[0]); event_of[0] = 0
            continue
        j = k - 1
        while True:
            if j < 0:                                           # nothing close enough before it
                ev_time.append(times[k]); ev_loc.append(locations[k]); event_of[k] = len(ev_time) - 1
                break
            if times[k] - times[j] < merge_time:
                if np.linalg.norm(locations[k] - locations[j]) < merge_distance:
                    event_of[k] = event_of[j]                   # same event as fragment j
                    break
                j -= 1                                          # in time, not in distance: keep looking
            else:                                               # past the time window: a new event
                ev_time.append(times[k]); ev_loc.append(locations[k]); event_of[k] = len(ev_time) - 1
                break
    E = len(ev_time)
    m0 = np.zeros(E)
    np.add.at(m0, event_of, moments)
    with np.errstate(divide="ignore"):
        mw = (np.log10(m0) - 9.05) / 1.5
    return np.asarray(ev_time), mw, np.asarray(ev_loc).reshape(-1, 3), event_of
