"""Input parsing and discretisation (host side), mirroring the reference's
RUN2 front end so the text input format is kept:

  ReadBulkInput          scripts/Functions_BuildInputFile.jl:216-274
  LRtoRake               scripts/Functions_BuildInputFile.jl:182-213
  BulkToSegment          scripts/Functions_BuildInputFile.jl:82-179
  ReadSegmentInput       scripts/Functions_BuildInputFile.jl:278-332
  RotVerts_UnitVectors   scripts/Functions_BuildInputFile.jl:338-377
  fault mass / RuptureDt scripts/QUAKEDFN_RunARG.jl:159-201

Bulk files are whitespace/tab delimited: line 1 a header, line 2 the global
parameters (switch, shear modulus, Poisson ratio, density, two drop criteria,
minimum normal stress), line 3 a header, then 18 columns per rectangle or 20
per triangle.
"""
import math

import numpy as np


# ---------------------------------------------------------------------------
# degree trigonometry, exact at multiples of 90 degrees (as Julia's sind/cosd)
def _deg2rad(x):
    return x * (math.pi / 180.0)


def sind(x):
    x = float(x)
    if math.isnan(x) or math.isinf(x):
        return math.nan
    rx = math.copysign(math.fmod(x, 360.0), x)
    arx = abs(rx)
    if rx == 0.0:
        return rx
    if arx < 45.0:
        return math.sin(_deg2rad(rx))
    if arx <= 135.0:
        return math.copysign(math.cos(_deg2rad(90.0 - arx)), rx)
    if arx == 180.0:
        return math.copysign(0.0, rx)
    if arx < 225.0:
        return math.sin(_deg2rad((180.0 - arx) * (1.0 if rx > 0 else -1.0)))
    if arx <= 315.0:
        return -math.copysign(math.cos(_deg2rad(270.0 - arx)), rx)
    return math.sin(_deg2rad(rx - math.copysign(360.0, rx)))


def cosd(x):
    x = float(x)
    if math.isnan(x) or math.isinf(x):
        return math.nan
    rx = abs(math.fmod(x, 360.0))
    if rx <= 45.0:
        return math.cos(_deg2rad(rx))
    if rx < 135.0:
        return math.sin(_deg2rad(90.0 - rx))
    if rx <= 225.0:
        return -math.cos(_deg2rad(180.0 - rx))
    if rx < 315.0:
        return math.sin(_deg2rad(rx - 270.0))
    return math.cos(_deg2rad(360.0 - rx))


class InputFormatError(ValueError):
    pass


def _read_table(path):
    rows = []
    with open(path) as f:
        for line in f:
            if line.strip() == "":
                continue
            rows.append(line.split())
    return rows


def _num(tok):
    try:
        return float(tok)
    except ValueError:
        return math.nan


def lr_to_rake(switch, bulk):
    """LRtoRake: column 8 (1-based) from +-1 to a rake angle in degrees."""
    bulk = bulk.copy()
    if switch == 1:
        for k in range(bulk.shape[0]):
            bulk[k, 7] = 0.0 if bulk[k, 7] == -1.0 else 180.0
    elif switch == 2:
        for k in range(bulk.shape[0]):
            if bulk[k, 6] < 90.0:
                bulk[k, 7] = 90.0 if bulk[k, 7] == -1.0 else 270.0
            else:
                bulk[k, 7] = 270.0 if bulk[k, 7] == -1.0 else 90.0
    return bulk


def bulk_to_segment(bulk):
    """BulkToSegment: grid every bulk rectangle into ceil(L/MaxLeng) x
    ceil(W/MaxLeng) patches; returns the 19-column segment table."""
    counts = [(math.ceil(bulk[k, 3] / bulk[k, 17]), math.ceil(bulk[k, 4] / bulk[k, 17]))
              for k in range(bulk.shape[0])]
    total = int(sum(lc * wc for lc, wc in counts))
    seg = np.zeros((total, 19))
    idx = 0
    for kb in range(bulk.shape[0]):
        lc, wc = counts[kb]
        Lb, Wb = bulk[kb, 3], bulk[kb, 4]
        st, dp = bulk[kb, 5], bulk[kb, 6]
        cb = bulk[kb, 0:3]
        for li in range(1, lc + 1):
            for wi in range(1, wc + 1):
                ls = Lb / lc
                ld = Wb / wc
                if lc * wc == 1:
                    centre = cb.copy()
                else:
                    rs = np.array([[cosd(st), -sind(st), 0.0], [sind(st), cosd(st), 0.0], [0.0, 0.0, 1.0]])
                    rd = np.array([[1.0, 0.0, 0.0], [0.0, cosd(dp), -sind(dp)], [0.0, sind(dp), cosd(dp)]])
                    v = np.array([-Lb / 2 + Lb * (2 * li - 1) / lc / 2, -Wb / 2 + Wb * (2 * wi - 1) / wc / 2, 0.0])
                    centre = rs @ (rd @ v) + np.array([cb[0], cb[1], -cb[2]])
                    centre[2] = -centre[2]
                seg[idx, 0:3] = centre
                seg[idx, 3] = ls
                seg[idx, 4] = ld
                seg[idx, 5:14] = bulk[kb, 5:14]
                seg[idx, 14] = bulk[kb, 14] + bulk[kb, 15] * centre[2]
                seg[idx, 15] = bulk[kb, 16]
                seg[idx, 16] = kb + 1
                seg[idx, 17] = bulk[kb, 3]
                seg[idx, 18] = bulk[kb, 4]
                idx += 1
    return seg


def read_bulk_input(path):
    """ReadBulkInput.  Returns a dict with Input_Segment, LoadingFaultCount,
    ShearModulus, PoissonRatio, RockDensity, Switch_StrikeSlip_or_ReverseNormal,
    DropCrit, DropCritNormalStressMultiplier, MinimumNS, RorT, FaultCount."""
    rows = _read_table(path)
    ncol = max(len(r) for r in rows)
    if ncol == 18:
        RorT = "R"
    elif ncol == 20:
        RorT = "T"
    else:
        raise InputFormatError("Input Bulk Fault Geometry file should have 18 or 20 columns")
    if len(rows) < 3:
        raise InputFormatError("bulk file needs two header lines and a parameter line")
    g = [_num(t) for t in rows[1]] + [math.nan] * 7
    out = dict(Switch_StrikeSlip_or_ReverseNormal=g[0], ShearModulus=g[1], PoissonRatio=g[2], RockDensity=g[3],
               DropCrit=g[4], DropCritNormalStressMultiplier=g[5], MinimumNS=g[6], RorT=RorT)
    data = rows[3:]
    bulk = np.array([[_num(t) for t in r] + [math.nan] * (ncol - len(r)) for r in data], dtype=float)
    if bulk.size == 0:
        bulk = np.zeros((0, ncol))
    if np.isnan(bulk).any():
        raise InputFormatError("non-numeric or missing entries in the geometry rows")
    if RorT == "R":
        if bulk.shape[0] and np.all(bulk[:, 2] < 0):
            bulk[:, 2] = -bulk[:, 2]
        bulk = bulk[np.argsort(bulk[:, 16], kind="stable")]
        bulk = lr_to_rake(out["Switch_StrikeSlip_or_ReverseNormal"], bulk)
        seg = bulk_to_segment(bulk)
        seg = seg[np.argsort(seg[:, 15], kind="stable")]  # loading faults last
        nload = int(np.sum(seg[:, 15] > 0))
    else:
        bulk = bulk[np.argsort(bulk[:, 18], kind="stable")]
        seg = bulk[np.argsort(bulk[:, 18], kind="stable")]
        nload = int(np.sum(seg[:, 18] > 0))
    out.update(Input_Segment=seg, LoadingFaultCount=nload, FaultCount=seg.shape[0])
    return out


def read_segment_input(seg, RorT):
    """ReadSegmentInput: split the segment table into named per-patch arrays."""
    n = seg.shape[0]
    if RorT == "R":
        d = dict(FaultCenter=seg[:, 0:3].copy(), FaultLengthStrike=seg[:, 3].copy(), FaultLengthDip=seg[:, 4].copy(),
                 FaultStrikeAngle=seg[:, 5].copy(), FaultDipAngle=seg[:, 6].copy(), FaultRakeAngle=seg[:, 7].copy(),
                 Fault_a=seg[:, 8].copy(), Fault_b=seg[:, 9].copy(), Fault_Dc=seg[:, 10].copy(),
                 Fault_Theta_i=seg[:, 11].copy(), Fault_V_i=seg[:, 12].copy(), Fault_Friction_i=seg[:, 13].copy(),
                 Fault_NormalStress=seg[:, 14].copy(), Fault_V_Const=seg[:, 15].copy(),
                 Fault_BulkIndex=seg[:, 16].copy(), FaultLengthStrike_Bulk=seg[:, 17].copy(),
                 FaultLengthDip_Bulk=seg[:, 18].copy(), NormalStiffnessZero=0)
    else:
        P1, P2, P3 = seg[:, 0:3], seg[:, 3:6], seg[:, 6:9]
        centre = np.zeros((n, 3))
        centre[:, 0] = (P1[:, 0] + P2[:, 0] + P3[:, 0]) / 3
        centre[:, 1] = (P1[:, 1] + P2[:, 1] + P3[:, 1]) / 3
        centre[:, 2] = (P1[:, 2] + P2[:, 2] + P3[:, 2]) / 3
        ls = np.max(np.abs(np.hstack([P1 - P2, P2 - P3, P1 - P3])), axis=1)
        d = dict(FaultCenter=centre, FaultRakeAngle=seg[:, 9].copy(), Fault_a=seg[:, 10].copy(),
                 Fault_b=seg[:, 11].copy(), Fault_Dc=seg[:, 12].copy(), Fault_Theta_i=seg[:, 13].copy(),
                 Fault_V_i=seg[:, 14].copy(), Fault_Friction_i=seg[:, 15].copy(),
                 Fault_NormalStress=seg[:, 16] - seg[:, 17] * centre[:, 2], Fault_V_Const=seg[:, 18].copy(),
                 Fault_BulkIndex=seg[:, 9] * 0, FaultLengthStrike=ls, FaultLengthDip=ls.copy(),
                 FaultStrikeAngle=np.zeros(n), FaultDipAngle=np.zeros(n), FaultLengthStrike_Bulk=ls.copy(),
                 FaultLengthDip_Bulk=ls.copy(), NormalStiffnessZero=0)
    return d


def rot_verts_unit_vectors(seg, rake):
    """RotVerts_UnitVectors: swap P1/P2 where the normal's y component is <= 0,
    then the unit normal, strike-slip, dip-slip and slip vectors."""
    n = seg.shape[0]
    P1, P2, P3 = seg[:, 0:3].copy(), seg[:, 3:6].copy(), seg[:, 6:9].copy()
    un, us, ud, uslip = (np.zeros((n, 3)) for _ in range(4))
    for k in range(n):
        p1, p2, p3 = P1[k].copy(), P2[k].copy(), P3[k].copy()
        c = np.cross(p2 - p1, p3 - p1)
        nv = c / np.linalg.norm(c)
        if nv[1] <= 0:
            p1, p2 = p2, p1
        P1[k], P2[k], P3[k] = p1, p2, p3
        c = np.cross(p2 - p1, p3 - p1)
        un[k] = c / np.linalg.norm(c)
        c = np.cross(un[k], np.array([0.0, 0.0, 1.0]))
        us[k] = c / np.linalg.norm(c)
        c = np.cross(us[k], un[k])
        ud[k] = c / np.linalg.norm(c)
        uslip[k] = us[k] * cosd(rake[k]) + ud[k] * sind(rake[k])
    return P1, P2, P3, un, us, ud, uslip


def read_obj_mesh(path):
    """Vertices and triangular faces of a Wavefront .obj mesh, read as
    Tools/TriangleMeshReader/ObjReader.jl:44-70 reads them: `v x y z` rows
    (extra colour columns ignored), `f a b c` rows whose entries may be
    `i/t/n` (the first index is kept, 1-based in the file; returned 0-based);
    other rows are skipped."""
    verts, faces = [], []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "v":
                verts.append([float(t) for t in tok[1:4]])
            elif tok[0] == "f":
                if len(tok) != 4:
                    raise InputFormatError("only triangular faces are supported")
                faces.append([int(t.split("/")[0]) - 1 for t in tok[1:4]])
    V = np.asarray(verts, dtype=np.float64).reshape(-1, 3)
    F = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    if F.size and (F.min() < 0 or F.max() >= V.shape[0]):
        raise InputFormatError("face index out of range")
    return V, F


# ObjReader.jl:17-38 defaults: the bulk header and the per-triangle properties
OBJ_DEFAULTS = dict(switch_ss_rn=0, shear_modulus=20e9, poisson=0.25, rock_density=2670.0, crit_too_close=1.05,
                    too_close_normal_multiplier=0.6, min_normal_stress=2e6, amp=100.0, rake=0.0, a=0.005, b=0.01,
                    Dc=1e-3, theta_i=1e5, V_i=1e-15, friction_i=0.6, normal_stress_surface=10e6,
                    normal_stress_gradient=0.0, V_const=0.0, min_segment_length=100000.0)


def obj_to_bulk(V, F, **kw):
    """The 20-column triangle bulk table and its header line that ObjReader.jl
    writes (:106-135): vertices scaled by `amp`, then P1, P2, P3, rake, a, b,
    Dc, Theta_i, V_i, Friction_i, normal stress at the surface, its gradient,
    V_const and the minimum segment length per triangle."""
    o = dict(OBJ_DEFAULTS, **kw)
    Vs = V * o["amp"]
    n = F.shape[0]
    bulk = np.zeros((n, 20))
    bulk[:, 0:3] = Vs[F[:, 0]]
    bulk[:, 3:6] = Vs[F[:, 1]]
    bulk[:, 6:9] = Vs[F[:, 2]]
    bulk[:, 9] = o["rake"]
    for col, key in ((10, "a"), (11, "b"), (12, "Dc"), (13, "theta_i"), (14, "V_i"), (15, "friction_i"),
                     (16, "normal_stress_surface"), (17, "normal_stress_gradient"), (18, "V_const"),
                     (19, "min_segment_length")):
        bulk[:, col] = o[key]
    header = [o["switch_ss_rn"], o["shear_modulus"], o["poisson"], o["rock_density"], o["crit_too_close"],
              o["too_close_normal_multiplier"], o["min_normal_stress"]]
    return header, bulk


def write_bulk_file(path, header, bulk):
    """Writes a bulk geometry file in the layout ReadBulkInput reads: a header
    line, the seven run parameters, a column-name line, then one row per bulk
    fault (18 columns for rectangles, 20 for triangles), tab-separated."""
    names = ("SwitchSS/RN\tShearMod\tPoissonRatio\tR_Density\tCrit_TooClose\tTooCloseNormal_Multiplier\t"
             "Minimum_NS")
    cols = ("P1_x P1_y P1_z P2_x P2_y P2_z P3_x P3_y P3_z Rake a b Dc Theta_i V_i Fric_i Sig0 SigGrad V_Const "
            "MaxLeng" if bulk.shape[1] == 20 else
            "Ctr_X Ctr_Y Ctr_Z St_L Dip_L StAng DipAng LR/RN a b Dc Theta_i V_i Fric_i Sig0 SigGrad V_Const MaxLeng")
    with open(path, "w") as f:
        f.write(names + "\n")
        f.write("\t".join(repr(float(x)) for x in header) + "\n")
        f.write("\t".join(cols.split()) + "\n")
        for row in bulk:
            f.write("\t".join(repr(float(x)) for x in row) + "\n")


def fault_mass(length_strike, length_dip, rho, vertical_length_scale=0.0):
    """FaultMass = VertScale * rho / 2 (QUAKEDFN_RunARG.jl:159-164)."""
    if vertical_length_scale == 0:
        vs = min(np.min(length_strike), np.min(length_dip))
    else:
        vs = vertical_length_scale
    return np.ones(len(length_strike)) * vs * rho / 2


def rupture_dt(mass, kself_diag, multiple):
    """RecTimeStep = min sqrt(M/|K_ii|)/10; RuptureDt = RecTimeStep * multiple
    (QUAKEDFN_RunARG.jl:189-201)."""
    period = np.sqrt(np.asarray(mass) / np.abs(np.asarray(kself_diag)))
    return float(np.min(period) / 10 * multiple)


def rect_records(d):
    """n x 8 records {cx, cy, cz, strike length, dip length, strike, dip, rake}
    for the assembly ABI."""
    c = d["FaultCenter"]
    return np.ascontiguousarray(np.column_stack([c[:, 0], c[:, 1], c[:, 2], d["FaultLengthStrike"],
                                                 d["FaultLengthDip"], d["FaultStrikeAngle"],
                                                 d["FaultDipAngle"], d["FaultRakeAngle"]]), dtype=np.float64)


# ---------------------------------------------------------------------------
# The same front end through the C ABI (qdfn_read_bulk_input,
# qdfn_bulk_to_segment, qdfn_rot_verts_unit_vectors): the entry points a
# non-Python caller (the Julia shim) uses.
def _abi():
    from . import _lib
    return _lib, _lib.load()


def read_bulk_input_abi(path):
    """read_bulk_input through the C ABI; same keys."""
    import ctypes as C
    _lib, L = _abi()
    info = _lib.BulkInfo()
    _lib.check(L.qdfn_read_bulk_input(path.encode(), C.byref(info), None, 0))
    seg = np.zeros((info.fault_count, info.columns))
    _lib.check(L.qdfn_read_bulk_input(path.encode(), C.byref(info), seg.ctypes.data, seg.shape[0]))
    return dict(Switch_StrikeSlip_or_ReverseNormal=info.switch_ss_rn, ShearModulus=info.shear_modulus,
                PoissonRatio=info.poisson_ratio, RockDensity=info.rock_density, DropCrit=info.drop_crit,
                DropCritNormalStressMultiplier=info.drop_crit_ns_multiplier, MinimumNS=info.minimum_ns,
                RorT="T" if info.is_triangle else "R", Input_Segment=seg,
                LoadingFaultCount=int(info.loading_fault_count), FaultCount=int(info.fault_count))


def bulk_to_segment_abi(bulk):
    """bulk_to_segment through the C ABI."""
    import ctypes as C
    _lib, L = _abi()
    bulk = np.ascontiguousarray(bulk, dtype=np.float64)
    n = C.c_int64(0)
    _lib.check(L.qdfn_bulk_to_segment(bulk.shape[0], bulk.ctypes.data, None, 0, C.byref(n)))
    seg = np.zeros((n.value, 19))
    _lib.check(L.qdfn_bulk_to_segment(bulk.shape[0], bulk.ctypes.data, seg.ctypes.data, seg.shape[0], C.byref(n)))
    return seg


def rot_verts_unit_vectors_abi(seg, rake):
    """rot_verts_unit_vectors through the C ABI."""
    _lib, L = _abi()
    n = seg.shape[0]
    P = [np.ascontiguousarray(seg[:, 3 * k:3 * k + 3], dtype=np.float64) for k in range(3)]
    rk = np.ascontiguousarray(rake, dtype=np.float64)
    out = [np.zeros((n, 3)) for _ in range(7)]
    _lib.check(L.qdfn_rot_verts_unit_vectors(n, *(a.ctypes.data for a in P), rk.ctypes.data,
                                              *(a.ctypes.data for a in out)))
    return tuple(out)
