// Input parsing and discretisation in the C ABI (host only): the reference's
// RUN2 front end, so a caller can go from the bulk text file to the segment
// table and the triangle frames without Julia.
//
//   ReadBulkInput          scripts/Functions_BuildInputFile.jl:216-274
//   LRtoRake               scripts/Functions_BuildInputFile.jl:182-213
//   BulkToSegment          scripts/Functions_BuildInputFile.jl:82-179
//   RotVerts_UnitVectors   scripts/Functions_BuildInputFile.jl:338-377
//
// Bulk files are whitespace delimited: line 1 a header, line 2 the global
// parameters (switch, shear modulus, Poisson ratio, density, two drop
// criteria, minimum normal stress), line 3 a header, then 18 columns per
// rectangle or 20 per triangle.  Degree trigonometry is exact at multiples of
// 90 degrees, as Julia's sind/cosd.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "qdfn_internal.h"

namespace qdfn {
namespace {

constexpr double kPi = 3.14159265358979323846;

double deg2rad(double x) { return x * (kPi / 180.0); }

double sind(double x) {
    if (std::isnan(x) || std::isinf(x)) return NAN;
    const double rx = std::copysign(std::fmod(x, 360.0), x);
    const double arx = std::fabs(rx);
    if (rx == 0.0) return rx;
    if (arx < 45.0) return std::sin(deg2rad(rx));
    if (arx <= 135.0) return std::copysign(std::cos(deg2rad(90.0 - arx)), rx);
    if (arx == 180.0) return std::copysign(0.0, rx);
    if (arx < 225.0) return std::sin(deg2rad((180.0 - arx) * (rx > 0 ? 1.0 : -1.0)));
    if (arx <= 315.0) return -std::copysign(std::cos(deg2rad(270.0 - arx)), rx);
    return std::sin(deg2rad(rx - std::copysign(360.0, rx)));
}

double cosd(double x) {
    if (std::isnan(x) || std::isinf(x)) return NAN;
    const double rx = std::fabs(std::fmod(x, 360.0));
    if (rx <= 45.0) return std::cos(deg2rad(rx));
    if (rx < 135.0) return std::sin(deg2rad(90.0 - rx));
    if (rx <= 225.0) return -std::cos(deg2rad(180.0 - rx));
    if (rx < 315.0) return std::sin(deg2rad(rx - 270.0));
    return std::cos(deg2rad(360.0 - rx));
}

// a whole token as a number, else NaN
double num(const std::string& tok) {
    const char* s = tok.c_str();
    char* end = nullptr;
    errno = 0;
    const double v = std::strtod(s, &end);
    if (end == s || *end != '\0') return NAN;
    return v;
}

// stable order of rows by one column
std::vector<size_t> stable_order(const std::vector<double>& t, size_t ncol, size_t col) {
    const size_t n = ncol ? t.size() / ncol : 0;
    std::vector<size_t> idx(n);
    std::iota(idx.begin(), idx.end(), size_t{0});
    std::stable_sort(idx.begin(), idx.end(),
                     [&](size_t a, size_t b) { return t[a * ncol + col] < t[b * ncol + col]; });
    return idx;
}

std::vector<double> permute_rows(const std::vector<double>& t, size_t ncol, const std::vector<size_t>& idx) {
    std::vector<double> out(t.size());
    for (size_t r = 0; r < idx.size(); ++r)
        std::memcpy(&out[r * ncol], &t[idx[r] * ncol], ncol * sizeof(double));
    return out;
}

// LRtoRake: column 8 (1-based) from +-1 to a rake angle in degrees
void lr_to_rake(double sw, std::vector<double>& bulk) {
    const size_t n = bulk.size() / 18;
    for (size_t k = 0; k < n; ++k) {
        double* b = &bulk[k * 18];
        if (sw == 1) {
            b[7] = b[7] == -1.0 ? 0.0 : 180.0;
        } else if (sw == 2) {
            if (b[6] < 90.0) b[7] = b[7] == -1.0 ? 90.0 : 270.0;
            else b[7] = b[7] == -1.0 ? 270.0 : 90.0;
        }
    }
}

// BulkToSegment: every bulk rectangle gridded into ceil(L/MaxLeng) x
// ceil(W/MaxLeng) patches, 19 columns per patch
std::vector<double> bulk_to_segment(const double* bulk, int64_t nbulk) {
    std::vector<double> seg;
    for (int64_t kb = 0; kb < nbulk; ++kb) {
        const double* b = bulk + kb * 18;
        const int64_t lc = (int64_t)std::ceil(b[3] / b[17]);
        const int64_t wc = (int64_t)std::ceil(b[4] / b[17]);
        const double Lb = b[3], Wb = b[4], st = b[5], dp = b[6];
        for (int64_t li = 1; li <= lc; ++li)
            for (int64_t wi = 1; wi <= wc; ++wi) {
                double c[3];
                if (lc * wc == 1) {
                    c[0] = b[0]; c[1] = b[1]; c[2] = b[2];
                } else {
                    const double rs[3][3] = {{cosd(st), -sind(st), 0.0}, {sind(st), cosd(st), 0.0}, {0.0, 0.0, 1.0}};
                    const double rd[3][3] = {{1.0, 0.0, 0.0}, {0.0, cosd(dp), -sind(dp)}, {0.0, sind(dp), cosd(dp)}};
                    const double v[3] = {-Lb / 2 + Lb * (2 * li - 1) / lc / 2, -Wb / 2 + Wb * (2 * wi - 1) / wc / 2,
                                         0.0};
                    double t[3];
                    for (int i = 0; i < 3; ++i) t[i] = rd[i][0] * v[0] + rd[i][1] * v[1] + rd[i][2] * v[2];
                    const double off[3] = {b[0], b[1], -b[2]};
                    for (int i = 0; i < 3; ++i) c[i] = rs[i][0] * t[0] + rs[i][1] * t[1] + rs[i][2] * t[2] + off[i];
                    c[2] = -c[2];
                }
                const size_t o = seg.size();
                seg.resize(o + 19);
                double* s = &seg[o];
                s[0] = c[0]; s[1] = c[1]; s[2] = c[2];
                s[3] = Lb / lc;
                s[4] = Wb / wc;
                for (int k = 5; k < 14; ++k) s[k] = b[k];
                s[14] = b[14] + b[15] * c[2];
                s[15] = b[16];
                s[16] = (double)(kb + 1);
                s[17] = b[3];
                s[18] = b[4];
            }
    }
    return seg;
}

// the gridding needs positive lengths and MaxLeng (else no finite patch count)
int check_bulk(const double* bulk, int64_t nbulk) {
    for (int64_t k = 0; k < nbulk; ++k) {
        const double* b = bulk + k * 18;
        if (!(b[17] > 0) || !(b[3] > 0) || !(b[4] > 0) || !std::isfinite(b[3] / b[17]) ||
            !std::isfinite(b[4] / b[17]))
            return fail(QDFN_ERR_INVALID, "bulk rectangle needs positive lengths and MaxLeng");
    }
    return QDFN_OK;
}

void cross(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

void unit(double* c) {
    const double n = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    c[0] /= n; c[1] /= n; c[2] /= n;
}

}  // namespace
}  // namespace qdfn

extern "C" int qdfn_bulk_to_segment(int64_t nbulk, const double* bulk, double* seg, int64_t cap_rows,
                                    int64_t* nseg) {
    if (nbulk < 0 || (nbulk > 0 && !bulk) || !nseg) return qdfn::fail(QDFN_ERR_INVALID, "bulk_to_segment arguments");
    if (int rc = qdfn::check_bulk(bulk, nbulk)) return rc;
    const std::vector<double> s = qdfn::bulk_to_segment(bulk, nbulk);
    *nseg = (int64_t)(s.size() / 19);
    if (seg) {
        if (cap_rows < *nseg) return qdfn::fail(QDFN_ERR_INVALID, "segment buffer too small");
        std::memcpy(seg, s.data(), s.size() * sizeof(double));
    }
    return QDFN_OK;
}

extern "C" int qdfn_read_bulk_input(const char* path, qdfn_bulk_info* info, double* seg, int64_t cap_rows) {
    if (!path || !info) return qdfn::fail(QDFN_ERR_INVALID, "read_bulk_input arguments");
    std::ifstream f(path);
    if (!f) return qdfn::fail(QDFN_ERR_INVALID, std::string("cannot open ") + path);
    std::vector<std::vector<std::string>> rows;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::vector<std::string> toks;
        std::string t;
        while (is >> t) toks.push_back(t);
        if (!toks.empty()) rows.push_back(toks);
    }
    size_t ncol = 0;
    for (const auto& r : rows) ncol = std::max(ncol, r.size());
    int tri;
    if (ncol == 18) tri = 0;
    else if (ncol == 20) tri = 1;
    else return qdfn::fail(QDFN_ERR_INVALID, "Input Bulk Fault Geometry file should have 18 or 20 columns");
    if (rows.size() < 3)
        return qdfn::fail(QDFN_ERR_INVALID, "bulk file needs two header lines and a parameter line");
    double g[7];
    for (int k = 0; k < 7; ++k) g[k] = k < (int)rows[1].size() ? qdfn::num(rows[1][k]) : NAN;
    std::vector<double> bulk;
    for (size_t r = 3; r < rows.size(); ++r)
        for (size_t k = 0; k < ncol; ++k) {
            const double v = k < rows[r].size() ? qdfn::num(rows[r][k]) : NAN;
            if (std::isnan(v)) return qdfn::fail(QDFN_ERR_INVALID, "non-numeric or missing entries in the geometry rows");
            bulk.push_back(v);
        }
    const size_t nb = bulk.size() / ncol;
    std::vector<double> out;
    int64_t nload = 0;
    if (!tri) {
        bool all_neg = nb > 0;
        for (size_t k = 0; k < nb; ++k) all_neg = all_neg && bulk[k * 18 + 2] < 0;
        if (all_neg)
            for (size_t k = 0; k < nb; ++k) bulk[k * 18 + 2] = -bulk[k * 18 + 2];
        bulk = qdfn::permute_rows(bulk, 18, qdfn::stable_order(bulk, 18, 16));
        qdfn::lr_to_rake(g[0], bulk);
        if (int rc = qdfn::check_bulk(bulk.data(), (int64_t)nb)) return rc;
        out = qdfn::bulk_to_segment(bulk.data(), (int64_t)nb);
        out = qdfn::permute_rows(out, 19, qdfn::stable_order(out, 19, 15));   // loading faults last
        for (size_t k = 0; k < out.size() / 19; ++k) nload += out[k * 19 + 15] > 0;
    } else {
        out = qdfn::permute_rows(bulk, 20, qdfn::stable_order(bulk, 20, 18));
        for (size_t k = 0; k < out.size() / 20; ++k) nload += out[k * 20 + 18] > 0;
    }
    const size_t oc = tri ? 20 : 19;
    info->switch_ss_rn = g[0];
    info->shear_modulus = g[1];
    info->poisson_ratio = g[2];
    info->rock_density = g[3];
    info->drop_crit = g[4];
    info->drop_crit_ns_multiplier = g[5];
    info->minimum_ns = g[6];
    info->is_triangle = tri;
    info->columns = (int32_t)oc;
    info->fault_count = (int64_t)(out.size() / oc);
    info->loading_fault_count = nload;
    if (seg) {
        if (cap_rows < info->fault_count) return qdfn::fail(QDFN_ERR_INVALID, "segment buffer too small");
        std::memcpy(seg, out.data(), out.size() * sizeof(double));
    }
    return QDFN_OK;
}

extern "C" int qdfn_rot_verts_unit_vectors(int64_t n, const double* P1in, const double* P2in, const double* P3in,
                                           const double* rake, double* P1, double* P2, double* P3, double* un,
                                           double* us, double* ud, double* uslip) {
    if (n < 0 || (n > 0 && (!P1in || !P2in || !P3in || !rake || !P1 || !P2 || !P3 || !un || !us || !ud || !uslip)))
        return qdfn::fail(QDFN_ERR_INVALID, "rot_verts_unit_vectors arguments");
    for (int64_t k = 0; k < n; ++k) {
        double p1[3], p2[3], p3[3], e1[3], e2[3], c[3];
        for (int i = 0; i < 3; ++i) { p1[i] = P1in[3 * k + i]; p2[i] = P2in[3 * k + i]; p3[i] = P3in[3 * k + i]; }
        for (int i = 0; i < 3; ++i) { e1[i] = p2[i] - p1[i]; e2[i] = p3[i] - p1[i]; }
        qdfn::cross(e1, e2, c);
        qdfn::unit(c);
        if (c[1] <= 0)   // normal pointing to -y: swap the first two vertices
            for (int i = 0; i < 3; ++i) std::swap(p1[i], p2[i]);
        for (int i = 0; i < 3; ++i) { e1[i] = p2[i] - p1[i]; e2[i] = p3[i] - p1[i]; }
        double* nk = un + 3 * k;
        qdfn::cross(e1, e2, nk);
        qdfn::unit(nk);
        const double ez[3] = {0.0, 0.0, 1.0};
        double* sk = us + 3 * k;
        qdfn::cross(nk, ez, sk);
        qdfn::unit(sk);
        double* dk = ud + 3 * k;
        qdfn::cross(sk, nk, dk);
        qdfn::unit(dk);
        const double cr = qdfn::cosd(rake[k]), sr = qdfn::sind(rake[k]);
        for (int i = 0; i < 3; ++i) {
            P1[3 * k + i] = p1[i];
            P2[3 * k + i] = p2[i];
            P3[3 * k + i] = p3[i];
            uslip[3 * k + i] = sk[i] * cr + dk[i] * sr;
        }
    }
    return QDFN_OK;
}
