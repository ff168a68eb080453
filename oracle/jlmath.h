// Oracle helpers: degree-argument trigonometry with the exact-at-multiples-of-90
// behaviour of Julia's Base `sind`/`cosd` (base/special/trig.jl), used by the
// reference wherever it writes `sind(...)`/`cosd(...)`.
//
// TEST INFRASTRUCTURE ONLY.  This directory is the CPU oracle that the tests,
// the smoke check and the bench's CPU-baseline leg compare the CUDA library
// against.  Nothing in the shipped library includes or links it.
#pragma once
#include <cmath>

namespace oracle {

// pi/180 split into a head that is exact in double and a tail, so that the
// degree->radian product is carried to ~2x double precision before sin/cos.
static inline double deg2rad_ext(double x) {
    const double h = 0.017453292519943295;        // fl(pi/180)
    const double t = 2.9486522708701687e-19;      // pi/180 - h
    double p = x * h;
    double e = std::fma(x, h, -p);               // exact error of x*h
    return p + (e + x * t);
}

// sind: reduce modulo 360 in degrees (exact), fold onto [-45,45] around a
// multiple of 90 (exact by Sterbenz), then evaluate sin or cos in radians.
static inline double sind(double x) {
    if (std::isnan(x) || std::isinf(x)) return NAN;
    double rx = std::copysign(std::fmod(x, 360.0), x);
    double arx = std::fabs(rx);
    if (rx == 0.0) return rx;
    if (arx < 45.0) return std::sin(deg2rad_ext(rx));
    if (arx <= 135.0) return std::copysign(std::cos(deg2rad_ext(90.0 - arx)), rx);
    if (arx == 180.0) return std::copysign(0.0, rx);
    if (arx < 225.0) {
        double s = rx > 0 ? 1.0 : -1.0;
        return std::sin(deg2rad_ext((180.0 - arx) * s));
    }
    if (arx <= 315.0) return -std::copysign(std::cos(deg2rad_ext(270.0 - arx)), rx);
    return std::sin(deg2rad_ext(rx - std::copysign(360.0, rx)));
}

static inline double cosd(double x) {
    if (std::isnan(x) || std::isinf(x)) return NAN;
    double rx = std::fabs(std::fmod(x, 360.0));
    if (rx <= 45.0) return std::cos(deg2rad_ext(rx));
    if (rx < 135.0) return std::sin(deg2rad_ext(90.0 - rx));
    if (rx <= 225.0) return -std::cos(deg2rad_ext(180.0 - rx));
    if (rx < 315.0) return std::sin(deg2rad_ext(rx - 270.0));
    return std::cos(deg2rad_ext(360.0 - rx));
}

}  // namespace oracle
