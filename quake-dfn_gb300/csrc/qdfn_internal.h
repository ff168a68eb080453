// Internal helpers shared by the libqdfn translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/qdfn.h"

namespace qdfn {

// Thread-local last error message (qdfn_last_error).
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define QDFN_CUDA(call)                                      \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return qdfn::cuda_fail(_e, #call); \
    } while (0)

int num_sms();

}  // namespace qdfn

// ---------------------------------------------------------------------------
// Device helpers
#ifdef __CUDACC__
#include <math_constants.h>
namespace qdfn {

// Degree-argument sine/cosine with exact results at multiples of 90 degrees:
// the argument is reduced modulo 360 in degrees (exact), folded onto [-45,45]
// around a multiple of 90 (exact by Sterbenz), and converted to radians with
// pi/180 carried to ~2x double precision.  Matches Julia's Base sind/cosd,
// which the reference uses for every angle.
__device__ __forceinline__ double deg2rad_ext(double x) {
    const double h = 0.017453292519943295;
    const double t = 2.9486522708701687e-19;
    double p = x * h;
    double e = fma(x, h, -p);
    return p + (e + x * t);
}
__device__ __forceinline__ double sind_d(double x) {
    if (isnan(x) || isinf(x)) return CUDART_NAN;
    double rx = copysign(fmod(x, 360.0), x);
    double arx = fabs(rx);
    if (rx == 0.0) return rx;
    if (arx < 45.0) return sin(deg2rad_ext(rx));
    if (arx <= 135.0) return copysign(cos(deg2rad_ext(90.0 - arx)), rx);
    if (arx == 180.0) return copysign(0.0, rx);
    if (arx < 225.0) return sin(deg2rad_ext((180.0 - arx) * (rx > 0 ? 1.0 : -1.0)));
    if (arx <= 315.0) return -copysign(cos(deg2rad_ext(270.0 - arx)), rx);
    return sin(deg2rad_ext(rx - copysign(360.0, rx)));
}
__device__ __forceinline__ double cosd_d(double x) {
    if (isnan(x) || isinf(x)) return CUDART_NAN;
    double rx = fabs(fmod(x, 360.0));
    if (rx <= 45.0) return cos(deg2rad_ext(rx));
    if (rx < 135.0) return sin(deg2rad_ext(90.0 - rx));
    if (rx <= 225.0) return -cos(deg2rad_ext(180.0 - rx));
    if (rx < 315.0) return sin(deg2rad_ext(rx - 270.0));
    return cos(deg2rad_ext(360.0 - rx));
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

}  // namespace qdfn
#endif
