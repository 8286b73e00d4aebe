// log10 of a single evaluated in double and rounded once, identical on the
// host and the device: the binary exponent is split off (mantissa in
// [sqrt(1/2), sqrt(2))), ln of the mantissa from the atanh series
// ln m = 2 (s + s^3/3 + ... + s^23/23), s = (m - 1) / (m + 1).
#pragma once

#include <cmath>

namespace tg {

__host__ __device__ inline float log10_single(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (isinf(x)) return x;
    int e;
    double m = frexp((double)x, &e);
    if (m < 0.70710678118654752) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double t = 1.0 / 23.0;
    for (int k = 21; k >= 1; k -= 2) t = 1.0 / k + s2 * t;
    const double ln = 2.0 * s * t + (double)e * 0.69314718055994530942;
    return (float)(ln / 2.30258509299404568402);
}

// slice layout of save_spectrum_2d (code/output.F90:828-852)
struct SpecGrid {
    int mxmin, mymin, nxb, nyb, gambins;
    float dxslice, dyslice;
};

inline SpecGrid spec_grid(int mx, int my, int ng, int gambins) {
    SpecGrid s;
    const int mxmin = (int)((float)(mx - ng) * 0.5f) - 1200 + (ng / 2 + 1);
    const int mxmax = (int)((float)(mx - ng) * 0.5f) + 400 + (ng / 2 + 1);
    const int mymin = ng / 2 + 1, mymax = my - ng / 2;
    s.mxmin = mxmin;
    s.mymin = mymin;
    s.nxb = (mxmax - mxmin) / 30 > 1 ? (mxmax - mxmin) / 30 : 1;
    s.nyb = (mymax - mymin) / 30 > 1 ? (mymax - mymin) / 30 : 1;
    s.gambins = gambins;
    s.dxslice = 1.0f * (float)(mxmax - mxmin) / (float)s.nxb;
    s.dyslice = 1.0f * (float)(mymax - mymin) / (float)s.nyb;
    return s;
}

}  // namespace tg
